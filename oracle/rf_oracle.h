/*
 * rf_oracle.h -- CPU oracle for the RayFactorCL Monte Carlo view-factor tracer.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * OpenCL kernels (RayFactorCL/RayFactorGPU.cl, "RFG" below) used as the checker
 * for the CUDA library.  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg may load it.  The product path never calls it.
 *
 * Parity pins: the Philox stream is pinned against the reference's own
 * Random123/philox.h compiled on the host (tests/golden/philox_kat.json), the
 * scene tables against the reference's Scene.cpp/affine code compiled on the
 * host (tests/golden/scenes/), and every ray's first hit against the
 * reference's own kernel source RayFactorGPU.cl, compiled as host C++ through
 * oracle/ref_tools/cl_compat.h and run work-item by work-item
 * (tests/golden/ref_kernel_rays.npz; equal on all 18 fixture scenes for runGPU
 * and runBVGPU under RFO_COMPAT_*, all set).  OpenCL leaves the builtins'
 * results implementation-defined, so both sides use one fixed IEEE op mapping:
 *   mad(a,b,c)      -> fmaf(a,b,c)
 *   native_sqrt(x)  -> sqrtf(x)             (correctly rounded)
 *   native_recip(x) -> 1.0f / x             (correctly rounded)
 *   native_rsqrt(x) -> 1.0f / sqrtf(x)
 *   sincos(x)       -> rfo_sincosf(x)       (project-owned, see rf_oracle.c)
 *   dot(a,b)        -> fmaf(a3,b3, fmaf(a2,b2, fmaf(a1,b1, a0*b0)))
 *   a*b + c in the source -> separately rounded multiply and add
 * compiled with -ffp-contract=off and no fast-math, IEEE inf/NaN kept.
 */
#ifndef RF_ORACLE_H
#define RF_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* RayfactorConstants.h:25-33 */
enum { RFO_CYLINDER = 0, RFO_FRUSTUM = 1, RFO_SPHERE = 2, RFO_ANNULUS = 3,
       RFO_RECTANGLE = 4, RFO_DISC = 5, RFO_NONE = 6 };

/* RayfactorConstants.h:38-45, 112 bytes */
typedef struct rfo_prim {
    float m[12];
    float invm[12];
    int32_t type;
    int32_t rayDensity;
    float util1;
    float util2;
} rfo_prim;

/* RayfactorConstants.h:48-56, 72 bytes */
typedef struct rfo_bv {
    float invm[12];
    int32_t type;
    int32_t settings;
    int32_t objStartIndex;
    int32_t objEndIndex;
    float util1;
    float util2;
} rfo_bv;

/* Behaviour switches; bit values equal the library's RF_COMPAT_* flags. */
#define RFO_COMPAT_BUDGET   (1u << 0) /* main.cpp:172 budget of emitter 0 for all  */
#define RFO_COMPAT_SPHERE   (1u << 1) /* RFG:272-278 discriminant without sqrt      */
#define RFO_COMPAT_BV_STALE (1u << 2) /* RFG:596-619 stale child index across BVs   */
#define RFO_COMPAT_STREAMS  (1u << 3) /* RFG:486-487 stream key = {gid, key1} only  */

typedef struct rfo_params {
    uint32_t compat;   /* RFO_COMPAT_* bits                                   */
    uint32_t key1;     /* Philox key word 1; 0xdecafbad in RFG:486            */
    float eps;         /* self-intersection threshold; 1e-3f in RFG:7         */
    int32_t use_bv;    /* 0: runGPU (RFG:481), 1: runBVGPU (RFG:530)          */
    uint32_t scene_id; /* folded into the counter outside compat mode         */
} rfo_params;

/* Philox4x32-10 (Salmon et al., SC'11), the function of Random123/philox.h. */
void rfo_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* Project-owned sin/cos of a float argument (method in rf_oracle.c). */
void rfo_sincosf(float x, float *s, float *c);
void rfo_sincosf_array(const float *x, int64_t n, float *s, float *c);

/* The four uniforms of one stream (RFG:486-500) for emitter `emitter`, id `gid`. */
void rfo_stream_uniforms(const rfo_params *p, int32_t emitter, int64_t gid, float out[4]);

/* Emit one ray (RFG:502-517 for sub-ray v of stream gid) in FP32: origin s[3], direction c[3]. */
void rfo_emit_ray(const rfo_prim *prims, int32_t emitter, const rfo_params *p,
                  int64_t ray, float s[3], float c[3]);

/* Per-ray hit index for rays [ray_begin, ray_end) of one emitter; -1 = no hit. */
int rfo_trace_rays(const rfo_prim *prims, int32_t n, const rfo_bv *bvs, int32_t nbv,
                   const rfo_params *p, int32_t emitter, int64_t ray_begin, int64_t ray_end,
                   int32_t *hit_out, int32_t n_threads);

/* Tally rays [0, n_rays) of one emitter into row[n] (int64, accumulated). */
int rfo_tally(const rfo_prim *prims, int32_t n, const rfo_bv *bvs, int32_t nbv,
              const rfo_params *p, int32_t emitter, int64_t n_rays, int64_t *row,
              int32_t n_threads);

/* Same streams, all geometry in double precision: the FP64 tracer. */
int rfo_tally_f64(const rfo_prim *prims, int32_t n, const rfo_bv *bvs, int32_t nbv,
                  const rfo_params *p, int32_t emitter, int64_t n_rays, int64_t *row,
                  int32_t n_threads);
int rfo_trace_rays_f64(const rfo_prim *prims, int32_t n, const rfo_bv *bvs, int32_t nbv,
                       const rfo_params *p, int32_t emitter, int64_t ray_begin, int64_t ray_end,
                       int32_t *hit_out, int32_t n_threads);

/* Reference launch size for one emitter (main.cpp:172-173): threads, rounded to
 * the nearest multiple of wg (ties down); returns -1 on int32 overflow. */
int64_t rfo_ref_nthreads(int32_t ray_density, int32_t n_samples, int32_t wg);

int32_t rfo_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
