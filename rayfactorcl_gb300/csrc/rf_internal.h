// rf_internal.h -- structures shared by the host C ABI and the kernel
// translation units.  Not part of the public interface.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "rayfactor_gb300.h"

namespace rf {

// Hit-test record of one surface, 64 bytes, 16-byte aligned so that a block
// stages the table into shared memory and reads it back as four 128-bit
// broadcast loads: the three rows of invm (world->object) and
// (type as int bits, util1, util2, 0).
struct __align__(16) HitRec {
    float4 r0, r1, r2, aux;
};
static_assert(sizeof(HitRec) == 64, "HitRec layout");

// One contiguous ray range of one emitter.  Chunks of kChunkGids Philox
// draws are numbered across segments; chunk_begin is their prefix sum.
struct Segment {
    int32_t emitter;     // primitive index within its scene
    int32_t scene;       // scene index (0 for single-scene traces)
    int64_t ray_begin;   // first ray (ray r uses draw r/4, rotation r%4)
    int64_t ray_end;     // one past the last ray
    int64_t chunk_begin; // first global chunk index of this segment
};

// Per-scene offsets for the batched kernel.
struct SceneInfo {
    int32_t n;           // primitives
    int32_t prim_off;    // first record in the concatenated tables
    int64_t hits_off;    // first tally of its n x n matrix
    float eps;           // self-hit threshold on t for this scene
    int32_t pad;
};

struct TraceParams {
    const HitRec *tab;              // surface hit records, n (concatenated over scenes)
    const rf_primitive *emit;       // reference-layout records (emission)
    const HitRec *bvtab;            // bounding-surface hit records, nbv
    const int4 *bvinfo;             // bounding surfaces: (settings, start, end, 0)
    const Segment *seg;             // segments
    const SceneInfo *scenes;        // batched kernel only
    unsigned long long *hits;       // n x n tallies (or all scenes' matrices)
    int32_t *rec;                   // per-ray hit index (record mode) or null
    int64_t rec_base;               // ray index written to rec[0]
    unsigned long long *refined;    // counter of FP64 re-evaluations (mixed)
    unsigned long long *queue;      // work-queue head (batched kernel)
    int32_t *err;                   // device error flag
    int64_t total_chunks;
    int32_t nseg;
    int32_t n;                      // primitives (single-scene kernels)
    int32_t nbv;
    uint32_t compat;
    uint32_t key1;
    uint32_t scene_id;
    float eps;
    int32_t use_smem_hist;          // 1: shared-memory row histogram, 0: global atomics
    const float4 *bsph;             // batched kernel: world bounding sphere per surface
    const int64_t *d_total;         // batched kernel: device-resident chunk count (or null)
    const int32_t *d_nseg;          // batched kernel: device-resident segment count (or null)
    unsigned long long *work;       // batched kernel: [0..5] ray x surface tests by type,
                                    // [6] candidate surfaces of packets, [7] packets
    const float4 *frame;            // mixed kernels: per emitter kEmitFrameWords (planar emission frame)
    const uint32_t *cmask;          // batched kernel: cell masks of all rows that have them
    const int64_t *mask_off;        // per global row (prim_off + emitter): first mask word, -1 = none
    const float4 *bvsph;            // mixed kernels: bounding sphere of each bounding surface (as bsph)
};

// Cell masks of the batched kernel (build_masks_kernel): one bit per surface for
// each of kMaskCells sort keys of a row (scene, emitter).
constexpr int kMaskCells = 4096;
constexpr int kChainMax = 8;            // bounding spheres per surface in the mask test
constexpr int kMaskMaxSurfaces = 1024;  // scenes up to this many surfaces get masks

struct MaskRow {
    int32_t scene;
    int32_t emitter;
    int64_t off;     // first word of the row's masks (kMaskCells x ceil(n/32) words)
};

struct MaskInputs {
    const MaskRow *rows;      // sorted by off
    int32_t nrows;
    int64_t total_words;
    const SceneInfo *scenes;
    const float4 *patch;      // per global prim: 16 parameter-patch balls (centre, radius)
    const float4 *cone;       // 256 direction cells: (axis, cos theta), (sin theta, 0, 0, 0)
    const float4 *chain;      // per global prim: kChainMax spheres (centre, radius; radius < 0: none)
    const float4 *plane;      // per global prim: (unit normal, normal . point); w NaN: not planar
};

constexpr int kBlock = 256;    // maximum threads per block of the single-scene kernels
constexpr int kTile = 256;     // surface records per shared-memory tile (16 KB)
constexpr int kHistMax = 8192; // largest row kept as a shared-memory histogram

struct MExact;
struct MFast;
struct MF64;

struct LaunchCfg {
    int grid = 0;
    int block = kBlock;
    int gpt = 1;        // Philox draws per thread per chunk (4 rays each)
    size_t smem = 0;
    bool bv = false;    // runBVGPU semantics
    bool rec = false;   // write per-ray hit indices instead of tallying
    bool stage = true;  // surfaces staged in shared memory (else read through L1)
    bool serial = false; // one ray at a time against all surfaces (else a thread's rays together)
};

// Implemented once per arithmetic policy (rf_kern_exact.cu, rf_kern_fast.cu).
template <class M> cudaError_t launch_trace(const LaunchCfg &cfg, const TraceParams &p, cudaStream_t st);
template <class M> int trace_blocks_per_sm(const LaunchCfg &cfg);

// Batched mixed-precision persistent kernel (rf_kern_batched.cu); count: also
// collect the work counters (TraceParams::work); stacks: some scene's tables
// have segment stacks (kStackType).
cudaError_t launch_batched(const TraceParams &p, bool rec, bool resident, bool count, bool stacks, int grid,
                           cudaStream_t st);
// The same kernel with runBVGPU's bounding-surface semantics (one resident scene).
cudaError_t launch_batched_bv(const TraceParams &p, bool rec, bool count, bool stacks, int grid, cudaStream_t st);
int batched_blocks_per_sm(bool rec, bool resident);
cudaError_t launch_build_masks(const MaskInputs &in, uint32_t *out, cudaStream_t st);
// Mixed-precision kernel for one small scene with the plain kernel's launch shape
// (rf_kern_fast.cu): gpt Philox draws per thread, block kSmallThreads.
constexpr int kSmallMax = 64;       // surfaces of the largest scene it takes
constexpr int kSmallThreads = 256;
cudaError_t launch_mixed_small(const TraceParams &p, int gpt, bool rec, int grid, cudaStream_t st);
int mixed_small_blocks_per_sm(int gpt, bool rec);
size_t batched_smem_bytes();
int batched_tile();  // scenes with at most this many surfaces use the resident kernel
constexpr int kBatchTile = 512;  // surfaces the resident kernel keeps in shared memory
// Hit-record types of the members of segment stacks in the mixed-precision
// tables.  kStackType: consecutive cylinders [a, a + m) that tile one longer
// cylinder, each member's record holding the stack's (the first member's invm,
// aux = (kStackType, m, util2, w)).  kPlateType: consecutive concentric annuli in
// one plane and frame, each one's outer radius the next one's inner, each member
// keeping its own record with aux = (kPlateType, util1, util2, w).  w = int bits
// of (m << 16) | (offset of the member in the stack).
constexpr int kStackType = 7;
constexpr int kPlateType = 8;
constexpr int kBatchBruteMax = 12;  // scenes up to this many surfaces are traced without culling
constexpr int kEmitFrameWords = 5;  // float4 words of a planar emitter's frame (mixed kernels)
constexpr int kBatchMaxBV = 64;     // bounding surfaces the mixed kernel takes (runBVGPU semantics)
constexpr int kBatchMaxSurfaces = 32767;  // nearest hits are kept as int16 in shared memory
constexpr int kBatchChunkDraws = 8192;  // Philox draws per chunk of the batched kernel
constexpr int kBatchBlock = 1024;       // threads per block of the batched kernel

// Emission frame of an emitter for the mixed kernels (rf_capi.cu): planar
// emitters get their origin, in-plane axes and alignment rotation in FP64.
void emit_frame(const rf_primitive &e, float4 *out);

// Host preparation of one scene for the batched kernel (rf_capi.cu); eps_out
// receives the scene's self-hit threshold for the configured eps; returns the
// number of segment stacks in the tables.
int prepare_mixed_tables(const rf_primitive *prims, int n, float eps, rf_primitive *emit, HitRec *tab, float4 *bs,
                         float *eps_out);

// FP64 post-processing and probes (rf_kern_post.cu).
cudaError_t launch_normalise_single(const unsigned long long *hits, const int64_t *rays, int n,
                                    double *F, cudaStream_t st);
cudaError_t launch_converge_step(const unsigned long long *hits, int64_t *rays,
                                 const int64_t *row_off, const int32_t *row_n, int64_t nrows,
                                 double *F, double tol, int64_t *next_rays, int64_t round_rays,
                                 int32_t *not_converged, cudaStream_t st);
cudaError_t launch_plan_round(int64_t nrows, const int32_t *row_scene, const int32_t *row_emitter,
                              int64_t *rays_total, const int64_t *next, Segment *seg, int32_t *d_nseg,
                              int64_t *d_total, unsigned long long *queue, int chunk_draws, cudaStream_t st);
cudaError_t launch_decide_round(int32_t *flags, int32_t max_rounds, unsigned long long handle,
                                cudaStream_t st);
cudaError_t launch_check_F(const double *F, const double *areas, int n, double *out2,
                           cudaStream_t st);
cudaError_t launch_fp32_probe(float *out, int iters, int grid, int block, cudaStream_t st);
cudaError_t launch_smooth(const double *F, const double *A, int n, int closed, int max_iter, double tol,
                          double *G, double *x0, double *x1, double *err_dev, double *F_out, int *iters,
                          double *final_err, cudaStream_t st);

}  // namespace rf
