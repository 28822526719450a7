/*
 * rayfactor_gb300.h -- C ABI of the GB300 (sm_103a) Monte Carlo view-factor
 * tracer.  Drop-in for the tracing path of RayFactorCL: the OpenCL kernels
 * runGPU / runBVGPU (RayFactorCL/RayFactorGPU.cl:481-626) and the launch,
 * tally and normalisation logic of runCL_GPURNG (RayFactorCL/main.cpp:54-272).
 *
 * Plain C types only.  The scene tables are the reference's own structs
 * (RayFactorCL/RayfactorConstants.h:38-56) byte for byte, so a caller holding
 * a reference Scene passes &scene.primitives[0] and &scene.boundingVolumes[0]
 * unchanged.  Every function returns an rf_status; none exits the process.
 * One rf_ctx per host thread: calls on one context are not re-entrant, but
 * several contexts may share a GPU.
 */
#ifndef RAYFACTOR_GB300_H
#define RAYFACTOR_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RF_ABI_VERSION 1

/* Error codes (replace CHECK/CHECKERR -> exit(1), RayFactorCL/util_opencl.h:123-131). */
typedef enum rf_status {
    RF_OK = 0,
    RF_ERR_INVALID_ARG = 1,  /* null pointer, negative size, bad enum               */
    RF_ERR_BAD_SCENE = 2,    /* unknown type, non-finite transform, bad BV range    */
    RF_ERR_OOM = 3,          /* device or host allocation failed                    */
    RF_ERR_CUDA = 4,         /* a CUDA runtime call failed (see rf_last_error)      */
    RF_ERR_TIMEOUT = 5,      /* a bounded device wait gave up                       */
    RF_ERR_OVERFLOW = 6,     /* a ray budget or launch size does not fit            */
    RF_ERR_NO_DEVICE = 7,    /* no CUDA device / device index out of range          */
    RF_ERR_UNSUPPORTED = 8,  /* mode not available for this scene or device         */
    RF_ERR_STATE = 9         /* call order (e.g. rf_trace before rf_set_scene)      */
} rf_status;

/* RayfactorConstants.h:25-33 */
typedef enum rf_primitive_type {
    RF_CYLINDER = 0, RF_FRUSTUM = 1, RF_SPHERE = 2, RF_ANNULUS = 3,
    RF_RECTANGLE = 4, RF_DISC = 5, RF_NONE = 6
} rf_primitive_type;

/* RayfactorConstants.h:38-45 -- 112 bytes.  m / invm: row-major 3x4
 * object->world and world->object transforms; util1: frustum top radius or
 * annulus inner radius^2; util2: annulus outer radius^2 or the inward/outward
 * normal sign (-1/+1) of cylinders, frusta and spheres. */
typedef struct rf_primitive {
    float m[12];
    float invm[12];
    int32_t type;
    int32_t rayDensity;
    float util1;
    float util2;
} rf_primitive;

/* RayfactorConstants.h:48-56 -- 72 bytes.  Children are primitives
 * [objStartIndex, objEndIndex); settings == 1 tests them immediately. */
typedef struct rf_bounding_volume {
    float invm[12];
    int32_t type;
    int32_t settings;
    int32_t objStartIndex;
    int32_t objEndIndex;
    float util1;
    float util2;
} rf_bounding_volume;

/* Behaviour of the reference that is kept only on request.  RF_COMPAT_ALL
 * reproduces the reference run for run; the default (0) fixes each item. */
#define RF_COMPAT_BUDGET   (1u << 0) /* every emitter gets emitter 0's budget (main.cpp:172)  */
#define RF_COMPAT_SPHERE   (1u << 1) /* sphere discriminant without sqrt (RayFactorGPU.cl:272) */
#define RF_COMPAT_BV_STALE (1u << 2) /* stale child index across BVs (RayFactorGPU.cl:596-619) */
#define RF_COMPAT_STREAMS  (1u << 3) /* stream key {gid, key1} only: all emitters share streams
                                        (RayFactorGPU.cl:486-487)                              */
#define RF_COMPAT_ALL      (RF_COMPAT_BUDGET | RF_COMPAT_SPHERE | RF_COMPAT_BV_STALE | RF_COMPAT_STREAMS)

/* Arithmetic of the intersection code. */
typedef enum rf_precision {
    RF_PREC_EXACT = 0, /* IEEE FP32 with the fixed op mapping: per-ray bit-exact with the
                          CPU restatement of RayFactorGPU.cl (the "plain" kernel)           */
    RF_PREC_FAST = 1,  /* FP32 with hardware approximations, like OpenCL native_*           */
    RF_PREC_MIXED = 2, /* batched kernel: FP32 approximations, quadric roots that fail a
                          conditioning test recomputed in FP64                              */
    RF_PREC_FP64 = 3   /* FP64 throughout on identical streams: the FP64 tracer             */
} rf_precision;

typedef struct rf_config {
    uint32_t struct_size; /* sizeof(rf_config); set by rf_config_default                    */
    uint32_t compat;      /* RF_COMPAT_* bits                                               */
    uint32_t precision;   /* rf_precision                                                   */
    uint32_t key1;        /* Philox key word 1 (0xdecafbad in RayFactorGPU.cl:486)           */
    float eps;            /* self-hit threshold on t: >= 0 absolute (1e-3f, RayFactorGPU.cl:7);
                           * < 0 relative, |eps| x the diagonal of the scene's bounding box
                           * (per scene in a batch)                                          */
    int32_t device;       /* CUDA device ordinal                                            */
    int32_t block_size;   /* 0: autotuned / built-in default                                */
    int32_t rays_per_thread; /* 0: default; 4 or 8 (one or two Philox draws)                */
    uint32_t scene_id;    /* folded into the stream counter outside RF_COMPAT_STREAMS       */
    int32_t tally_mode;   /* 0: autotuned / default; 1: shared-memory row histogram; 2: global atomics */
    int32_t table_mode;   /* 0: autotuned / default; 1: surfaces staged in shared memory; 2: read through L1 */
    int32_t test_order;   /* 0: autotuned / default; 1: a thread's 4 or 8 rays tested together against
                           * each surface; 2: one ray at a time against all surfaces (smaller code) */
    int32_t work_counts;  /* RF_PREC_MIXED: 1 = the batched kernel also counts its tests for
                           * rf_last_work_counts (a few per cent slower); 0 = no counting      */
    int32_t batched_grid; /* RF_PREC_MIXED: 0 = one persistent block per SM; > 0 = at most this
                           * many blocks (results do not depend on it)                         */
    int32_t split_stacks; /* RF_PREC_MIXED: 0 = a segment stack is one test -- consecutive cylinders
                           * that tile one longer cylinder (a furnace wall of rings): one cylinder
                           * whose root's z names the ring; consecutive concentric annuli in one
                           * plane (an end plate of rings): one plane hit whose radius names the
                           * ring; 1 = every ring tested on its own                              */
    uint32_t reserved;
} rf_config;

typedef struct rf_ctx rf_ctx;

/* Reference-compatible defaults: compat = 0, EXACT, key1 = 0xdecafbad, eps = 1e-3. */
void rf_config_default(rf_config *cfg);

rf_status rf_create(rf_ctx **ctx, const rf_config *cfg);
void rf_destroy(rf_ctx *ctx);
const char *rf_last_error(const rf_ctx *ctx);
const char *rf_status_string(rf_status s);
int32_t rf_abi_version(void);

/* Copy a scene to the device (replaces the clCreateBuffer/clEnqueueWriteBuffer of
 * main.cpp:113-149).  The caller keeps ownership of both tables. */
rf_status rf_set_scene(rf_ctx *ctx, const rf_primitive *prims, int32_t n_prims,
                       const rf_bounding_volume *bvs, int32_t n_bvs);

/* Trace rays_per_emitter[e] rays from every emitter e (0 = skip) and tally the
 * first surface hit (RayFactorGPU.cl:481-626, one launch for all emitters
 * instead of main.cpp:168-181's launch per emitter).  use_bv selects runBVGPU
 * semantics.  hits_out: n x n int64 tallies, row = emitter (caller-owned, may be
 * NULL); F_out: n x n doubles hits/rays (main.cpp:241-249, FP64; NaN for rows
 * with no rays; may be NULL).  Synchronous. */
rf_status rf_trace(rf_ctx *ctx, const int64_t *rays_per_emitter, int32_t use_bv,
                   uint64_t *hits_out, double *F_out);

/* (No counterpart in the reference, which always starts every emitter at ray 0.)
 * Trace rays [first_ray[e], first_ray[e] + count[e]) of every emitter e and add
 * the tallies to the context's running tallies (accumulate = 1, after a trace or
 * rf_set_tallies) or start new ones (accumulate = 0).  A ray's stream depends
 * only on (emitter, ray index), so a run split into ranges -- resumed from a
 * checkpoint, or divided between processes whose tallies are summed -- gives
 * exactly the tallies of one run.  Asynchronous like rf_trace_async;
 * rf_read_results normalises by all rays traced so far. */
rf_status rf_trace_range(rf_ctx *ctx, const int64_t *first_ray, const int64_t *count,
                         int32_t use_bv, int32_t accumulate);

/* (No counterpart in the reference.)
 * Restore running tallies and ray counts (a checkpoint: n x n tallies and the
 * rays traced per emitter), to continue with rf_trace_range(accumulate = 1). */
rf_status rf_set_tallies(rf_ctx *ctx, const uint64_t *hits, const int64_t *rays_per_emitter);

/* rf_trace split in two (main.cpp:160-234 likewise enqueues, then reads back),
 * for callers that time or overlap the GPU work:
 * rf_trace_async enqueues on the context's stream and returns; rf_read_results
 * waits and copies the tallies (and F) of the last trace. */
rf_status rf_trace_async(rf_ctx *ctx, const int64_t *rays_per_emitter, int32_t use_bv);
rf_status rf_read_results(rf_ctx *ctx, uint64_t *hits_out, double *F_out);

/* (No counterpart in the reference.)  The context's CUDA stream (a cudaStream_t), for callers that record their
 * own events or order other work after a trace. */
void *rf_stream(rf_ctx *ctx);

/* In place of the reference's getticks() prints around enqueue + execute
 * (main.cpp:156-192): milliseconds of the last trace's kernels on the device (CUDA events on the
 * context's stream) and the number of kernel launches it made. */
rf_status rf_last_trace_stats(rf_ctx *ctx, double *kernel_ms, int32_t *launches);

/* (No counterpart in the reference.)  Per-ray first-hit index (-1 = none) of rays [first_ray, first_ray+n_rays) of
 * one emitter, for parity checks against the CPU restatement. */
rf_status rf_trace_rays(rf_ctx *ctx, int32_t emitter, int64_t first_ray, int64_t n_rays,
                        int32_t use_bv, int32_t *hit_index_out);

/* runCL_GPURNG (main.cpp:54-272) without the file output: budget per emitter
 * = round_to_128(rayDensity * n_samples / 4) * 4 (main.cpp:172-173;
 * RF_COMPAT_BUDGET uses emitter 0's rayDensity for all), kernel chosen by
 * use_bv (main.cpp:68-75), tallies normalised by the rays shot (main.cpp:178,
 * 241-249).  rays_out (n, may be NULL) receives the budgets. */
rf_status rf_run_gpurng(rf_ctx *ctx, int32_t n_samples, int32_t use_bv, int64_t *rays_out,
                        uint64_t *hits_out, double *F_out);

/* The budget rule alone (host arithmetic, no GPU). */
rf_status rf_ray_budgets(const rf_primitive *prims, int32_t n_prims, int32_t n_samples,
                         uint32_t compat, int64_t *rays_out);

/* Surface area of every primitive under its affine transform, in FP64 (closed
 * form for the planar types, quadrature of the parametric surface for
 * cylinders, frusta and spheres; exact for non-uniform scaling, unlike the
 * rayDensity proxies of Scene.cpp:361-387). */
rf_status rf_surface_areas(const rf_primitive *prims, int32_t n_prims, double *areas_out);

/* (No counterpart in the reference.)  The segment stacks RF_PREC_MIXED traces as
 * one test each (rf_config.split_stacks): runs of consecutive cylinders that
 * tile one longer cylinder and of consecutive concentric annuli in one plane
 * whose radii meet, never across a bounding surface's child range
 * (bvs may be NULL when n_bvs = 0).  Host only.  first_out / count_out get up to
 * cap stacks (first surface, number of surfaces); *n_stacks_out the number found. */
rf_status rf_segment_stacks(const rf_primitive *prims, int32_t n_prims, const rf_bounding_volume *bvs,
                            int32_t n_bvs, int32_t *first_out, int32_t *count_out, int32_t cap,
                            int32_t *n_stacks_out);

/* Budget planner: total_rays spread over the emitters in proportion to their
 * areas, in multiples of four (one Philox draw), at least four per non-empty
 * surface.  No int32 limits (compare main.cpp:172). */
rf_status rf_budgets_by_area(const rf_primitive *prims, int32_t n_prims, int64_t total_rays,
                             int64_t *rays_out);

/* The same with the scene file's per-primitive <rayDensity value> honoured
 * exactly: budgets proportional to density[i] * area[i] (density NULL: all 1).
 * The reference reads that value (Scene.cpp:307-321) but folds it, truncated to
 * an integer, into a truncated area proxy (Scene.cpp:362-387). */
rf_status rf_budgets_by_density(const rf_primitive *prims, int32_t n_prims, const double *density,
                                int64_t total_rays, int64_t *rays_out);

/* Write F like main.cpp:236-249: one row per emitter, 8 significant digits,
 * every value followed by a comma. */
rf_status rf_write_output_txt(const char *path, const double *F, int32_t n);

/* ---------------------------------------------------------------------------
 * Batched mixed-precision tracing: many independent scenes, many emitters with
 * uneven budgets, one persistent launch that pulls (scene, emitter, ray chunk)
 * work items from a device queue.  A scene has at most 32767 surfaces here
 * (RF_ERR_OVERFLOW beyond; the plain kernels take any number).  No counterpart
 * in the reference (one scene per run, main.cpp:275-284), nor for the FP64
 * checks and smoothing below (the reference writes raw F, main.cpp:236-249).
 * ------------------------------------------------------------------------- */
typedef struct rf_scene_desc {
    const rf_primitive *prims;
    int32_t n_prims;
    int32_t reserved;
    const int64_t *rays_per_emitter; /* initial budget per emitter (n_prims entries) */
} rf_scene_desc;

/* Trace every scene once with its budgets.  hits_out: the scenes' n_i x n_i
 * tally matrices back to back (sum n_i^2 entries); F_out likewise (may be NULL). */
rf_status rf_trace_batch(rf_ctx *ctx, const rf_scene_desc *scenes, int32_t n_scenes,
                         uint64_t *hits_out, double *F_out);

/* Convergence loop: add rays to every emitter whose row still has a binomial
 * standard error sqrt(F(1-F)/rays) above tol, until every row is below tol or
 * max_rounds rounds ran.  Each round gives such a row the rays its current
 * estimate still needs, ceil(max_j F(1-F)/tol^2) - rays rounded up to a
 * multiple of 4, but at most round_rays (and at least 4).  The round is
 * a CUDA graph (trace + FP64 normalisation + convergence test) replayed by a
 * device-side loop.  rays_out (sum n_i, may be NULL) gets the final budgets;
 * rounds_out the rounds run. */
rf_status rf_converge_batch(rf_ctx *ctx, const rf_scene_desc *scenes, int32_t n_scenes,
                            double tol, int64_t round_rays, int32_t max_rounds,
                            uint64_t *hits_out, double *F_out, int64_t *rays_out,
                            int32_t *rounds_out);

/* FP64 checks on a tally (device, FP64): max |sum_j F_ij - 1| over rows
 * (summation rule of a closed enclosure) and max |A_i F_ij - A_j F_ji| /
 * max(A_i F_ij, A_j F_ji) over pairs with both tallies non-zero (reciprocity). */
rf_status rf_check_F(rf_ctx *ctx, const double *F, const double *areas, int32_t n,
                     double *max_sum_err, double *max_recip_err);

/* Post-processing of F in FP64 on the device: the closest reciprocal F (A_i F_ij
 * = A_j F_ji, by symmetrising the exchange matrix A_i F_ij) and, when closed is
 * set (a closed enclosure), the symmetric scaling of that matrix whose rows sum
 * to A_i, i.e. sum_j F_ij = 1 with reciprocity kept.  Rows without rays (NaN)
 * count as zero.  iterations / residual (may be NULL): scaling iterations and
 * the last max_i |sum_j F_ij - 1|.  F and F_out may be the same array. */
rf_status rf_smooth_F(rf_ctx *ctx, const double *F, const double *areas, int32_t n, int32_t closed,
                      double *F_out, int32_t *iterations, double *residual);

/* (No counterpart in the reference, whose work-group size is fixed at 128,
 * util_opencl.h:52.)  Pick the launch shape of the single-scene kernels for the current scene by
 * timing runs of about 2^25 rays (spread over the emitters like the budgets of
 * the context's last trace, else evenly) of every combination of threads per block
 * (128, 256), rays per thread (4, 8), surface staging (shared-memory tiles or
 * reads through L1), tallying (shared-memory row histogram or global
 * atomics) and test order (a thread's rays together per surface, or one ray
 * at a time); the choice is cached per scene shape in memory and, when cache_path
 * is not NULL, appended to that file and read back by later processes.  Applies
 * the choice to the context.  RF_PREC_MIXED: for one scene of at most 64 surfaces, the choice
 * between the batched kernel and the small-scene kernel with 4 or 8 rays per thread (cached
 * the same way); with use_bv, a check that the scene fits the bounding-surface variant.
 * Results of a trace do not depend on the launch shape. */
rf_status rf_autotune(rf_ctx *ctx, int32_t use_bv, const char *cache_path);

/* (No counterpart in the reference.)  The launch shape the context uses now (after rf_autotune, or the defaults).
 * RF_PREC_MIXED: the kernel the next trace of the current scene without bounding surfaces takes -- block
 * 1024 and 32 rays per thread for the batched kernel, 256 and 4 or 8 for the small-scene kernel (with
 * bounding surfaces it is always the batched kernel). */
rf_status rf_get_launch_config(rf_ctx *ctx, int32_t *block, int32_t *rays_per_thread,
                               int32_t *smem_hist, int32_t *smem_table, int32_t *one_ray_at_a_time);

/* (No counterpart in the reference.)  Counters of the last mixed-precision run: tests re-evaluated in FP64. */
rf_status rf_last_refine_count(rf_ctx *ctx, uint64_t *refined_tests);

/* (No counterpart in the reference.)  Work of the last mixed-precision run made with
 * rf_config.work_counts = 1 (zeros otherwise): counts[0..5] ray x surface tests
 * performed by surface type (RF_CYLINDER..RF_DISC; with bounding surfaces, the
 * tests of their children: each ray also tests every bounding surface; a segment
 * stack's one test counts once, as its members' type), counts[6] candidate
 * surfaces the packets checked ray by ray (from the union of their rays' cell
 * masks, or the surfaces their bounds can reach; the other members of a stack
 * once it is tested are not checked), counts[7] ray packets (32 rays).  Tests
 * skipped by culling are the all-pairs count minus the sum of counts[0..5]. */
rf_status rf_last_work_counts(rf_ctx *ctx, uint64_t *counts);

/* (No counterpart in the reference.)  FP32 issue-rate probe: dependent-FMA throughput of the device in FMA/s
 * (one FMA counted as one operation), measured with CUDA events. */
rf_status rf_measure_fp32_peak(int32_t device, double *fma_per_s);

/* ---------------------------------------------------------------------------
 * Tracing without any device allocation.  No counterpart in the reference.
 *
 * For hosts that must not let a library allocate GPU memory: an application
 * that has already reserved the device's memory in its own pool, or a
 * latency-bound loop that cannot afford the device-wide synchronisation a
 * cudaMalloc may cause.  The call allocates nothing (no cudaMalloc, cudaFree
 * or other allocating routine, on the device or the host heap): the caller
 * passes the scene and budgets in host memory and the tally matrix in device
 * memory it owns; the prepared surface tables, the segment plan and the
 * work-queue counters live in one static device array of
 * RF_NOALLOC_SCRATCH_BYTES per GPU, held from library load until process exit.
 *
 * Runs the batched mixed-precision kernel on one scene of at most
 * RF_NOALLOC_MAX_PRIMS surfaces (more: RF_ERR_OVERFLOW) on the current device,
 * enqueued on `stream` (a cudaStream_t; NULL = default stream) and returning
 * without waiting: hits_dev (n x n uint64, zeroed by the call) holds the
 * tallies once the stream reaches that point.  The tallies equal those of
 * rf_trace on a context with precision RF_PREC_MIXED, scene_id 0 and the same
 * compat, key1 and eps (eps >= 0 absolute, eps < 0 relative to the scene's
 * bounding-box diagonal, as in rf_config; segment stacks as rf_config.split_stacks = 0).
 * The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress).  Every call reuses the same array and clears what must start at
 * zero; calls whose GPU work overlaps (other streams, other host threads) race
 * on it and must be serialised by the caller.
 * ------------------------------------------------------------------------- */
#define RF_NOALLOC_MAX_PRIMS 512
#define RF_NOALLOC_SCRATCH_BYTES (160 * 1024)

rf_status rf_trace_mixed_noalloc(const rf_primitive *prims, int32_t n_prims,
                                 const int64_t *rays_per_emitter, uint32_t compat, uint32_t key1,
                                 float eps, uint64_t *hits_dev, void *stream);

#ifdef __cplusplus
}
#endif
#endif
