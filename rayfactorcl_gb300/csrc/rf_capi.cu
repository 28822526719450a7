// rf_capi.cu -- the C ABI (include/rayfactor_gb300.h): contexts, scene
// validation and upload, launch planning, tallies, normalisation and output.
//
// Replaces runCL_GPURNG (RayFactorCL/main.cpp:54-272) and the OpenCL device
// layer (RayFactorCL/util_opencl.h:133-352) with the CUDA runtime on one GPU.
#include <algorithm>
#include <array>
#include <utility>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <limits>
#include <map>
#include <mutex>
#include <new>
#include <sstream>
#include <string>
#include <vector>

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include "rayfactor_gb300.h"
#include "rf_internal.h"

using namespace rf;

namespace {
// NVTX range around an API call (a no-op unless a profiler is attached).
struct ApiRange {
    explicit ApiRange(const char *name) { nvtxRangePushA(name); }
    ~ApiRange() { nvtxRangePop(); }
    ApiRange(const ApiRange &) = delete;
    ApiRange &operator=(const ApiRange &) = delete;
};
}  // namespace

namespace {

constexpr int32_t kMaxPrims = 16384;            // n x n int64 tallies: 2 GiB
constexpr int64_t kMaskBudgetWords = 1ll << 28;  // cell masks of one upload: at most 1 GiB
constexpr int64_t kMaxRaysPerEmitter = 1ll << 46;

struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes)
    {
        if (bytes <= cap && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        size_t want = std::max<size_t>(bytes, 256);
        cudaError_t e = cudaMalloc(&p, want);
        if (e == cudaSuccess) cap = want;
        return e;
    }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
    template <class T> T *as() const { return static_cast<T *>(p); }
};

struct PinBuf {
    void *p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes)
    {
        if (bytes <= cap && p) return cudaSuccess;
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
        size_t want = std::max<size_t>(bytes, 256);
        cudaError_t e = cudaMallocHost(&p, want);
        if (e == cudaSuccess) cap = want;
        return e;
    }
    void release()
    {
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
    }
    template <class T> T *as() const { return static_cast<T *>(p); }
};

}  // namespace

struct rf_ctx {
    rf_config cfg{};
    int device = 0;
    int sms = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::string err;

    // scene
    int32_t n = 0, nbv = 0;
    float eps = 1e-3f;  // the scene's self-hit threshold (cfg.eps, or scaled when negative)
    std::vector<rf_primitive> prims;
    DevBuf d_tab, d_emit, d_bvtab, d_bvinfo;

    // trace state
    DevBuf d_hits, d_seg, d_rays, d_F, d_rec, d_err, d_misc;
    PinBuf h_seg, h_rays, h_misc;
    std::vector<Segment> seg_cache;  // the plan in d_seg when seg_valid
    bool seg_valid = false;
    std::vector<int64_t> last_rays;
    bool have_results = false;
    int last_launches = 0;
    bool timed = false;

    // launch choices (0 / -1 = default); set by rf_config or rf_autotune
    int block = 0, gpt = 0, hist = -1, stage = -1, order = -1;  // order 1: one ray at a time

    // batched mixed-precision path: scenes concatenated, re-centred in FP64
    DevBuf b_tab, b_emit, b_bsph, b_scenes, b_hits, b_rows, b_counters;
    // cell masks of the batched kernel and their inputs (built at upload)
    DevBuf b_patch, b_chain, b_plane, b_cone, b_maskrows, b_maskoff, b_mask, b_frame;
    DevBuf b_bvtab, b_bvinfo, b_bvsph;  // the single scene's bounding surfaces, re-centred like its surfaces
    bool b_masks = false;
    double b_mask_ms = 0.0;     // device time of the last mask build
    std::vector<SceneInfo> b_info;
    int64_t b_hits_total = 0;
    bool b_single = false;      // b_* hold the scene of rf_set_scene
    unsigned long long last_refined = 0;
    unsigned long long last_work[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    // single-scene MIXED traces: 0 = by surface count, 1 = small-scene kernel,
    // 2 = batched kernel (set by rf_autotune)
    int mixed_path = 0;
    int b_stacks = 0;  // segment stacks in the mixed tables
    std::vector<int> b_test_type;  // scene 0 of the mixed tables: type each surface's test counts as
                                   // (a stack: RF_CYLINDER at its first member, -1 at the others)
    bool last_small = false;                 // the last MIXED launch was the small-scene kernel
    unsigned long long small_work[8] = {0, 0, 0, 0, 0, 0, 0, 0};
};

namespace {

rf_status fail(rf_ctx *c, rf_status s, const char *fmt, ...)
{
    if (c) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        c->err = buf;
    }
    return s;
}

rf_status cuda_fail(rf_ctx *c, cudaError_t e, const char *what)
{
    if (e == cudaErrorMemoryAllocation)
        return fail(c, RF_ERR_OOM, "%s: %s", what, cudaGetErrorString(e));
    return fail(c, RF_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define RF_CUDA(ctx, call)                                   \
    do {                                                     \
        cudaError_t e_ = (call);                             \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
    } while (0)

bool finite_all(const float *v, int k)
{
    for (int i = 0; i < k; ++i)
        if (!std::isfinite(v[i])) return false;
    return true;
}

bool uses_util1(int t) { return t == RF_FRUSTUM || t == RF_ANNULUS; }
bool uses_util2(int t) { return t != RF_DISC && t != RF_RECTANGLE; }

HitRec make_hitrec(const float *invm, int type, float util1, float util2)
{
    HitRec h;
    h.r0 = make_float4(invm[0], invm[1], invm[2], invm[3]);
    h.r1 = make_float4(invm[4], invm[5], invm[6], invm[7]);
    h.r2 = make_float4(invm[8], invm[9], invm[10], invm[11]);
    float t;
    int32_t ti = type;
    std::memcpy(&t, &ti, 4);
    h.aux = make_float4(t, uses_util1(type) ? util1 : 0.f, uses_util2(type) ? util2 : 0.f, 0.f);
    return h;
}

int arith_of(const rf_ctx *c)
{
    return (int)c->cfg.precision;
}

// Occupancy of the kernel that will run; 0 when the query fails.
int blocks_per_sm(int arith, const LaunchCfg &lc)
{
    switch (arith) {
    case RF_PREC_EXACT: return trace_blocks_per_sm<MExact>(lc);
    case RF_PREC_FAST: return trace_blocks_per_sm<MFast>(lc);
    case RF_PREC_FP64: return trace_blocks_per_sm<MF64>(lc);
    default: return trace_blocks_per_sm<MFast>(lc);
    }
}

cudaError_t launch_arith(int arith, const LaunchCfg &lc, const TraceParams &p, cudaStream_t st)
{
    switch (arith) {
    case RF_PREC_EXACT: return launch_trace<MExact>(lc, p, st);
    case RF_PREC_FAST: return launch_trace<MFast>(lc, p, st);
    case RF_PREC_FP64: return launch_trace<MF64>(lc, p, st);
    default: return launch_trace<MFast>(lc, p, st);
    }
}

rf_status check_budgets(rf_ctx *c, const int64_t *rays, int n)
{
    for (int e = 0; e < n; ++e) {
        if (rays[e] < 0) return fail(c, RF_ERR_INVALID_ARG, "rays_per_emitter[%d] = %lld < 0", e, (long long)rays[e]);
        if (rays[e] > kMaxRaysPerEmitter)
            return fail(c, RF_ERR_OVERFLOW, "rays_per_emitter[%d] = %lld exceeds 2^46", e, (long long)rays[e]);
        if ((c->cfg.compat & RF_COMPAT_STREAMS) && rays[e] > (4ll << 32))
            return fail(c, RF_ERR_OVERFLOW,
                        "emitter %d: %lld rays exceed the 2^32 draws of the reference stream key", e,
                        (long long)rays[e]);
    }
    return RF_OK;
}

// Segments [first_ray, first_ray + count) per emitter, chunked by chunk_gids draws.
int64_t plan_segments(std::vector<Segment> &seg, int emitter, int scene, int64_t first,
                      int64_t count, int64_t chunk_gids, int64_t chunk0)
{
    if (count <= 0) return chunk0;
    Segment s;
    s.emitter = emitter;
    s.scene = scene;
    s.ray_begin = first;
    s.ray_end = first + count;
    s.chunk_begin = chunk0;
    const int64_t g0 = first >> 2, g1 = (first + count + 3) >> 2;
    const int64_t chunks = (g1 - g0 + chunk_gids - 1) / chunk_gids;
    seg.push_back(s);
    return chunk0 + chunks;
}

struct Plan {
    LaunchCfg lc;
    bool hist = false;
    bool stage = true;
};

// Launch shape for the single-scene kernels.
Plan make_plan(rf_ctx *c, bool bv, bool rec)
{
    Plan pl;
    pl.lc.bv = bv;
    pl.lc.rec = rec;
    pl.lc.block = c->block > 0 ? c->block : (c->cfg.block_size > 0 ? c->cfg.block_size : kBlock);
    pl.lc.block = std::max(32, std::min(kBlock, pl.lc.block / 32 * 32));
    int gpt = c->gpt > 0 ? c->gpt : (c->cfg.rays_per_thread == 8 ? 2 : 1);
    if (bv || rec || c->cfg.precision == RF_PREC_FP64) gpt = 1;
    pl.lc.gpt = gpt;
    pl.hist = !rec && (c->hist >= 0 ? c->hist == 1 : true) && c->n <= kHistMax;
    pl.stage = !bv && (rec || (c->stage >= 0 ? c->stage == 1 : true));
    pl.lc.stage = pl.stage;
    pl.lc.serial = !bv && !rec && c->order == 1;
    const int tab = pl.stage ? std::min(c->n, kTile) : 0;
    pl.lc.smem = (size_t)tab * sizeof(HitRec) + (pl.hist ? (size_t)c->n * 4 : 0);
    return pl;
}

// Put a launch's segment plan in d_seg, unless it is the plan already there (a trace
// repeated with the same budgets): then nothing is copied and nothing waits, so the
// host can queue the next launch while the GPU runs the previous one.  Otherwise the
// pinned staging buffer may still feed an earlier copy: wait for the stream first.
rf_status upload_segments(rf_ctx *c, const std::vector<Segment> &seg)
{
    const size_t bytes = seg.size() * sizeof(Segment);
    if (c->seg_valid && c->seg_cache.size() == seg.size() && std::memcmp(c->seg_cache.data(), seg.data(), bytes) == 0)
        return RF_OK;
    c->seg_valid = false;
    RF_CUDA(c, c->h_seg.ensure(bytes));
    RF_CUDA(c, c->d_seg.ensure(bytes));
    RF_CUDA(c, cudaStreamSynchronize(c->stream));
    std::memcpy(c->h_seg.p, seg.data(), bytes);
    RF_CUDA(c, cudaMemcpyAsync(c->d_seg.p, c->h_seg.p, bytes, cudaMemcpyHostToDevice, c->stream));
    c->seg_cache = seg;
    c->seg_valid = true;
    return RF_OK;
}

rf_status run_trace(rf_ctx *c, const std::vector<Segment> &seg, int64_t total_chunks, Plan &pl,
                    int32_t *d_rec, int64_t rec_base, bool zero_hits)
{
    const int n = c->n;
    if (zero_hits) RF_CUDA(c, cudaMemsetAsync(c->d_hits.p, 0, (size_t)n * n * 8, c->stream));
    c->last_launches = 0;
    c->timed = false;
    if (seg.empty() || total_chunks == 0) return RF_OK;
    if (rf_status st = upload_segments(c, seg); st != RF_OK) return st;

    TraceParams p{};
    p.tab = c->d_tab.as<HitRec>();
    p.emit = c->d_emit.as<rf_primitive>();
    p.bvtab = c->d_bvtab.as<HitRec>();
    p.bvinfo = c->d_bvinfo.as<int4>();
    p.seg = c->d_seg.as<Segment>();
    p.hits = c->d_hits.as<unsigned long long>();
    p.rec = d_rec;
    p.rec_base = rec_base;
    p.err = c->d_err.as<int32_t>();
    p.total_chunks = total_chunks;
    p.nseg = (int32_t)seg.size();
    p.n = n;
    p.nbv = c->nbv;
    p.compat = c->cfg.compat;
    p.key1 = c->cfg.key1;
    p.scene_id = c->cfg.scene_id;
    p.eps = c->eps;
    p.use_smem_hist = pl.hist ? 1 : 0;

    const int arith = arith_of(c);
    int bps = blocks_per_sm(arith, pl.lc);
    if (bps <= 0) bps = 1;
    const int64_t wave = (int64_t)c->sms * bps;
    pl.lc.grid = (int)std::max<int64_t>(1, std::min<int64_t>(wave, total_chunks));
    RF_CUDA(c, cudaEventRecord(c->ev0, c->stream));
    RF_CUDA(c, launch_arith(arith, pl.lc, p, c->stream));
    RF_CUDA(c, cudaEventRecord(c->ev1, c->stream));
    c->last_launches = 1;
    c->timed = true;
    return RF_OK;
}

rf_status validate_prims(rf_ctx *c, const rf_primitive *prims, int32_t n, int scene)
{
    if (!prims || n <= 0) return fail(c, RF_ERR_INVALID_ARG, "scene %d: empty (n_prims = %d)", scene, n);
    if (n > kMaxPrims) return fail(c, RF_ERR_OVERFLOW, "scene %d: %d primitives exceed %d", scene, n, kMaxPrims);
    for (int i = 0; i < n; ++i) {
        const rf_primitive &p = prims[i];
        if (p.type < 0 || p.type > RF_DISC)
            return fail(c, RF_ERR_BAD_SCENE, "scene %d primitive %d: type %d is not a surface", scene, i, p.type);
        if (!finite_all(p.m, 12) || !finite_all(p.invm, 12))
            return fail(c, RF_ERR_BAD_SCENE, "scene %d primitive %d: non-finite transform", scene, i);
        if ((uses_util1(p.type) && !std::isfinite(p.util1)) || (uses_util2(p.type) && !std::isfinite(p.util2)))
            return fail(c, RF_ERR_BAD_SCENE, "scene %d primitive %d: non-finite util1/util2", scene, i);
    }
    return RF_OK;
}

// The kernel's ray/sphere test takes the squared radius, widened by 1 % for
// directions that are unit only to ~1e-3 and for FP32 rounding.
float4 widen_sq(float4 b)
{
    const double r = (double)b.w * 1.01 + 1e-6 + 1e-6 * std::sqrt((double)b.x * b.x + (double)b.y * b.y + (double)b.z * b.z);
    return make_float4(b.x, b.y, b.z, (float)(r * r));
}

// Bounding sphere (centre, radius) of the object-space box [-ext, ext]^2 x [z0, z1]
// under a re-centred record's m, with a margin for FP32 rounding.
float4 object_box_sphere(const rf_primitive &e, double ext, double z0, double z1)
{
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300}, pts[8][3];
    for (int q = 0; q < 8; ++q) {
        const double o[3] = {(q & 1) ? ext : -ext, (q & 2) ? ext : -ext, (q & 4) ? z1 : z0};
        for (int k = 0; k < 3; ++k) {
            const float *r = e.m + 4 * k;
            pts[q][k] = r[0] * o[0] + r[1] * o[1] + r[2] * o[2] + r[3];
            lo[k] = std::min(lo[k], pts[q][k]);
            hi[k] = std::max(hi[k], pts[q][k]);
        }
    }
    const double cx = 0.5 * (lo[0] + hi[0]), cy = 0.5 * (lo[1] + hi[1]), cz = 0.5 * (lo[2] + hi[2]);
    double rad = 0.0;
    for (int q = 0; q < 8; ++q) {
        const double dx = pts[q][0] - cx, dy = pts[q][1] - cy, dz = pts[q][2] - cz;
        rad = std::max(rad, std::sqrt(dx * dx + dy * dy + dz * dz));
    }
    const double cn = std::sqrt(cx * cx + cy * cy + cz * cz);
    return make_float4((float)cx, (float)cy, (float)cz, (float)(rad * (1.0 + 1e-5) + 1e-6 * (cn + rad) + 1e-7));
}

// Bounding sphere of a surface (object-space box [-ext,ext]^2 x [z0,z1] by type)
// under a re-centred record's m.
float4 surface_sphere(const rf_primitive &e)
{
    double ext = 1.0, z0 = 0.0, z1 = 0.0;
    switch (e.type) {
    case RF_CYLINDER: z1 = 1.0; break;
    case RF_FRUSTUM: ext = std::max(1.0, std::fabs((double)e.util1)); z1 = 1.0; break;
    case RF_SPHERE: z0 = -1.0; z1 = 1.0; break;
    case RF_ANNULUS: ext = std::sqrt(std::max(0.0, (double)e.util2)); break;
    default: break;
    }
    return object_box_sphere(e, ext, z0, z1);
}

// Mixed-precision tables of one scene.  The world origin moves (in FP64) to the
// mean of the surfaces' translations, so a scene placed far from the origin keeps
// its FP32 resolution: m' = m - anchor, invm' = invm o (x + anchor).  Each surface
// also gets a conservative world bounding sphere (its object-space box mapped by m').
void prepare_mixed(const rf_primitive *prims, int n, rf_primitive *emit, HitRec *tab, float4 *bs)
{
    double a[3] = {0, 0, 0};
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k) a[k] += prims[i].m[4 * k + 3];
    for (int k = 0; k < 3; ++k) a[k] /= n;
    for (int i = 0; i < n; ++i) {
        rf_primitive e = prims[i];
        for (int k = 0; k < 3; ++k) {
            e.m[4 * k + 3] = (float)((double)prims[i].m[4 * k + 3] - a[k]);
            const float *r = prims[i].invm + 4 * k;
            e.invm[4 * k + 3] = (float)((double)r[3] + (double)r[0] * a[0] + (double)r[1] * a[1] + (double)r[2] * a[2]);
        }
        emit[i] = e;
        tab[i] = make_hitrec(e.invm, e.type, e.util1, e.util2);
        bs[i] = surface_sphere(e);
    }
}

// Segment stacks of one scene's mixed tables, runs [a, a + m) of 2 <= m <= 65535
// consecutive surfaces.  Cylinder stacks (kStackType): the same linear part of m
// (axes and radii), the same normal sign (util2) and each translation one axis
// column (m's third column) past the previous one's, so that member k is the
// first member shifted by k lengths along its axis (to 1e-6 of the transform's
// scale); each member's record becomes the stack's -- the first member's invm,
// aux = (kStackType, m, util2, w).  Plates (kPlateType): annuli with bit-equal
// transforms, each one's util2 (outer radius squared) bit-equal to the next
// one's util1; each member keeps its record with aux = (kPlateType, util1, util2,
// w).  w = int bits of (m << 16) | k for member k.  A stack never continues
// across an index i with cut[i] set (a bounding surface's children start or end
// there).  Every member's bounding sphere becomes the stack's.  Returns the
// number of stacks.
int mark_stacks(const rf_primitive *e, int n, HitRec *tab, float4 *bs, const std::vector<char> &cut)
{
    auto cont = [&](int j) { return j < n && !((size_t)j < cut.size() && cut[j]); };
    int nstacks = 0;
    for (int i = 0; i < n;) {
        int j = i + 1;
        if (e[i].type == RF_ANNULUS) {
            while (cont(j) && j - i < 65535 && e[j].type == RF_ANNULUS &&
                   std::memcmp(e[j].m, e[i].m, sizeof e[i].m) == 0 &&
                   std::memcmp(e[j].invm, e[i].invm, sizeof e[i].invm) == 0 && e[j].util1 == e[j - 1].util2 &&
                   e[j].util1 < e[j].util2 && e[j - 1].util1 < e[j - 1].util2)
                ++j;
            const int m = j - i;
            if (m >= 2) {
                const float4 sph = object_box_sphere(e[i], std::sqrt((double)e[j - 1].util2), 0.0, 0.0);
                for (int k = 0; k < m; ++k) {
                    int32_t ti = kPlateType, w = (m << 16) | k;
                    std::memcpy(&tab[i + k].aux.x, &ti, 4);
                    std::memcpy(&tab[i + k].aux.w, &w, 4);
                    bs[i + k] = sph;
                }
                ++nstacks;
            }
            i = j;
            continue;
        }
        if (e[i].type == RF_CYLINDER) {
            double scale = 0.0;  // largest column of the linear part
            for (int col = 0; col < 3; ++col) {
                double c2 = 0.0;
                for (int r = 0; r < 3; ++r) c2 += (double)e[i].m[4 * r + col] * e[i].m[4 * r + col];
                scale = std::max(scale, std::sqrt(c2));
            }
            while (cont(j) && j - i < 65535 && e[j].type == RF_CYLINDER && e[j].util2 == e[i].util2) {
                bool ok = true;
                for (int r = 0; r < 3 && ok; ++r) {
                    for (int col = 0; col < 3 && ok; ++col)
                        ok = std::fabs((double)e[j].m[4 * r + col] - e[i].m[4 * r + col]) <= 1e-6 * scale;
                    const double want = (double)e[j - 1].m[4 * r + 3] + e[i].m[4 * r + 2];
                    ok = ok && std::fabs((double)e[j].m[4 * r + 3] - want) <= 1e-6 * (scale + std::fabs(want));
                }
                if (!ok) break;
                ++j;
            }
        }
        const int m = j - i;
        if (m >= 2) {
            HitRec u = tab[i];
            int32_t ti = kStackType;
            std::memcpy(&u.aux.x, &ti, 4);
            u.aux.y = (float)m;
            const float4 sph = object_box_sphere(e[i], 1.0, 0.0, (double)m);
            for (int k = 0; k < m; ++k) {
                tab[i + k] = u;
                const int32_t w = (m << 16) | k;
                std::memcpy(&tab[i + k].aux.w, &w, 4);
                bs[i + k] = sph;
            }
            ++nstacks;
        }
        i = j;
    }
    return nstacks;
}

// Self-hit threshold of a scene: eps >= 0 is absolute (the reference's 1e-3,
// RayFactorGPU.cl:7); eps < 0 is relative, |eps| times the diagonal of the box
// around the surfaces' bounding spheres, so thin surfaces (a fibre of radius
// 6e-5 under the reference's absolute 1e-3) and large scenes get one threshold
// scaled to the scene.
float scene_eps(float eps, const float4 *bs, int n)
{
    if (eps >= 0.0f || n <= 0) return eps;
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int i = 0; i < n; ++i) {
        const double c[3] = {bs[i].x, bs[i].y, bs[i].z};
        for (int k = 0; k < 3; ++k) {
            lo[k] = std::min(lo[k], c[k] - (double)bs[i].w);
            hi[k] = std::max(hi[k], c[k] + (double)bs[i].w);
        }
    }
    const double dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
    return (float)(-(double)eps * std::sqrt(dx * dx + dy * dy + dz * dz));
}

// --- cell-mask inputs (FP64 on the host, in the scene's re-centred frame) ---

// World point of an object-space point under a re-centred record's m.
void xf_point(const rf_primitive &e, const double o[3], double w[3])
{
    for (int k = 0; k < 3; ++k) {
        const float *r = e.m + 4 * k;
        w[k] = (double)r[0] * o[0] + (double)r[1] * o[1] + (double)r[2] * o[2] + (double)r[3];
    }
}

// Candidate angles of an angular interval for the extremes of sin and cos:
// its ends and the multiples of pi/2 inside it.
int angle_candidates(double t0, double t1, double *out)
{
    int k = 0;
    out[k++] = t0;
    out[k++] = t1;
    for (int q = 0; q <= 8; ++q) {
        const double a = q * (M_PI / 2);
        if (a > t0 && a < t1) out[k++] = a;
    }
    return k;
}

// Object-space box of parameter patch (pi, pj) of an emitter -- the points its
// rays start from when r[0] in [pi/4, (pi+1)/4) and r[1] in [pj/4, (pj+1)/4)
// (emission formulas RayFactorGPU.cl:298-443).  Each coordinate is linear in the
// radius-like parameter for a fixed angle, and the angle's extremes are at the
// ends of its interval or at multiples of pi/2, so the listed points bound the
// patch.  Returns false when the formulas give no finite point (a frustum whose
// top radius is 1).
bool patch_box(const rf_primitive &e, int pi, int pj, double lo[3], double hi[3])
{
    const double a0 = pi / 4.0, a1 = (pi + 1) / 4.0, b0 = pj / 4.0, b1 = (pj + 1) / 4.0;
    const double u1 = e.util1, u2 = e.util2;
    double th[16], pts[64][3];
    int np = 0, nt;
    auto add = [&](double x, double y, double z) {
        pts[np][0] = x; pts[np][1] = y; pts[np][2] = z; ++np;
    };
    switch (e.type) {
    case RF_DISC:
    case RF_ANNULUS: {
        double r0, r1;
        if (e.type == RF_DISC) { r0 = std::sqrt(b0); r1 = std::sqrt(b1); }
        else {
            r0 = std::sqrt(std::max(0.0, u1 + (u2 - u1) * b0));
            r1 = std::sqrt(std::max(0.0, u1 + (u2 - u1) * b1));
        }
        nt = angle_candidates(2 * M_PI * a0, 2 * M_PI * a1, th);
        for (int k = 0; k < nt; ++k)
            for (double r : {r0, r1}) add(r * std::sin(th[k]), r * std::cos(th[k]), 0.0);
        break;
    }
    case RF_RECTANGLE:
        for (double x : {2 * a0 - 1, 2 * a1 - 1})
            for (double y : {2 * b0 - 1, 2 * b1 - 1}) add(x, y, 0.0);
        break;
    case RF_CYLINDER:
        nt = angle_candidates(2 * M_PI * a0, 2 * M_PI * a1, th);
        for (int k = 0; k < nt; ++k)
            for (double z : {b0, b1}) add(std::cos(th[k]), std::sin(th[k]), z);
        break;
    case RF_FRUSTUM: {
        auto zf = [&](double a) { return (std::sqrt(1.0 - a + a * u1 * u1) - 1.0) / (u1 - 1.0); };
        const double z0 = zf(a0), z1 = zf(a1);
        if (!std::isfinite(z0) || !std::isfinite(z1)) return false;
        nt = angle_candidates(2 * M_PI * b0, 2 * M_PI * b1, th);
        for (int k = 0; k < nt; ++k)
            for (double z : {z0, z1}) {
                const double rho = 1.0 + z * (u1 - 1.0);
                add(rho * std::cos(th[k]), rho * std::sin(th[k]), z);
            }
        break;
    }
    case RF_SPHERE: {
        double zs[3] = {2 * a0 - 1, 2 * a1 - 1, 0.0};
        const int nz = (zs[0] < 0.0 && zs[1] > 0.0) ? 3 : 2;
        nt = angle_candidates(2 * M_PI * b0, 2 * M_PI * b1, th);
        for (int k = 0; k < nt; ++k)
            for (int q = 0; q < nz; ++q) {
                const double rho = std::sqrt(std::max(0.0, 1.0 - zs[q] * zs[q]));
                add(rho * std::cos(th[k]), rho * std::sin(th[k]), zs[q]);
            }
        break;
    }
    default:
        return false;
    }
    for (int k = 0; k < 3; ++k) { lo[k] = 1e300; hi[k] = -1e300; }
    for (int q = 0; q < np; ++q)
        for (int k = 0; k < 3; ++k) {
            lo[k] = std::min(lo[k], pts[q][k]);
            hi[k] = std::max(hi[k], pts[q][k]);
        }
    return true;
}

// Ball around the image of an object-space box: the image of the box centre and
// the farthest image of a corner (the image is a parallelepiped), widened for
// the FP32 emission's rounding and approximations.
float4 box_ball(const rf_primitive &e, const double lo[3], const double hi[3])
{
    const double oc[3] = {0.5 * (lo[0] + hi[0]), 0.5 * (lo[1] + hi[1]), 0.5 * (lo[2] + hi[2])};
    double c[3], rad = 0.0;
    xf_point(e, oc, c);
    for (int q = 0; q < 8; ++q) {
        const double o[3] = {(q & 1) ? hi[0] : lo[0], (q & 2) ? hi[1] : lo[1], (q & 4) ? hi[2] : lo[2]};
        double w[3];
        xf_point(e, o, w);
        rad = std::max(rad, std::sqrt((w[0] - c[0]) * (w[0] - c[0]) + (w[1] - c[1]) * (w[1] - c[1]) +
                                      (w[2] - c[2]) * (w[2] - c[2])));
    }
    const double cn = std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
    return make_float4((float)c[0], (float)c[1], (float)c[2], (float)(rad * (1 + 1e-4) + 1e-5 * (cn + rad) + 1e-7));
}

// Sixteen parameter-patch balls of an emitter (infinite radius when a patch has
// no finite bound: every surface is then a candidate).
void patch_balls(const rf_primitive &e, float4 *out)
{
    for (int pi = 0; pi < 4; ++pi)
        for (int pj = 0; pj < 4; ++pj) {
            double lo[3], hi[3];
            out[4 * pi + pj] = patch_box(e, pi, pj, lo, hi) ? box_ball(e, lo, hi)
                                                            : make_float4(0.f, 0.f, 0.f, INFINITY);
        }
}

// Spheres covering a surface: for a cylinder or frustum longer than it is wide,
// a chain of up to kChainMax spheres along its axis (points A + rho(z) (c0 cos +
// c1 sin) + Z z of slab [z0, z1] lie within rmax * max rho + |Z| (z1 - z0) / 2 of
// the slab's axis midpoint, rmax the largest radius of the ellipse spanned by the
// first two columns); otherwise the bounding sphere `bs` (radius in w).
int surface_chain(const rf_primitive &e, float4 bs, float4 *out)
{
    for (int k = 0; k < kChainMax; ++k) out[k] = make_float4(0.f, 0.f, 0.f, -1.f);
    out[0] = bs;
    if (e.type != RF_CYLINDER && e.type != RF_FRUSTUM) return 1;
    double A[3], Z[3], c0[3], c1[3];
    for (int k = 0; k < 3; ++k) {
        A[k] = e.m[4 * k + 3];
        c0[k] = e.m[4 * k + 0];
        c1[k] = e.m[4 * k + 1];
        Z[k] = e.m[4 * k + 2];
    }
    const double L = std::sqrt(Z[0] * Z[0] + Z[1] * Z[1] + Z[2] * Z[2]);
    const double g00 = c0[0] * c0[0] + c0[1] * c0[1] + c0[2] * c0[2];
    const double g11 = c1[0] * c1[0] + c1[1] * c1[1] + c1[2] * c1[2];
    const double g01 = c0[0] * c1[0] + c0[1] * c1[1] + c0[2] * c1[2];
    const double rmax = std::sqrt(0.5 * (g00 + g11 + std::sqrt((g00 - g11) * (g00 - g11) + 4 * g01 * g01)));
    const double top = e.type == RF_FRUSTUM ? (double)e.util1 : 1.0;
    const double wide = rmax * std::max(1.0, std::fabs(top));
    if (!(L > 0.0) || !(wide > 0.0) || !std::isfinite(L + wide)) return 1;
    const int K = (int)std::min<double>(kChainMax, std::ceil(L / wide));
    if (K < 2) return 1;
    for (int k = 0; k < K; ++k) {
        const double z0 = (double)k / K, z1 = (double)(k + 1) / K, zm = 0.5 * (z0 + z1);
        const double rho = std::max(std::fabs(1.0 + z0 * (top - 1.0)), std::fabs(1.0 + z1 * (top - 1.0)));
        const double c[3] = {A[0] + Z[0] * zm, A[1] + Z[1] * zm, A[2] + Z[2] * zm};
        const double r = rmax * rho + 0.5 * L * (z1 - z0);
        const double cn = std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
        out[k] = make_float4((float)c[0], (float)c[1], (float)c[2], (float)(r * (1 + 1e-4) + 1e-5 * (cn + r) + 1e-7));
    }
    return K;
}

// Plane of a disc, annulus or rectangle: object z = 0 is row 2 of invm.
float4 surface_plane(const rf_primitive &e)
{
    if (e.type != RF_DISC && e.type != RF_ANNULUS && e.type != RF_RECTANGLE) return make_float4(0.f, 0.f, 0.f, NAN);
    const double n[3] = {e.invm[8], e.invm[9], e.invm[10]};
    const double nn = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    if (!(nn > 0.0)) return make_float4(0.f, 0.f, 0.f, NAN);
    return make_float4((float)(n[0] / nn), (float)(n[1] / nn), (float)(n[2] / nn), (float)(-(double)e.invm[11] / nn));
}

// Unit direction of octahedral-map point (u, v): the inverse of the map that
// the kernel's direction_cell applies.
void oct_dir(double u, double v, double d[3])
{
    if (std::fabs(u) + std::fabs(v) <= 1.0) {
        d[0] = u; d[1] = v; d[2] = 1.0 - std::fabs(u) - std::fabs(v);
    } else {
        d[0] = (1.0 - std::fabs(v)) * (u < 0 ? -1.0 : 1.0);
        d[1] = (1.0 - std::fabs(u)) * (v < 0 ? -1.0 : 1.0);
        d[2] = -(std::fabs(u) + std::fabs(v) - 1.0);
    }
    const double l = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    d[0] /= l; d[1] /= l; d[2] /= l;
}

// Cones of the 256 direction cells, indexed by the kernel's Morton code: axis
// through the cell's boundary samples, half-angle = the largest angle to a
// sample (the angle to a fixed axis peaks on the cell's boundary) plus 0.01 rad,
// far more than the gap between samples (the map moves directions by at most
// ~2.5 rad per unit of (u, v); samples are 1/2048 apart) and than the kernel's
// rounding when it assigns a direction to a cell.
const std::vector<float4> &direction_cones()
{
    static std::vector<float4> cones;
    static std::once_flag once;
    std::call_once(once, [] {
        cones.assign(512, make_float4(0.f, 0.f, 0.f, 0.f));
        constexpr int kS = 256;
        for (int i = 0; i < 16; ++i)
            for (int j = 0; j < 16; ++j) {
                const double u0 = -1 + i / 8.0, v0 = -1 + j / 8.0, h = 1 / 8.0;
                std::vector<std::array<double, 3>> smp;
                for (int q = 0; q <= kS; ++q) {
                    const double f = (double)q / kS;
                    const double uv[4][2] = {{u0 + f * h, v0}, {u0 + f * h, v0 + h}, {u0, v0 + f * h}, {u0 + h, v0 + f * h}};
                    for (auto &p : uv) {
                        std::array<double, 3> d;
                        oct_dir(p[0], p[1], d.data());
                        smp.push_back(d);
                    }
                }
                double ax[3] = {0, 0, 0};
                for (auto &d : smp)
                    for (int k = 0; k < 3; ++k) ax[k] += d[k];
                const double al = std::sqrt(ax[0] * ax[0] + ax[1] * ax[1] + ax[2] * ax[2]);
                for (int k = 0; k < 3; ++k) ax[k] /= al;
                double th = 0.0;
                for (auto &d : smp)
                    th = std::max(th, std::acos(std::min(1.0, d[0] * ax[0] + d[1] * ax[1] + d[2] * ax[2])));
                th = std::min(M_PI, th + 0.01);
                int code = 0;
                for (int b = 0; b < 4; ++b) code |= (((i >> b) & 1) << (2 * b)) | (((j >> b) & 1) << (2 * b + 1));
                cones[2 * code] = make_float4((float)ax[0], (float)ax[1], (float)ax[2], (float)std::cos(th));
                cones[2 * code + 1] = make_float4((float)std::sin(th), 0.f, 0.f, 0.f);
            }
    });
    return cones;
}

}  // namespace

// Planar emitters: origin and in-plane axes (columns of m), and the rotation of
// alignRayDirection (RayFactorGPU.cl:87-97) for the fixed normal n = row 2 of invm,
// normalised (transformNormal of (0,0,1), :73-85), all in FP64.  d = 1/(1 + n.z),
// formed as (1 - n.z)/(n.x^2 + n.y^2) for a normal facing -z (the same value for
// a unit normal, without cancellation), and 0.5 where it is infinite (:91).
void rf::emit_frame(const rf_primitive &e, float4 *f)
{
    for (int k = 0; k < kEmitFrameWords; ++k) f[k] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (e.type != RF_DISC && e.type != RF_ANNULUS && e.type != RF_RECTANGLE) return;  // flag 0: per-ray normal
    double n[3] = {e.invm[8], e.invm[9], e.invm[10]};
    const double nn = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    if (!(nn > 0.0) || !std::isfinite(nn)) return;
    for (double &v : n) v /= nn;
    double d = n[2] < 0.0 ? (1.0 - n[2]) / (n[0] * n[0] + n[1] * n[1]) : 1.0 / (1.0 + n[2]);
    if (std::isinf(d)) d = 0.5;
    const double R[9] = {n[2] + d * n[1] * n[1], -d * n[0] * n[1], n[0],
                         -d * n[0] * n[1], n[2] + d * n[0] * n[0], n[1],
                         -n[0], -n[1], n[2]};
    f[0] = make_float4(e.m[3], e.m[7], e.m[11], 1.0f);
    f[1] = make_float4(e.m[0], e.m[4], e.m[8], (float)R[8]);
    f[2] = make_float4(e.m[1], e.m[5], e.m[9], 0.0f);
    f[3] = make_float4((float)R[0], (float)R[1], (float)R[2], (float)R[3]);
    f[4] = make_float4((float)R[4], (float)R[5], (float)R[6], (float)R[7]);
}

// Mixed-precision tables of one scene as the batched kernel reads them
// (re-centred transforms, hit records, bounding spheres with squared radius)
// and the scene's self-hit threshold (eps < 0: relative, as rf_trace forms it).
int rf::prepare_mixed_tables(const rf_primitive *prims, int n, float eps, rf_primitive *emit, HitRec *tab,
                             float4 *bs, float *eps_out)
{
    prepare_mixed(prims, n, emit, tab, bs);
    *eps_out = scene_eps(eps, bs, n);
    const int nstacks = mark_stacks(emit, n, tab, bs, std::vector<char>());
    for (int i = 0; i < n; ++i) bs[i] = widen_sq(bs[i]);
    return nstacks;
}

namespace {

// Upload the scenes of a batch (one scene for rf_set_scene in MIXED mode).
rf_status upload_batch(rf_ctx *c, const rf_scene_desc *scenes, int ns, bool with_budgets,
                       const std::vector<char> &cut0 = std::vector<char>())
{
    if (ns <= 0 || !scenes) return fail(c, RF_ERR_INVALID_ARG, "no scenes");
    int64_t nprim = 0, nhits = 0;
    for (int s = 0; s < ns; ++s) {
        rf_status st = validate_prims(c, scenes[s].prims, scenes[s].n_prims, s);
        if (st != RF_OK) return st;
        if (scenes[s].n_prims > kBatchMaxSurfaces)
            return fail(c, RF_ERR_OVERFLOW, "scene %d: %d surfaces; the mixed-precision kernel takes at most %d", s,
                        scenes[s].n_prims, kBatchMaxSurfaces);
        if (with_budgets && !scenes[s].rays_per_emitter)
            return fail(c, RF_ERR_INVALID_ARG, "scene %d: rays_per_emitter is NULL", s);
        nprim += scenes[s].n_prims;
        nhits += (int64_t)scenes[s].n_prims * scenes[s].n_prims;
    }
    if (nprim > (1ll << 31) / 4) return fail(c, RF_ERR_OVERFLOW, "too many surfaces in the batch");
    std::vector<rf_primitive> emit(nprim);
    std::vector<HitRec> tab(nprim);
    std::vector<float4> bs(nprim), patch((size_t)nprim * 16), chain((size_t)nprim * kChainMax), plane(nprim),
        frame((size_t)nprim * kEmitFrameWords);
    c->b_info.resize(ns);
    c->b_stacks = 0;
    int64_t off = 0, hoff = 0;
    for (int s = 0; s < ns; ++s) {
        const int n = scenes[s].n_prims;
        prepare_mixed(scenes[s].prims, n, emit.data() + off, tab.data() + off, bs.data() + off);
        c->b_info[s].eps = scene_eps(c->cfg.eps, bs.data() + off, n);
        c->b_info[s].pad = 0;
        for (int i = 0; i < n; ++i) {
            const int64_t g = off + i;
            patch_balls(emit[g], patch.data() + g * 16);
            surface_chain(emit[g], bs[g], chain.data() + g * kChainMax);  // the masks: per surface
            plane[g] = surface_plane(emit[g]);
            emit_frame(emit[g], frame.data() + g * kEmitFrameWords);
        }
        if (!c->cfg.split_stacks)
            c->b_stacks += mark_stacks(emit.data() + off, n, tab.data() + off, bs.data() + off,
                                       s == 0 ? cut0 : std::vector<char>());
        if (s == 0) {
            c->b_test_type.assign(n, 0);
            for (int i = 0; i < n; ++i) {
                int32_t ti, w;
                std::memcpy(&ti, &tab[off + i].aux.x, 4);
                std::memcpy(&w, &tab[off + i].aux.w, 4);
                const int own = ti == kStackType ? (int)RF_CYLINDER : (ti == kPlateType ? (int)RF_ANNULUS : ti);
                c->b_test_type[i] = (ti < kStackType || (w & 0xffff) == 0) ? own : -1;
            }
        }
        for (int i = 0; i < n; ++i) bs[off + i] = widen_sq(bs[off + i]);
        c->b_info[s].n = n;
        c->b_info[s].prim_off = (int32_t)off;
        c->b_info[s].hits_off = hoff;
        off += n;
        hoff += (int64_t)n * n;
    }
    // cell masks for every row of the scenes culling serves (more than
    // kBatchBruteMax and at most kMaskMaxSurfaces surfaces) while they fit
    // kMaskBudgetWords
    std::vector<MaskRow> mrows;
    std::vector<int64_t> moff(nprim, -1);
    int64_t mwords = 0;
    for (int s = 0; s < ns; ++s) {
        const SceneInfo &si = c->b_info[s];
        if (si.n <= kBatchBruteMax || si.n > kMaskMaxSurfaces) continue;
        const int64_t row_words = (int64_t)kMaskCells * ((si.n + 31) / 32);
        if (mwords + row_words * si.n > kMaskBudgetWords) continue;
        for (int e = 0; e < si.n; ++e) {
            MaskRow r;
            r.scene = s;
            r.emitter = e;
            r.off = mwords;
            mrows.push_back(r);
            moff[si.prim_off + e] = mwords;
            mwords += row_words;
        }
    }
    RF_CUDA(c, cudaSetDevice(c->device));
    RF_CUDA(c, cudaStreamSynchronize(c->stream));
    RF_CUDA(c, c->b_tab.ensure(sizeof(HitRec) * nprim));
    RF_CUDA(c, c->b_emit.ensure(sizeof(rf_primitive) * nprim));
    RF_CUDA(c, c->b_bsph.ensure(sizeof(float4) * nprim));
    RF_CUDA(c, c->b_scenes.ensure(sizeof(SceneInfo) * ns));
    RF_CUDA(c, c->b_frame.ensure(sizeof(float4) * frame.size()));
    RF_CUDA(c, cudaMemcpyAsync(c->b_frame.p, frame.data(), sizeof(float4) * frame.size(), cudaMemcpyHostToDevice,
                               c->stream));

    RF_CUDA(c, c->b_hits.ensure((size_t)nhits * 8));
    RF_CUDA(c, c->b_counters.ensure(256));
    RF_CUDA(c, cudaMemcpyAsync(c->b_tab.p, tab.data(), sizeof(HitRec) * nprim, cudaMemcpyHostToDevice, c->stream));
    RF_CUDA(c, cudaMemcpyAsync(c->b_emit.p, emit.data(), sizeof(rf_primitive) * nprim, cudaMemcpyHostToDevice, c->stream));
    RF_CUDA(c, cudaMemcpyAsync(c->b_bsph.p, bs.data(), sizeof(float4) * nprim, cudaMemcpyHostToDevice, c->stream));
    RF_CUDA(c, cudaMemcpyAsync(c->b_scenes.p, c->b_info.data(), sizeof(SceneInfo) * ns, cudaMemcpyHostToDevice, c->stream));

    c->b_masks = !mrows.empty();
    c->b_mask_ms = 0.0;
    if (c->b_masks) {
        const std::vector<float4> &cones = direction_cones();
        RF_CUDA(c, c->b_patch.ensure(sizeof(float4) * patch.size()));
        RF_CUDA(c, c->b_chain.ensure(sizeof(float4) * chain.size()));
        RF_CUDA(c, c->b_plane.ensure(sizeof(float4) * plane.size()));
        RF_CUDA(c, c->b_cone.ensure(sizeof(float4) * cones.size()));
        RF_CUDA(c, c->b_maskrows.ensure(sizeof(MaskRow) * mrows.size()));
        RF_CUDA(c, c->b_maskoff.ensure(sizeof(int64_t) * moff.size()));
        RF_CUDA(c, c->b_mask.ensure(sizeof(uint32_t) * (size_t)mwords));
        RF_CUDA(c, cudaMemcpyAsync(c->b_patch.p, patch.data(), sizeof(float4) * patch.size(), cudaMemcpyHostToDevice, c->stream));
        RF_CUDA(c, cudaMemcpyAsync(c->b_chain.p, chain.data(), sizeof(float4) * chain.size(), cudaMemcpyHostToDevice, c->stream));
        RF_CUDA(c, cudaMemcpyAsync(c->b_plane.p, plane.data(), sizeof(float4) * plane.size(), cudaMemcpyHostToDevice, c->stream));
        RF_CUDA(c, cudaMemcpyAsync(c->b_cone.p, cones.data(), sizeof(float4) * cones.size(), cudaMemcpyHostToDevice, c->stream));
        RF_CUDA(c, cudaMemcpyAsync(c->b_maskrows.p, mrows.data(), sizeof(MaskRow) * mrows.size(), cudaMemcpyHostToDevice, c->stream));
        RF_CUDA(c, cudaMemcpyAsync(c->b_maskoff.p, moff.data(), sizeof(int64_t) * moff.size(), cudaMemcpyHostToDevice, c->stream));
        MaskInputs in{};
        in.rows = c->b_maskrows.as<MaskRow>();
        in.nrows = (int32_t)mrows.size();
        in.total_words = mwords;
        in.scenes = c->b_scenes.as<SceneInfo>();
        in.patch = c->b_patch.as<float4>();
        in.cone = c->b_cone.as<float4>();
        in.chain = c->b_chain.as<float4>();
        in.plane = c->b_plane.as<float4>();
        RF_CUDA(c, cudaEventRecord(c->ev0, c->stream));
        RF_CUDA(c, launch_build_masks(in, c->b_mask.as<uint32_t>(), c->stream));
        RF_CUDA(c, cudaEventRecord(c->ev1, c->stream));
        RF_CUDA(c, cudaStreamSynchronize(c->stream));
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, c->ev0, c->ev1) == cudaSuccess) c->b_mask_ms = ms;
    }

    RF_CUDA(c, cudaStreamSynchronize(c->stream));
    c->b_hits_total = nhits;
    return RF_OK;
}

// Counters of the batched kernel inside b_counters.
struct BatchCounters {
    unsigned long long queue;
    unsigned long long refined;
    int64_t total;
    int32_t nseg;
    int32_t flags[2];  // not-converged rows, rounds
    int32_t pad;
    unsigned long long work[8];
};

TraceParams batch_params(rf_ctx *c)
{
    TraceParams p{};
    BatchCounters *bc = c->b_counters.as<BatchCounters>();
    p.tab = c->b_tab.as<HitRec>();
    p.emit = c->b_emit.as<rf_primitive>();
    p.bsph = c->b_bsph.as<float4>();
    p.frame = c->b_frame.as<float4>();
    p.scenes = c->b_scenes.as<SceneInfo>();

    p.hits = c->b_hits.as<unsigned long long>();
    p.queue = &bc->queue;
    p.refined = &bc->refined;
    p.work = bc->work;
    p.err = c->d_err.as<int32_t>();
    p.compat = c->cfg.compat;
    p.key1 = c->cfg.key1;
    p.scene_id = c->cfg.scene_id;
    p.eps = c->cfg.eps;  // per scene: SceneInfo::eps
    if (c->b_masks) {
        p.cmask = c->b_mask.as<uint32_t>();
        p.mask_off = c->b_maskoff.as<int64_t>();
    }
    return p;
}

bool batch_resident(const rf_ctx *c)
{
    for (const SceneInfo &si : c->b_info)
        if (si.n > batched_tile()) return false;
    return true;
}

int batched_grid(rf_ctx *c, bool rec)
{
    int bps = batched_blocks_per_sm(rec, batch_resident(c));
    if (bps <= 0) bps = 1;
    const int wave = c->sms * bps;
    return c->cfg.batched_grid > 0 ? std::min(wave, (int)c->cfg.batched_grid) : wave;
}

// One persistent launch over host-planned segments.
rf_status run_batched(rf_ctx *c, const std::vector<Segment> &seg, int64_t total_chunks, bool rec,
                      int32_t *d_rec, int64_t rec_base, bool zero_hits, bool bv = false)
{
    c->last_small = false;
    c->last_launches = 0;
    c->timed = false;
    if (zero_hits) RF_CUDA(c, cudaMemsetAsync(c->b_hits.p, 0, (size_t)c->b_hits_total * 8, c->stream));
    RF_CUDA(c, cudaMemsetAsync(c->b_counters.p, 0, sizeof(BatchCounters), c->stream));
    if (seg.empty() || total_chunks == 0) return RF_OK;
    if (rf_status st = upload_segments(c, seg); st != RF_OK) return st;
    TraceParams p = batch_params(c);
    p.seg = c->d_seg.as<Segment>();
    p.nseg = (int32_t)seg.size();
    p.total_chunks = total_chunks;
    p.rec = d_rec;
    p.rec_base = rec_base;
    const int grid = (int)std::min<int64_t>(batched_grid(c, rec), total_chunks);
    RF_CUDA(c, cudaEventRecord(c->ev0, c->stream));
    if (bv) {
        p.bvtab = c->b_bvtab.as<HitRec>();
        p.bvinfo = c->b_bvinfo.as<int4>();
        p.bvsph = c->b_bvsph.as<float4>();
        p.nbv = c->nbv;
        RF_CUDA(c, launch_batched_bv(p, rec, c->cfg.work_counts != 0, c->b_stacks > 0, grid, c->stream));
    } else {
        RF_CUDA(c, launch_batched(p, rec, batch_resident(c), c->cfg.work_counts != 0, c->b_stacks > 0, grid,
                                  c->stream));
    }
    RF_CUDA(c, cudaEventRecord(c->ev1, c->stream));
    c->last_launches = 1;
    c->timed = true;
    return RF_OK;
}

// Single scenes of at most this many surfaces take the small-scene kernel
// unless rf_autotune measured otherwise.
constexpr int kSmallDefaultMax = 16;

bool use_small(const rf_ctx *c)
{
    if (!c->b_single || c->n > kSmallMax) return false;
    if (c->mixed_path != 0) return c->mixed_path == 1;
    return c->n <= kSmallDefaultMax;
}

int small_gpt(const rf_ctx *c, bool rec)
{
    if (rec) return 1;
    if (c->gpt > 0) return c->gpt == 2 ? 2 : 1;
    return c->cfg.rays_per_thread == 8 ? 2 : 1;
}

int64_t mixed_chunk_draws(const rf_ctx *c, bool rec, bool bv)
{
    return !bv && use_small(c) ? (int64_t)kSmallThreads * small_gpt(c, rec) : (int64_t)kBatchChunkDraws;
}

// One launch of the small-scene kernel over host-planned segments (chunks of
// kSmallThreads * gpt draws) of the scene held in the batch tables.
rf_status run_small(rf_ctx *c, const std::vector<Segment> &seg, int64_t total_chunks, bool rec, int32_t *d_rec,
                    int64_t rec_base, bool zero_hits)
{
    c->last_launches = 0;
    c->timed = false;
    c->last_small = true;
    std::fill(std::begin(c->small_work), std::end(c->small_work), 0ull);
    if (zero_hits) RF_CUDA(c, cudaMemsetAsync(c->b_hits.p, 0, (size_t)c->b_hits_total * 8, c->stream));
    RF_CUDA(c, cudaMemsetAsync(c->b_counters.p, 0, sizeof(BatchCounters), c->stream));
    if (seg.empty() || total_chunks == 0) return RF_OK;
    if (c->cfg.work_counts) {  // every ray against every surface but a planar emitter itself, a stack once
        for (const Segment &sg : seg) {
            const int64_t rays = sg.ray_end - sg.ray_begin;
            const int et = c->prims[sg.emitter].type;
            const bool planar = et == RF_DISC || et == RF_ANNULUS || et == RF_RECTANGLE;
            for (int j = 0; j < (int)c->b_test_type.size(); ++j) {
                if ((planar && j == sg.emitter) || c->b_test_type[j] < 0) continue;
                c->small_work[c->b_test_type[j]] += (unsigned long long)rays;
            }
        }
    }
    if (rf_status st = upload_segments(c, seg); st != RF_OK) return st;
    TraceParams p = batch_params(c);
    p.cmask = nullptr;
    p.mask_off = nullptr;
    p.n = c->b_info[0].n;
    p.eps = c->b_info[0].eps;
    p.seg = c->d_seg.as<Segment>();
    p.nseg = (int32_t)seg.size();
    p.total_chunks = total_chunks;
    p.rec = d_rec;
    p.rec_base = rec_base;
    const int gpt = small_gpt(c, rec);
    int bps = mixed_small_blocks_per_sm(gpt, rec);
    if (bps <= 0) bps = 1;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)c->sms * bps, total_chunks));
    RF_CUDA(c, cudaEventRecord(c->ev0, c->stream));
    RF_CUDA(c, launch_mixed_small(p, gpt, rec, grid, c->stream));
    RF_CUDA(c, cudaEventRecord(c->ev1, c->stream));
    c->last_launches = 1;
    c->timed = true;
    return RF_OK;
}

// A MIXED trace of the single scene: small-scene or batched kernel; with its
// bounding surfaces (runBVGPU semantics), the batched kernel's BV variant.
rf_status run_mixed(rf_ctx *c, const std::vector<Segment> &seg, int64_t total_chunks, bool rec, int32_t *d_rec,
                    int64_t rec_base, bool zero_hits, bool bv)
{
    if (bv) return run_batched(c, seg, total_chunks, rec, d_rec, rec_base, zero_hits, true);
    if (use_small(c)) return run_small(c, seg, total_chunks, rec, d_rec, rec_base, zero_hits);
    return run_batched(c, seg, total_chunks, rec, d_rec, rec_base, zero_hits);
}

// Can the mixed kernel trace this scene with its bounding surfaces?
rf_status check_mixed_bv(rf_ctx *c)
{
    if (c->nbv > kBatchMaxBV)
        return fail(c, RF_ERR_UNSUPPORTED, "the mixed-precision kernel takes at most %d bounding surfaces (scene: %d)",
                    kBatchMaxBV, c->nbv);
    if (c->n > batched_tile())
        return fail(c, RF_ERR_UNSUPPORTED, "bounding surfaces with the mixed-precision kernel: at most %d surfaces",
                    batched_tile());
    return RF_OK;
}

rf_status require_scene(rf_ctx *c)
{
    if (!c) return RF_ERR_INVALID_ARG;
    if (c->n <= 0) return fail(c, RF_ERR_STATE, "no scene: call rf_set_scene first");
    return RF_OK;
}

}  // namespace

extern "C" {

void rf_config_default(rf_config *cfg)
{
    if (!cfg) return;
    std::memset(cfg, 0, sizeof *cfg);
    cfg->struct_size = sizeof(rf_config);
    cfg->compat = 0;
    cfg->precision = RF_PREC_EXACT;
    cfg->key1 = 0xdecafbadu;  // RayFactorGPU.cl:486
    cfg->eps = 1e-3f;         // RayFactorGPU.cl:7
    cfg->device = 0;
}

int32_t rf_abi_version(void) { return RF_ABI_VERSION; }

const char *rf_status_string(rf_status s)
{
    switch (s) {
    case RF_OK: return "ok";
    case RF_ERR_INVALID_ARG: return "invalid argument";
    case RF_ERR_BAD_SCENE: return "bad scene";
    case RF_ERR_OOM: return "out of memory";
    case RF_ERR_CUDA: return "CUDA error";
    case RF_ERR_TIMEOUT: return "device wait timed out";
    case RF_ERR_OVERFLOW: return "size overflow";
    case RF_ERR_NO_DEVICE: return "no CUDA device";
    case RF_ERR_UNSUPPORTED: return "unsupported";
    case RF_ERR_STATE: return "wrong call order";
    }
    return "unknown status";
}

rf_status rf_create(rf_ctx **out, const rf_config *cfg)
{
    if (!out) return RF_ERR_INVALID_ARG;
    *out = nullptr;
    rf_config c;
    rf_config_default(&c);
    if (cfg) {
        if (cfg->struct_size != sizeof(rf_config)) return RF_ERR_INVALID_ARG;
        c = *cfg;
    }
    if (c.precision > RF_PREC_FP64) return RF_ERR_INVALID_ARG;
    if (!std::isfinite(c.eps)) return RF_ERR_INVALID_ARG;
    if (c.rays_per_thread != 0 && c.rays_per_thread != 4 && c.rays_per_thread != 8)
        return RF_ERR_INVALID_ARG;
    if (c.block_size < 0 || c.block_size > kBlock || (c.block_size % 32) != 0) return RF_ERR_INVALID_ARG;
    if (c.tally_mode < 0 || c.tally_mode > 2 || c.table_mode < 0 || c.table_mode > 2) return RF_ERR_INVALID_ARG;
    if (c.work_counts < 0 || c.work_counts > 1 || c.batched_grid < 0 || c.split_stacks < 0 || c.split_stacks > 1)
        return RF_ERR_INVALID_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) {
        cudaGetLastError();
        return RF_ERR_NO_DEVICE;
    }
    if (c.device < 0 || c.device >= ndev) return RF_ERR_NO_DEVICE;
    rf_ctx *ctx = new (std::nothrow) rf_ctx;
    if (!ctx) return RF_ERR_OOM;
    ctx->cfg = c;
    ctx->device = c.device;
    if (c.tally_mode) ctx->hist = c.tally_mode == 1 ? 1 : 0;
    if (c.table_mode) ctx->stage = c.table_mode == 1 ? 1 : 0;
    if (c.test_order) ctx->order = c.test_order == 2 ? 1 : 0;
    if (cudaSetDevice(c.device) != cudaSuccess ||
        cudaDeviceGetAttribute(&ctx->sms, cudaDevAttrMultiProcessorCount, c.device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&ctx->ev0) != cudaSuccess || cudaEventCreate(&ctx->ev1) != cudaSuccess ||
        ctx->d_err.ensure(64) != cudaSuccess ||
        cudaMemset(ctx->d_err.p, 0, 64) != cudaSuccess) {
        cudaGetLastError();
        rf_destroy(ctx);
        return RF_ERR_CUDA;
    }
    *out = ctx;
    return RF_OK;
}

void rf_destroy(rf_ctx *c)
{
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (DevBuf *b : {&c->d_tab, &c->d_emit, &c->d_bvtab, &c->d_bvinfo, &c->d_hits, &c->d_seg,
                      &c->d_rays, &c->d_F, &c->d_rec, &c->d_err, &c->d_misc, &c->b_tab, &c->b_emit,
                      &c->b_bsph, &c->b_scenes, &c->b_hits, &c->b_rows, &c->b_counters, &c->b_patch,
                      &c->b_chain, &c->b_plane, &c->b_cone, &c->b_maskrows, &c->b_maskoff, &c->b_mask, &c->b_frame, &c->b_bvtab,
                      &c->b_bvinfo, &c->b_bvsph})
        b->release();
    c->h_seg.release();
    c->h_rays.release();
    c->h_misc.release();
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

const char *rf_last_error(const rf_ctx *c)
{
    if (!c) return "null context";
    return c->err.c_str();
}

rf_status rf_set_scene(rf_ctx *c, const rf_primitive *prims, int32_t n, const rf_bounding_volume *bvs,
                       int32_t nbv)
{
    ApiRange nvtx_range("rf_set_scene");
    if (!c) return RF_ERR_INVALID_ARG;
    rf_status st = validate_prims(c, prims, n, 0);
    if (st != RF_OK) return st;
    if (nbv < 0 || (nbv > 0 && !bvs)) return fail(c, RF_ERR_INVALID_ARG, "bad bounding-volume arguments");
    std::vector<HitRec> tab(n);
    for (int i = 0; i < n; ++i) tab[i] = make_hitrec(prims[i].invm, prims[i].type, prims[i].util1, prims[i].util2);
    std::vector<HitRec> bvtab(std::max(nbv, 1));
    std::vector<int4> bvinfo(std::max(nbv, 1));
    for (int b = 0; b < nbv; ++b) {
        const rf_bounding_volume &v = bvs[b];
        if (v.type < 0 || v.type > RF_DISC)
            return fail(c, RF_ERR_BAD_SCENE, "bounding volume %d: type %d is not a surface", b, v.type);
        if (!finite_all(v.invm, 12))
            return fail(c, RF_ERR_BAD_SCENE, "bounding volume %d: non-finite transform", b);
        if ((uses_util1(v.type) && !std::isfinite(v.util1)))
            return fail(c, RF_ERR_BAD_SCENE, "bounding volume %d: non-finite util1", b);
        if (v.objStartIndex < 0 || v.objEndIndex < v.objStartIndex || v.objEndIndex > n)
            return fail(c, RF_ERR_BAD_SCENE, "bounding volume %d: children [%d,%d) outside [0,%d)", b,
                        v.objStartIndex, v.objEndIndex, n);
        bvtab[b] = make_hitrec(v.invm, v.type, v.util1, v.util2);
        bvinfo[b] = make_int4(v.settings, v.objStartIndex, v.objEndIndex, 0);
    }
    RF_CUDA(c, cudaSetDevice(c->device));
    RF_CUDA(c, cudaStreamSynchronize(c->stream));
    RF_CUDA(c, c->d_tab.ensure(sizeof(HitRec) * n));
    RF_CUDA(c, c->d_emit.ensure(sizeof(rf_primitive) * n));
    RF_CUDA(c, c->d_bvtab.ensure(sizeof(HitRec) * bvtab.size()));
    RF_CUDA(c, c->d_bvinfo.ensure(sizeof(int4) * bvinfo.size()));
    RF_CUDA(c, c->d_hits.ensure((size_t)n * n * 8));
    RF_CUDA(c, cudaMemcpyAsync(c->d_tab.p, tab.data(), sizeof(HitRec) * n, cudaMemcpyHostToDevice, c->stream));
    RF_CUDA(c, cudaMemcpyAsync(c->d_emit.p, prims, sizeof(rf_primitive) * n, cudaMemcpyHostToDevice, c->stream));
    RF_CUDA(c, cudaMemcpyAsync(c->d_bvtab.p, bvtab.data(), sizeof(HitRec) * bvtab.size(),
                               cudaMemcpyHostToDevice, c->stream));
    RF_CUDA(c, cudaMemcpyAsync(c->d_bvinfo.p, bvinfo.data(), sizeof(int4) * bvinfo.size(),
                               cudaMemcpyHostToDevice, c->stream));
    RF_CUDA(c, cudaStreamSynchronize(c->stream));
    c->prims.assign(prims, prims + n);
    c->n = n;
    c->nbv = nbv;
    c->have_results = false;
    c->b_single = false;
    c->eps = c->cfg.eps;
    if (c->cfg.eps < 0.0f) {  // scale-relative: from the scene's bounding spheres
        std::vector<rf_primitive> e(n);
        std::vector<HitRec> t(n);
        std::vector<float4> b(n);
        prepare_mixed(prims, n, e.data(), t.data(), b.data());
        c->eps = scene_eps(c->cfg.eps, b.data(), n);
    }
    if (c->cfg.precision == RF_PREC_MIXED) {
        rf_scene_desc d{prims, n, 0, nullptr};
        std::vector<char> cut(n + 1, 0);  // segment stacks stay inside bounding-surface child ranges
        for (int b = 0; b < nbv; ++b) {
            if (bvs[b].objStartIndex >= 0 && bvs[b].objStartIndex <= n) cut[bvs[b].objStartIndex] = 1;
            if (bvs[b].objEndIndex >= 0 && bvs[b].objEndIndex <= n) cut[bvs[b].objEndIndex] = 1;
        }
        if ((st = upload_batch(c, &d, 1, false, cut)) != RF_OK) return st;
        c->b_single = true;
        if (nbv > 0) {  // bounding surfaces in the surfaces' re-centred frame (prepare_mixed's anchor)
            double a[3] = {0, 0, 0};
            for (int i = 0; i < n; ++i)
                for (int k = 0; k < 3; ++k) a[k] += prims[i].m[4 * k + 3];
            for (int k = 0; k < 3; ++k) a[k] /= n;
            std::vector<HitRec> rb(nbv);
            std::vector<float4> bsv(nbv);
            for (int b = 0; b < nbv; ++b) {
                float im[12];
                std::memcpy(im, bvs[b].invm, sizeof im);
                for (int k = 0; k < 3; ++k) {
                    const float *r = bvs[b].invm + 4 * k;
                    im[4 * k + 3] = (float)((double)r[3] + (double)r[0] * a[0] + (double)r[1] * a[1] + (double)r[2] * a[2]);
                }
                rb[b] = make_hitrec(im, bvs[b].type, bvs[b].util1, bvs[b].util2);
                // its bounding sphere: m = the inverse of the re-centred invm (FP64)
                rf_primitive e{};
                e.type = bvs[b].type;
                e.util1 = bvs[b].util1;
                e.util2 = bvs[b].util2;
                const double A[9] = {im[0], im[1], im[2], im[4], im[5], im[6], im[8], im[9], im[10]};
                const double det = A[0] * (A[4] * A[8] - A[5] * A[7]) - A[1] * (A[3] * A[8] - A[5] * A[6]) +
                                   A[2] * (A[3] * A[7] - A[4] * A[6]);
                const double inv[9] = {(A[4] * A[8] - A[5] * A[7]) / det, (A[2] * A[7] - A[1] * A[8]) / det,
                                       (A[1] * A[5] - A[2] * A[4]) / det, (A[5] * A[6] - A[3] * A[8]) / det,
                                       (A[0] * A[8] - A[2] * A[6]) / det, (A[2] * A[3] - A[0] * A[5]) / det,
                                       (A[3] * A[7] - A[4] * A[6]) / det, (A[1] * A[6] - A[0] * A[7]) / det,
                                       (A[0] * A[4] - A[1] * A[3]) / det};
                for (int r = 0; r < 3; ++r) {
                    for (int k = 0; k < 3; ++k) e.m[4 * r + k] = (float)inv[3 * r + k];
                    e.m[4 * r + 3] = (float)-(inv[3 * r] * im[3] + inv[3 * r + 1] * im[7] + inv[3 * r + 2] * im[11]);
                }
                bsv[b] = std::isfinite(det) && det != 0.0 ? widen_sq(surface_sphere(e))
                                                         : make_float4(0.f, 0.f, 0.f, std::numeric_limits<float>::infinity());
            }
            RF_CUDA(c, c->b_bvtab.ensure(sizeof(HitRec) * nbv));
            RF_CUDA(c, c->b_bvinfo.ensure(sizeof(int4) * nbv));
            RF_CUDA(c, c->b_bvsph.ensure(sizeof(float4) * nbv));
            RF_CUDA(c, cudaMemcpyAsync(c->b_bvsph.p, bsv.data(), sizeof(float4) * nbv, cudaMemcpyHostToDevice,
                                       c->stream));
            RF_CUDA(c, cudaMemcpyAsync(c->b_bvtab.p, rb.data(), sizeof(HitRec) * nbv, cudaMemcpyHostToDevice, c->stream));
            RF_CUDA(c, cudaMemcpyAsync(c->b_bvinfo.p, bvinfo.data(), sizeof(int4) * nbv, cudaMemcpyHostToDevice,
                                       c->stream));
            RF_CUDA(c, cudaStreamSynchronize(c->stream));
        }
    }
    return RF_OK;
}

rf_status rf_trace_async(rf_ctx *c, const int64_t *rays, int32_t use_bv)
{
    ApiRange nvtx_range("rf_trace_async");
    rf_status s = require_scene(c);
    if (s != RF_OK) return s;
    if (!rays) return fail(c, RF_ERR_INVALID_ARG, "rays_per_emitter is NULL");
    if (use_bv && c->nbv <= 0) return fail(c, RF_ERR_STATE, "use_bv set but the scene has no bounding volumes");
    if ((s = check_budgets(c, rays, c->n)) != RF_OK) return s;
    RF_CUDA(c, cudaSetDevice(c->device));
    c->last_rays.assign(rays, rays + c->n);
    c->have_results = false;
    if (c->cfg.precision == RF_PREC_MIXED) {
        if (use_bv && (s = check_mixed_bv(c)) != RF_OK) return s;
        if (!c->b_single) return fail(c, RF_ERR_STATE, "scene not prepared for the mixed kernel");
        std::vector<Segment> seg;
        int64_t chunks = 0;
        const int64_t cg = mixed_chunk_draws(c, false, use_bv != 0);
        for (int e = 0; e < c->n; ++e) chunks = plan_segments(seg, e, 0, 0, rays[e], cg, chunks);
        if ((s = run_mixed(c, seg, chunks, false, nullptr, 0, true, use_bv != 0)) != RF_OK) return s;
        c->have_results = true;
        return RF_OK;
    }
    Plan pl = make_plan(c, use_bv != 0, false);
    const int64_t chunk_gids = (int64_t)pl.lc.block * pl.lc.gpt;
    std::vector<Segment> seg;
    int64_t chunks = 0;
    for (int e = 0; e < c->n; ++e) chunks = plan_segments(seg, e, 0, 0, rays[e], chunk_gids, chunks);
    if ((s = run_trace(c, seg, chunks, pl, nullptr, 0, true)) != RF_OK) return s;
    c->have_results = true;
    return RF_OK;
}

rf_status rf_trace_range(rf_ctx *c, const int64_t *first_ray, const int64_t *count, int32_t use_bv,
                         int32_t accumulate)
{
    ApiRange nvtx_range("rf_trace_range");
    rf_status s = require_scene(c);
    if (s != RF_OK) return s;
    if (!first_ray || !count) return fail(c, RF_ERR_INVALID_ARG, "first_ray / count is NULL");
    if (use_bv && c->nbv <= 0) return fail(c, RF_ERR_STATE, "use_bv set but the scene has no bounding volumes");
    if (use_bv && c->cfg.precision == RF_PREC_MIXED && (s = check_mixed_bv(c)) != RF_OK) return s;
    if (accumulate && (int)c->last_rays.size() != c->n)
        return fail(c, RF_ERR_STATE, "nothing to accumulate into: trace or rf_set_tallies first");
    std::vector<int64_t> ends(c->n);
    for (int e = 0; e < c->n; ++e) {
        if (first_ray[e] < 0 || count[e] < 0) return fail(c, RF_ERR_INVALID_ARG, "negative ray range (emitter %d)", e);
        if (first_ray[e] > kMaxRaysPerEmitter || count[e] > kMaxRaysPerEmitter)
            return fail(c, RF_ERR_OVERFLOW, "ray range of emitter %d beyond 2^46", e);
        ends[e] = first_ray[e] + count[e];
    }
    if ((s = check_budgets(c, ends.data(), c->n)) != RF_OK) return s;
    RF_CUDA(c, cudaSetDevice(c->device));
    std::vector<Segment> seg;
    int64_t chunks = 0;
    const bool mixed = c->cfg.precision == RF_PREC_MIXED;
    Plan pl = make_plan(c, use_bv != 0, false);
    const int64_t chunk_gids = mixed ? mixed_chunk_draws(c, false, use_bv != 0) : (int64_t)pl.lc.block * pl.lc.gpt;
    for (int e = 0; e < c->n; ++e) chunks = plan_segments(seg, e, 0, first_ray[e], count[e], chunk_gids, chunks);
    if (!accumulate) c->last_rays.assign(c->n, 0);
    for (int e = 0; e < c->n; ++e) c->last_rays[e] += count[e];
    c->have_results = false;
    if (mixed) {
        if (!c->b_single) return fail(c, RF_ERR_STATE, "scene not prepared for the mixed kernel");
        s = run_mixed(c, seg, chunks, false, nullptr, 0, !accumulate, use_bv != 0);
    } else {
        s = run_trace(c, seg, chunks, pl, nullptr, 0, !accumulate);
    }
    if (s != RF_OK) return s;
    c->have_results = true;
    return RF_OK;
}

rf_status rf_set_tallies(rf_ctx *c, const uint64_t *hits, const int64_t *rays)
{
    rf_status s = require_scene(c);
    if (s != RF_OK) return s;
    if (!hits || !rays) return fail(c, RF_ERR_INVALID_ARG, "hits / rays is NULL");
    for (int e = 0; e < c->n; ++e)
        if (rays[e] < 0) return fail(c, RF_ERR_INVALID_ARG, "negative ray count (emitter %d)", e);
    RF_CUDA(c, cudaSetDevice(c->device));
    const size_t nn = (size_t)c->n * c->n;
    DevBuf &dst = c->cfg.precision == RF_PREC_MIXED ? c->b_hits : c->d_hits;
    RF_CUDA(c, cudaStreamSynchronize(c->stream));
    RF_CUDA(c, cudaMemcpyAsync(dst.p, hits, nn * 8, cudaMemcpyHostToDevice, c->stream));
    RF_CUDA(c, cudaStreamSynchronize(c->stream));
    c->last_rays.assign(rays, rays + c->n);
    c->have_results = true;
    return RF_OK;
}

rf_status rf_read_results(rf_ctx *c, uint64_t *hits_out, double *F_out)
{
    ApiRange nvtx_range("rf_read_results");
    rf_status s = require_scene(c);
    if (s != RF_OK) return s;
    if (!c->have_results) return fail(c, RF_ERR_STATE, "no trace to read");
    RF_CUDA(c, cudaSetDevice(c->device));
    const int n = c->n;
    const size_t nn = (size_t)n * n;
    const unsigned long long *hits_dev = c->cfg.precision == RF_PREC_MIXED ? c->b_hits.as<unsigned long long>()
                                                                           : c->d_hits.as<unsigned long long>();
    if (F_out) {
        RF_CUDA(c, c->d_rays.ensure(n * sizeof(int64_t)));
        RF_CUDA(c, c->d_F.ensure(nn * sizeof(double)));
        RF_CUDA(c, c->h_rays.ensure(n * sizeof(int64_t)));
        RF_CUDA(c, cudaStreamSynchronize(c->stream));
        std::memcpy(c->h_rays.p, c->last_rays.data(), n * sizeof(int64_t));
        RF_CUDA(c, cudaMemcpyAsync(c->d_rays.p, c->h_rays.p, n * sizeof(int64_t), cudaMemcpyHostToDevice,
                                   c->stream));
        RF_CUDA(c, launch_normalise_single(hits_dev, c->d_rays.as<int64_t>(), n, c->d_F.as<double>(),
                                           c->stream));
        RF_CUDA(c, cudaMemcpyAsync(F_out, c->d_F.p, nn * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    }
    if (hits_out) RF_CUDA(c, cudaMemcpyAsync(hits_out, hits_dev, nn * 8, cudaMemcpyDeviceToHost, c->stream));
    if (c->cfg.precision == RF_PREC_MIXED)
    {
        RF_CUDA(c, cudaMemcpyAsync(&c->last_refined, &c->b_counters.as<BatchCounters>()->refined,
                                   sizeof(unsigned long long), cudaMemcpyDeviceToHost, c->stream));
        RF_CUDA(c, cudaMemcpyAsync(c->last_work, c->b_counters.as<BatchCounters>()->work,
                                   sizeof c->last_work, cudaMemcpyDeviceToHost, c->stream));
    }
    RF_CUDA(c, cudaStreamSynchronize(c->stream));
    if (c->cfg.precision == RF_PREC_MIXED && c->last_small)
        std::copy(std::begin(c->small_work), std::end(c->small_work), std::begin(c->last_work));
    int32_t err = 0;
    RF_CUDA(c, cudaMemcpy(&err, c->d_err.p, 4, cudaMemcpyDeviceToHost));
    if (err) return fail(c, RF_ERR_TIMEOUT, "device reported error %d", err);
    return RF_OK;
}

rf_status rf_trace(rf_ctx *c, const int64_t *rays, int32_t use_bv, uint64_t *hits_out, double *F_out)
{
    ApiRange nvtx_range("rf_trace");
    rf_status s = rf_trace_async(c, rays, use_bv);
    if (s != RF_OK) return s;
    return rf_read_results(c, hits_out, F_out);
}

void *rf_stream(rf_ctx *c) { return c ? static_cast<void *>(c->stream) : nullptr; }

rf_status rf_last_trace_stats(rf_ctx *c, double *kernel_ms, int32_t *launches)
{
    if (!c) return RF_ERR_INVALID_ARG;
    if (launches) *launches = c->last_launches;
    if (kernel_ms) {
        *kernel_ms = 0.0;
        if (c->timed) {
            RF_CUDA(c, cudaEventSynchronize(c->ev1));
            float ms = 0.f;
            RF_CUDA(c, cudaEventElapsedTime(&ms, c->ev0, c->ev1));
            *kernel_ms = ms;
        }
    }
    return RF_OK;
}

rf_status rf_trace_rays(rf_ctx *c, int32_t emitter, int64_t first_ray, int64_t n_rays, int32_t use_bv,
                        int32_t *out)
{
    rf_status s = require_scene(c);
    if (s != RF_OK) return s;
    if (emitter < 0 || emitter >= c->n) return fail(c, RF_ERR_INVALID_ARG, "emitter %d out of range", emitter);
    if (first_ray < 0 || n_rays < 0 || !out) return fail(c, RF_ERR_INVALID_ARG, "bad ray range");
    if (n_rays > (1ll << 31)) return fail(c, RF_ERR_OVERFLOW, "at most 2^31 rays per call");
    if (first_ray + n_rays > kMaxRaysPerEmitter) return fail(c, RF_ERR_OVERFLOW, "ray index beyond 2^46");
    if ((c->cfg.compat & RF_COMPAT_STREAMS) && first_ray + n_rays > (4ll << 32))
        return fail(c, RF_ERR_OVERFLOW, "ray index beyond the reference stream key");
    if (use_bv && c->nbv <= 0) return fail(c, RF_ERR_STATE, "use_bv set but the scene has no bounding volumes");
    if (n_rays == 0) return RF_OK;
    RF_CUDA(c, cudaSetDevice(c->device));
    RF_CUDA(c, c->d_rec.ensure((size_t)n_rays * 4));
    if (c->cfg.precision == RF_PREC_MIXED) {
        if (use_bv && (s = check_mixed_bv(c)) != RF_OK) return s;
        std::vector<Segment> seg;
        const int64_t chunks =
            plan_segments(seg, emitter, 0, first_ray, n_rays, mixed_chunk_draws(c, true, use_bv != 0), 0);
        if ((s = run_mixed(c, seg, chunks, true, c->d_rec.as<int32_t>(), first_ray, false, use_bv != 0)) != RF_OK)
            return s;
    } else {
        Plan pl = make_plan(c, use_bv != 0, true);
        const int64_t chunk_gids = (int64_t)pl.lc.block * pl.lc.gpt;
        std::vector<Segment> seg;
        const int64_t chunks = plan_segments(seg, emitter, 0, first_ray, n_rays, chunk_gids, 0);
        if ((s = run_trace(c, seg, chunks, pl, c->d_rec.as<int32_t>(), first_ray, false)) != RF_OK) return s;
    }
    RF_CUDA(c, cudaMemcpyAsync(out, c->d_rec.p, (size_t)n_rays * 4, cudaMemcpyDeviceToHost, c->stream));
    RF_CUDA(c, cudaStreamSynchronize(c->stream));
    c->have_results = false;  // the tallies were not produced by this call
    return RF_OK;
}

rf_status rf_ray_budgets(const rf_primitive *prims, int32_t n, int32_t n_samples, uint32_t compat,
                         int64_t *rays_out)
{
    if (!prims || n <= 0 || !rays_out || n_samples < 0) return RF_ERR_INVALID_ARG;
    const int64_t wg = 128;  // WG_SIZE, RayFactorCL/util_opencl.h:52
    for (int e = 0; e < n; ++e) {
        // main.cpp:172 indexes the table with the device number (0 for one device)
        const int64_t rd = (compat & RF_COMPAT_BUDGET) ? prims[0].rayDensity : prims[e].rayDensity;
        const int64_t prod = rd * (int64_t)n_samples;
        if (prod > INT32_MAX || prod < INT32_MIN) return RF_ERR_OVERFLOW;  // int overflow in the reference
        const int64_t nt = (int64_t)((int32_t)prod / 4);
        if (nt < 0) return RF_ERR_OVERFLOW;
        const int64_t rem = nt % wg;
        const int64_t nthreads = rem > wg / 2 ? nt + wg - rem : nt - rem;  // main.cpp:173
        rays_out[e] = nthreads * 4;                                       // main.cpp:178
    }
    return RF_OK;
}

rf_status rf_run_gpurng(rf_ctx *c, int32_t n_samples, int32_t use_bv, int64_t *rays_out,
                        uint64_t *hits_out, double *F_out)
{
    rf_status s = require_scene(c);
    if (s != RF_OK) return s;
    std::vector<int64_t> rays(c->n);
    if ((s = rf_ray_budgets(c->prims.data(), c->n, n_samples, c->cfg.compat, rays.data())) != RF_OK)
        return fail(c, s, "ray budget rayDensity*n_samples overflows int32 (main.cpp:172)");
    if (rays_out) std::copy(rays.begin(), rays.end(), rays_out);
    return rf_trace(c, rays.data(), use_bv, hits_out, F_out);
}

namespace {

// |a x b| of two 3-vectors
double cross_norm(const double a[3], const double b[3])
{
    const double x = a[1] * b[2] - a[2] * b[1], y = a[2] * b[0] - a[0] * b[2], z = a[0] * b[1] - a[1] * b[0];
    return std::sqrt(x * x + y * y + z * z);
}

// M v for the linear part of a row-major 3x4 transform
void lin(const float *m, const double v[3], double out[3])
{
    for (int k = 0; k < 3; ++k) out[k] = m[4 * k] * v[0] + m[4 * k + 1] * v[1] + m[4 * k + 2] * v[2];
}

// Area of a surface of revolution patch p(theta, z) = M (rho(z) cos, rho(z) sin, z)
// (rho = 1 + (top-1) z, or the unit sphere when sphere is set): the periodic
// direction by the trapezoid rule, the other by composite Gauss-Legendre.
double revolution_area(const float *m, double top, bool sphere)
{
    static const double gx[4] = {-0.8611363115940526, -0.3399810435848563, 0.3399810435848563, 0.8611363115940526};
    static const double gw[4] = {0.3478548451374538, 0.6521451548625461, 0.6521451548625461, 0.3478548451374538};
    const int NT = 256, NZ = 64;  // theta samples; z panels of 4 points
    double area = 0.0;
    for (int iz = 0; iz < NZ; ++iz)
        for (int q = 0; q < 4; ++q) {
            // sphere: parameter u in [-pi/2, pi/2] (latitude); others: z in [0, 1]
            const double a = sphere ? -M_PI / 2 : 0.0, b = sphere ? M_PI / 2 : 1.0;
            const double h = (b - a) / NZ;
            const double u = a + h * (iz + 0.5 + 0.5 * gx[q]);
            const double wz = 0.5 * h * gw[q];
            for (int it = 0; it < NT; ++it) {
                const double th = 2.0 * M_PI * it / NT;
                const double c = std::cos(th), s = std::sin(th);
                double du[3], dt[3], v[3];
                if (sphere) {
                    const double cu = std::cos(u), su = std::sin(u);
                    v[0] = -cu * s; v[1] = cu * c; v[2] = 0.0;  // d/dtheta
                    lin(m, v, dt);
                    v[0] = -su * c; v[1] = -su * s; v[2] = cu;  // d/du
                    lin(m, v, du);
                } else {
                    const double rho = 1.0 + (top - 1.0) * u;
                    v[0] = -rho * s; v[1] = rho * c; v[2] = 0.0;
                    lin(m, v, dt);
                    v[0] = (top - 1.0) * c; v[1] = (top - 1.0) * s; v[2] = 1.0;
                    lin(m, v, du);
                }
                area += wz * (2.0 * M_PI / NT) * cross_norm(dt, du);
            }
        }
    return area;
}

}  // namespace

rf_status rf_surface_areas(const rf_primitive *prims, int32_t n, double *areas)
{
    if (!prims || n <= 0 || !areas) return RF_ERR_INVALID_ARG;
    for (int i = 0; i < n; ++i) {
        const rf_primitive &p = prims[i];
        if (p.type < 0 || p.type > RF_DISC || !finite_all(p.m, 12)) return RF_ERR_BAD_SCENE;
        const double ex[3] = {1, 0, 0}, ey[3] = {0, 1, 0};
        double mx[3], my[3];
        lin(p.m, ex, mx);
        lin(p.m, ey, my);
        const double plane = cross_norm(mx, my);  // area scale of the plane z = 0
        switch (p.type) {
        case RF_DISC: areas[i] = M_PI * plane; break;
        case RF_ANNULUS: areas[i] = M_PI * std::max(0.0, (double)p.util2 - (double)p.util1) * plane; break;
        case RF_RECTANGLE: areas[i] = 4.0 * plane; break;
        case RF_CYLINDER: areas[i] = revolution_area(p.m, 1.0, false); break;
        case RF_FRUSTUM: areas[i] = revolution_area(p.m, p.util1, false); break;
        default: areas[i] = revolution_area(p.m, 1.0, true); break;
        }
    }
    return RF_OK;
}

rf_status rf_segment_stacks(const rf_primitive *prims, int32_t n, const rf_bounding_volume *bvs, int32_t nbv,
                            int32_t *first_out, int32_t *count_out, int32_t cap, int32_t *n_stacks_out)
{
    if (!prims || n <= 0 || nbv < 0 || (nbv > 0 && !bvs) || cap < 0 || !n_stacks_out ||
        (cap > 0 && (!first_out || !count_out)))
        return RF_ERR_INVALID_ARG;
    std::vector<rf_primitive> e(n);
    std::vector<HitRec> tab(n);
    std::vector<float4> bs(n);
    prepare_mixed(prims, n, e.data(), tab.data(), bs.data());
    std::vector<char> cut(n + 1, 0);
    for (int b = 0; b < nbv; ++b) {
        if (bvs[b].objStartIndex >= 0 && bvs[b].objStartIndex <= n) cut[bvs[b].objStartIndex] = 1;
        if (bvs[b].objEndIndex >= 0 && bvs[b].objEndIndex <= n) cut[bvs[b].objEndIndex] = 1;
    }
    mark_stacks(e.data(), n, tab.data(), bs.data(), cut);
    int32_t k = 0;
    for (int i = 0; i < n;) {
        int32_t ti, w;
        std::memcpy(&ti, &tab[i].aux.x, 4);
        std::memcpy(&w, &tab[i].aux.w, 4);
        if (ti != kStackType && ti != kPlateType) { ++i; continue; }
        const int m = (int)((uint32_t)w >> 16);
        if (k < cap) {
            first_out[k] = i;
            count_out[k] = m;
        }
        ++k;
        i += m;
    }
    *n_stacks_out = k;
    return RF_OK;
}

rf_status rf_budgets_by_area(const rf_primitive *prims, int32_t n, int64_t total_rays, int64_t *rays_out)
{
    return rf_budgets_by_density(prims, n, nullptr, total_rays, rays_out);
}

rf_status rf_budgets_by_density(const rf_primitive *prims, int32_t n, const double *density, int64_t total_rays,
                                int64_t *rays_out)
{
    if (!prims || n <= 0 || !rays_out || total_rays < 0) return RF_ERR_INVALID_ARG;
    if (total_rays > (kMaxRaysPerEmitter / 2)) return RF_ERR_OVERFLOW;
    std::vector<double> a(n);
    rf_status s = rf_surface_areas(prims, n, a.data());
    if (s != RF_OK) return s;
    if (density)
        for (int i = 0; i < n; ++i) {
            if (!(density[i] >= 0.0) || !std::isfinite(density[i])) return RF_ERR_INVALID_ARG;
            a[i] *= density[i];
        }
    double tot = 0.0;
    for (double v : a) tot += v;
    if (!(tot > 0.0)) return RF_ERR_BAD_SCENE;
    for (int i = 0; i < n; ++i) {
        const int64_t r = (int64_t)std::llround((double)total_rays * a[i] / tot / 4.0) * 4;
        rays_out[i] = (a[i] > 0.0 && total_rays > 0) ? std::max<int64_t>(4, r) : 0;
    }
    return RF_OK;
}

rf_status rf_write_output_txt(const char *path, const double *F, int32_t n)
{
    if (!path || !F || n <= 0) return RF_ERR_INVALID_ARG;
    FILE *f = std::fopen(path, "w");
    if (!f) return RF_ERR_INVALID_ARG;
    for (int i = 0; i < n; ++i) {
        for (int j = 0; j < n; ++j) {
            // the reference stores F as float and prints with precision 8 (main.cpp:216, 238-246)
            std::fprintf(f, "%.8g,", (double)(float)F[(size_t)i * n + j]);
        }
        std::fputc('\n', f);
    }
    return std::fclose(f) == 0 ? RF_OK : RF_ERR_INVALID_ARG;
}

rf_status rf_check_F(rf_ctx *c, const double *F, const double *areas, int32_t n, double *max_sum_err,
                     double *max_recip_err)
{
    if (!c || !F || n <= 0) return RF_ERR_INVALID_ARG;
    RF_CUDA(c, cudaSetDevice(c->device));
    const size_t nn = (size_t)n * n;
    RF_CUDA(c, c->d_F.ensure(nn * sizeof(double)));
    RF_CUDA(c, c->d_misc.ensure(n * sizeof(double) + 64));
    RF_CUDA(c, cudaStreamSynchronize(c->stream));
    RF_CUDA(c, cudaMemcpyAsync(c->d_F.p, F, nn * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    double *d_areas = nullptr;
    if (areas) {
        d_areas = reinterpret_cast<double *>(static_cast<char *>(c->d_misc.p) + 64);
        RF_CUDA(c, cudaMemcpyAsync(d_areas, areas, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    }
    double *out2 = c->d_misc.as<double>();
    RF_CUDA(c, launch_check_F(c->d_F.as<double>(), d_areas, n, out2, c->stream));
    double h[2] = {0, 0};
    RF_CUDA(c, cudaMemcpyAsync(h, out2, sizeof h, cudaMemcpyDeviceToHost, c->stream));
    RF_CUDA(c, cudaStreamSynchronize(c->stream));
    if (max_sum_err) *max_sum_err = h[0];
    if (max_recip_err) *max_recip_err = h[1];
    return RF_OK;
}

rf_status rf_smooth_F(rf_ctx *c, const double *F, const double *areas, int32_t n, int32_t closed,
                      double *F_out, int32_t *iterations, double *residual)
{
    ApiRange nvtx_range("rf_smooth_F");
    if (!c || !F || !areas || !F_out || n <= 0) return RF_ERR_INVALID_ARG;
    for (int i = 0; i < n; ++i)
        if (!(areas[i] >= 0.0) || !std::isfinite(areas[i])) return fail(c, RF_ERR_INVALID_ARG, "bad area %d", i);
    RF_CUDA(c, cudaSetDevice(c->device));
    const size_t nn = (size_t)n * n;
    RF_CUDA(c, c->d_F.ensure(nn * sizeof(double)));
    RF_CUDA(c, c->d_misc.ensure((nn + 4 * (size_t)n + 8) * sizeof(double)));
    double *d_G = c->d_misc.as<double>();
    double *d_A = d_G + nn, *d_x0 = d_A + n, *d_x1 = d_x0 + n, *d_out = d_x1 + n, *d_err = d_out + n;
    // F_out goes through the F buffer: input first, result afterwards
    RF_CUDA(c, cudaStreamSynchronize(c->stream));
    RF_CUDA(c, cudaMemcpyAsync(c->d_F.p, F, nn * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    RF_CUDA(c, cudaMemcpyAsync(d_A, areas, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    DevBuf out;
    RF_CUDA(c, out.ensure(nn * sizeof(double)));
    int it = 0;
    double err = 0.0;
    cudaError_t e = launch_smooth(c->d_F.as<double>(), d_A, n, closed ? 1 : 0, 2000, 1e-13, d_G, d_x0, d_x1, d_err,
                                  out.as<double>(), &it, &err, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(F_out, out.p, nn * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    out.release();
    (void)d_out;
    if (e != cudaSuccess) return cuda_fail(c, e, "smoothing");
    if (iterations) *iterations = it;
    if (residual) *residual = err;
    return RF_OK;
}

rf_status rf_measure_fp32_peak(int32_t device, double *fma_per_s)
{
    if (!fma_per_s) return RF_ERR_INVALID_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        cudaGetLastError();
        return RF_ERR_NO_DEVICE;
    }
    if (cudaSetDevice(device) != cudaSuccess) return RF_ERR_CUDA;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int block = 256, grid = sms * 8, iters = 4096;
    float *out = nullptr;
    cudaEvent_t a, b;
    if (cudaMalloc(&out, (size_t)grid * block * 4) != cudaSuccess) return RF_ERR_OOM;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    double best = 0.0;
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(a);
        launch_fp32_probe(out, iters, grid, block, 0);
        cudaEventRecord(b);
        cudaEventSynchronize(b);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        const double fmas = (double)grid * block * iters * 16.0 * 8.0;
        if (rep > 0 && ms > 0) best = std::max(best, fmas / (ms * 1e-3));
    }
    cudaError_t e = cudaGetLastError();
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(out);
    if (e != cudaSuccess) return RF_ERR_CUDA;
    *fma_per_s = best;
    return RF_OK;
}

rf_status rf_trace_batch(rf_ctx *c, const rf_scene_desc *scenes, int32_t n_scenes, uint64_t *hits_out,
                         double *F_out)
{
    ApiRange nvtx_range("rf_trace_batch");
    if (!c) return RF_ERR_INVALID_ARG;
    rf_status st = upload_batch(c, scenes, n_scenes, true);
    if (st != RF_OK) return st;
    c->b_single = false;
    c->have_results = false;
    std::vector<Segment> seg;
    int64_t chunks = 0, nrows = 0;
    for (int s = 0; s < n_scenes; ++s) {
        if ((st = check_budgets(c, scenes[s].rays_per_emitter, scenes[s].n_prims)) != RF_OK) return st;
        for (int e = 0; e < scenes[s].n_prims; ++e)
            chunks = plan_segments(seg, e, s, 0, scenes[s].rays_per_emitter[e], kBatchChunkDraws, chunks);
        nrows += scenes[s].n_prims;
    }
    if ((st = run_batched(c, seg, chunks, false, nullptr, 0, true)) != RF_OK) return st;
    // FP64 normalisation of every row (one warp per row)
    std::vector<int64_t> rows(3 * nrows);
    int64_t r = 0;
    for (int s = 0; s < n_scenes; ++s)
        for (int e = 0; e < scenes[s].n_prims; ++e, ++r) {
            rows[r] = c->b_info[s].hits_off + (int64_t)e * scenes[s].n_prims;     // row offset
            rows[nrows + r] = scenes[s].rays_per_emitter[e];                      // rays
            reinterpret_cast<int32_t *>(&rows[2 * nrows])[r] = scenes[s].n_prims;  // row length
        }
    RF_CUDA(c, c->b_rows.ensure(rows.size() * 8 + 8 * nrows));
    RF_CUDA(c, c->d_F.ensure((size_t)c->b_hits_total * sizeof(double)));
    int64_t *d_rows = c->b_rows.as<int64_t>();
    RF_CUDA(c, cudaMemcpyAsync(d_rows, rows.data(), rows.size() * 8, cudaMemcpyHostToDevice, c->stream));
    BatchCounters *bc = c->b_counters.as<BatchCounters>();
    RF_CUDA(c, launch_converge_step(c->b_hits.as<unsigned long long>(), d_rows + nrows, d_rows, 
                                    reinterpret_cast<int32_t *>(d_rows + 2 * nrows), nrows,
                                    c->d_F.as<double>(), 0.0, d_rows + 3 * nrows, 0, &bc->flags[0], c->stream));
    if (hits_out)
        RF_CUDA(c, cudaMemcpyAsync(hits_out, c->b_hits.p, (size_t)c->b_hits_total * 8, cudaMemcpyDeviceToHost, c->stream));
    if (F_out)
        RF_CUDA(c, cudaMemcpyAsync(F_out, c->d_F.p, (size_t)c->b_hits_total * 8, cudaMemcpyDeviceToHost, c->stream));
    RF_CUDA(c, cudaMemcpyAsync(&c->last_refined, &bc->refined, 8, cudaMemcpyDeviceToHost, c->stream));
    RF_CUDA(c, cudaMemcpyAsync(c->last_work, bc->work, sizeof c->last_work, cudaMemcpyDeviceToHost, c->stream));
    RF_CUDA(c, cudaStreamSynchronize(c->stream));
    return RF_OK;
}

rf_status rf_converge_batch(rf_ctx *c, const rf_scene_desc *scenes, int32_t n_scenes, double tol,
                            int64_t round_rays, int32_t max_rounds, uint64_t *hits_out, double *F_out,
                            int64_t *rays_out, int32_t *rounds_out)
{
    ApiRange nvtx_range("rf_converge_batch");
    if (!c) return RF_ERR_INVALID_ARG;
    if (!(tol > 0.0) || round_rays <= 0 || max_rounds <= 0)
        return fail(c, RF_ERR_INVALID_ARG, "tol > 0, round_rays > 0 and max_rounds > 0 are required");
    rf_status st = upload_batch(c, scenes, n_scenes, true);
    if (st != RF_OK) return st;
    c->b_single = false;
    c->have_results = false;
    int64_t nrows = 0;
    for (int s = 0; s < n_scenes; ++s) {
        if ((st = check_budgets(c, scenes[s].rays_per_emitter, scenes[s].n_prims)) != RF_OK) return st;
        nrows += scenes[s].n_prims;
    }
    if ((int64_t)max_rounds * round_rays > kMaxRaysPerEmitter / 2)
        return fail(c, RF_ERR_OVERFLOW, "max_rounds * round_rays is too large");
    // row tables: off, rays_total, next, n | scene, emitter
    std::vector<int64_t> off(nrows), next(nrows);
    std::vector<int32_t> len(nrows), rsc(nrows), rem(nrows);
    int64_t r = 0;
    for (int s = 0; s < n_scenes; ++s)
        for (int e = 0; e < scenes[s].n_prims; ++e, ++r) {
            off[r] = c->b_info[s].hits_off + (int64_t)e * scenes[s].n_prims;
            next[r] = scenes[s].rays_per_emitter[e];
            len[r] = scenes[s].n_prims;
            rsc[r] = s;
            rem[r] = e;
        }
    RF_CUDA(c, c->b_rows.ensure((size_t)nrows * (8 * 3 + 4 * 3) + 64));
    int64_t *d_off = c->b_rows.as<int64_t>(), *d_total = d_off + nrows, *d_next = d_total + nrows;
    int32_t *d_len = reinterpret_cast<int32_t *>(d_next + nrows), *d_sc = d_len + nrows, *d_em = d_sc + nrows;
    c->seg_valid = false;  // the round planner writes d_seg on the device
    RF_CUDA(c, c->d_seg.ensure((size_t)nrows * sizeof(Segment)));
    RF_CUDA(c, c->d_F.ensure((size_t)c->b_hits_total * sizeof(double)));
    RF_CUDA(c, cudaMemcpyAsync(d_off, off.data(), nrows * 8, cudaMemcpyHostToDevice, c->stream));
    RF_CUDA(c, cudaMemsetAsync(d_total, 0, nrows * 8, c->stream));
    RF_CUDA(c, cudaMemcpyAsync(d_next, next.data(), nrows * 8, cudaMemcpyHostToDevice, c->stream));
    RF_CUDA(c, cudaMemcpyAsync(d_len, len.data(), nrows * 4, cudaMemcpyHostToDevice, c->stream));
    RF_CUDA(c, cudaMemcpyAsync(d_sc, rsc.data(), nrows * 4, cudaMemcpyHostToDevice, c->stream));
    RF_CUDA(c, cudaMemcpyAsync(d_em, rem.data(), nrows * 4, cudaMemcpyHostToDevice, c->stream));
    RF_CUDA(c, cudaMemsetAsync(c->b_hits.p, 0, (size_t)c->b_hits_total * 8, c->stream));
    RF_CUDA(c, cudaMemsetAsync(c->b_counters.p, 0, sizeof(BatchCounters), c->stream));
    RF_CUDA(c, cudaStreamSynchronize(c->stream));

    BatchCounters *bc = c->b_counters.as<BatchCounters>();
    TraceParams p = batch_params(c);
    p.seg = c->d_seg.as<Segment>();
    p.d_total = &bc->total;
    p.d_nseg = &bc->nseg;
    const int grid = batched_grid(c, false);  // also sets the kernel's shared-memory attribute

    // Graph: while (not converged && rounds < max) { plan; trace; converge; decide }
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaGraphConditionalHandle handle = 0;
    auto body_ops = [&](unsigned long long h) -> cudaError_t {
        cudaError_t e;
        if ((e = launch_plan_round(nrows, d_sc, d_em, d_total, d_next, c->d_seg.as<Segment>(), &bc->nseg, &bc->total, &bc->queue,
                                   kBatchChunkDraws, c->stream)) != cudaSuccess) return e;
        if ((e = launch_batched(p, false, batch_resident(c), c->cfg.work_counts != 0, c->b_stacks > 0, grid,
                                c->stream)) != cudaSuccess)
            return e;
        if ((e = launch_converge_step(c->b_hits.as<unsigned long long>(), d_total, d_off, d_len, nrows, nullptr,
                                      tol, d_next, round_rays, &bc->flags[0], c->stream)) != cudaSuccess) return e;
        return launch_decide_round(&bc->flags[0], max_rounds, h, c->stream);
    };
    cudaError_t e = cudaGraphCreate(&graph, 0);
    if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&handle, graph, 1, cudaGraphCondAssignDefault);
    cudaGraphNode_t node;
    cudaGraphNodeParams np{};
    if (e == cudaSuccess) {
        np.type = cudaGraphNodeTypeConditional;
        np.conditional.handle = handle;
        np.conditional.type = cudaGraphCondTypeWhile;
        np.conditional.size = 1;
        e = cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &np);
    }
    if (e == cudaSuccess) {
        cudaGraph_t body = np.conditional.phGraph_out[0];
        e = cudaStreamBeginCaptureToGraph(c->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
        if (e == cudaSuccess) {
            cudaError_t e1 = body_ops((unsigned long long)handle);
            cudaGraph_t captured = nullptr;
            cudaError_t e2 = cudaStreamEndCapture(c->stream, &captured);
            e = e1 != cudaSuccess ? e1 : e2;
        }
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
    if (e == cudaSuccess) {
        RF_CUDA(c, cudaEventRecord(c->ev0, c->stream));
        e = cudaGraphLaunch(exec, c->stream);
        RF_CUDA(c, cudaEventRecord(c->ev1, c->stream));
    }
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda_fail(c, e, "convergence graph");
    c->timed = true;
    c->last_launches = -1;  // rounds x 4 kernels, counted below
    // final FP64 normalisation
    RF_CUDA(c, launch_converge_step(c->b_hits.as<unsigned long long>(), d_total, d_off, d_len, nrows,
                                    c->d_F.as<double>(), tol, d_next, 0, &bc->flags[0], c->stream));
    int32_t flags[2] = {0, 0};
    RF_CUDA(c, cudaMemcpyAsync(flags, &bc->flags[0], 8, cudaMemcpyDeviceToHost, c->stream));
    RF_CUDA(c, cudaMemcpyAsync(&c->last_refined, &bc->refined, 8, cudaMemcpyDeviceToHost, c->stream));
    RF_CUDA(c, cudaMemcpyAsync(c->last_work, bc->work, sizeof c->last_work, cudaMemcpyDeviceToHost, c->stream));
    if (hits_out)
        RF_CUDA(c, cudaMemcpyAsync(hits_out, c->b_hits.p, (size_t)c->b_hits_total * 8, cudaMemcpyDeviceToHost, c->stream));
    if (F_out)
        RF_CUDA(c, cudaMemcpyAsync(F_out, c->d_F.p, (size_t)c->b_hits_total * 8, cudaMemcpyDeviceToHost, c->stream));
    if (rays_out) RF_CUDA(c, cudaMemcpyAsync(rays_out, d_total, nrows * 8, cudaMemcpyDeviceToHost, c->stream));
    RF_CUDA(c, cudaStreamSynchronize(c->stream));
    if (rounds_out) *rounds_out = flags[1];
    c->last_launches = 4 * flags[1];
    return RF_OK;
}

// Autotuner of the single-scene kernels: times every launch shape on a short
// trace of the current scene and keeps the fastest.  Knobs: threads per block
// (128 / 256), Philox draws per thread (1 / 2, i.e. 4 or 8 rays in registers),
// surface staging (shared-memory tiles / reads through L1), tallying (row
// histogram in shared memory / warp-aggregated global atomics) and test order
// (a thread's rays together per surface / one ray at a time).  Results are
// cached per scene shape (precision, kernel, surface count and type mix, SM
// count) in memory and, optionally, in a text file of
// "key|block gpt hist stage order" lines.  The mixed-precision kernel has one launch shape (a persistent grid of
// 1024-thread blocks) and needs no tuning.
namespace {
struct TuneChoice {
    int block, gpt, hist, stage, order;
};
std::mutex g_tune_mu;
std::map<std::string, TuneChoice> g_tune_cache;

std::string tune_key(const rf_ctx *c, int use_bv)
{
    int types[6] = {0, 0, 0, 0, 0, 0};
    for (const rf_primitive &p : c->prims) ++types[p.type];
    std::ostringstream k;
    k << "v2 prec=" << c->cfg.precision << " bv=" << use_bv << " n=" << c->n << " nbv=" << c->nbv << " t=";
    for (int i = 0; i < 6; ++i) k << types[i] << (i < 5 ? "," : "");
    k << " sm=" << c->sms;
    return k.str();
}

bool tune_lookup_file(const char *path, const std::string &key, TuneChoice &out)
{
    std::ifstream f(path);
    std::string line;
    bool found = false;
    while (std::getline(f, line)) {
        const size_t bar = line.find('|');
        if (bar == std::string::npos || line.compare(0, bar, key) != 0 || bar != key.size()) continue;
        std::istringstream v(line.substr(bar + 1));
        TuneChoice t{};
        if (v >> t.block >> t.gpt >> t.hist >> t.stage >> t.order) {
            out = t;
            found = true;  // the last entry wins
        }
    }
    return found;
}

void tune_apply(rf_ctx *c, const TuneChoice &t)
{
    c->block = t.block;
    c->gpt = t.gpt;
    c->hist = t.hist;
    c->stage = t.stage;
    c->order = t.order;
}

// Trial budgets of the autotuner: about 2^25 rays (the steady state of a
// persistent wave, a few ms), spread like the last trace's budgets when there
// was one (the workload being tuned for), else evenly.
std::vector<int64_t> tune_budgets(const rf_ctx *c)
{
    const double target = (double)((int64_t)1 << 25);
    std::vector<int64_t> rays(c->n, std::max<int64_t>(4096, ((int64_t)1 << 25) / c->n) / 4 * 4);
    if ((int)c->last_rays.size() == c->n) {
        double tot = 0.0;
        for (int64_t r : c->last_rays) tot += (double)r;
        if (tot > 0.0)
            for (int e = 0; e < c->n; ++e) rays[e] = (int64_t)(target * (double)c->last_rays[e] / tot) / 4 * 4;
    }
    return rays;
}

// MIXED: a single scene of at most kSmallMax surfaces may take the small-scene
// kernel (4 or 8 rays per thread) instead of the batched kernel; time the three
// and keep the fastest (results are the same ray for ray: same arithmetic, and a
// ray's result depends on the ray alone).  The choice is cached like the plain
// kernels' (block field 1 = small-scene kernel, 2 = batched kernel).
rf_status autotune_mixed(rf_ctx *c, const char *cache_path)
{
    if (!c->b_single || c->n > kSmallMax) return RF_OK;  // the batched kernel only
    const std::string key = tune_key(c, 0);
    TuneChoice best{};
    bool found = false;
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) { best = it->second; found = true; }
    }
    if (!found && cache_path && tune_lookup_file(cache_path, key, best)) {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        g_tune_cache[key] = best;
        found = true;
    }
    if (found) {
        c->mixed_path = best.block;
        c->gpt = best.gpt;
        return RF_OK;
    }
    const std::vector<int64_t> rays = tune_budgets(c);
    const int saved_path = c->mixed_path, saved_gpt = c->gpt;
    double best_ms = 1e300;
    for (int path : {2, 1})
        for (int gpt : {1, 2}) {
            if (path == 2 && gpt == 2) continue;
            c->mixed_path = path;
            c->gpt = gpt;
            double ms_min = 1e300;
            for (int rep = 0; rep < 3; ++rep) {
                rf_status s = rf_trace_async(c, rays.data(), 0);
                double ms = 0.0;
                if (s == RF_OK) s = rf_last_trace_stats(c, &ms, nullptr);
                if (s != RF_OK) {
                    c->mixed_path = saved_path;
                    c->gpt = saved_gpt;
                    return s;
                }
                if (rep > 0) ms_min = std::min(ms_min, ms);  // the first run warms up
            }
            if (ms_min < best_ms) {
                best_ms = ms_min;
                best = TuneChoice{path, gpt, -1, -1, -1};
            }
        }
    c->have_results = false;
    c->mixed_path = best.block;
    c->gpt = best.gpt;
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        g_tune_cache[key] = best;
    }
    if (cache_path) {
        std::ofstream f(cache_path, std::ios::app);
        if (f) f << key << "|" << best.block << " " << best.gpt << " -1 -1 -1\n";
    }
    return RF_OK;
}
}  // namespace

rf_status rf_autotune(rf_ctx *c, int32_t use_bv, const char *cache_path)
{
    ApiRange nvtx_range("rf_autotune");
    rf_status s = require_scene(c);
    if (s != RF_OK) return s;
    if (use_bv && c->nbv <= 0) return fail(c, RF_ERR_STATE, "use_bv set but the scene has no bounding volumes");
    if (c->cfg.precision == RF_PREC_MIXED)  // with bounding surfaces: one kernel, nothing to choose
        return use_bv ? check_mixed_bv(c) : autotune_mixed(c, cache_path);
    const std::string key = tune_key(c, use_bv ? 1 : 0);
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            tune_apply(c, it->second);
            return RF_OK;
        }
    }
    TuneChoice best{};
    if (cache_path && tune_lookup_file(cache_path, key, best)) {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        g_tune_cache[key] = best;
        tune_apply(c, best);
        return RF_OK;
    }
    // trials long enough for the steady state of a persistent wave: about 2^25
    // rays (a few ms each), spread like the last trace's budgets when there was
    // one (the workload being tuned for), else evenly
    const std::vector<int64_t> rays = tune_budgets(c);
    const bool bv = use_bv != 0;
    const bool wide = !bv && c->cfg.precision != RF_PREC_FP64;
    double best_ms = 1e300;
    const TuneChoice saved{c->block, c->gpt, c->hist, c->stage, c->order};
    for (int block : {128, 256})
        for (int gpt : {1, 2}) {
            if (gpt == 2 && !wide) continue;
            for (int hist : {1, 0}) {
                if (hist && c->n > kHistMax) continue;
                for (int stage : {1, 0})
                for (int order : {0, 1}) {
                    if (bv && stage == 0) continue;  // the bounding-surface kernel reads through L1 anyway
                    if (bv && order == 1) continue;  // and tests one ray at a time anyway
                    tune_apply(c, TuneChoice{block, gpt, hist, stage, order});
                    double ms_min = 1e300;
                    for (int rep = 0; rep < 3; ++rep) {
                        if ((s = rf_trace_async(c, rays.data(), use_bv)) != RF_OK) {
                            tune_apply(c, saved);
                            return s;
                        }
                        double ms = 0.0;
                        if ((s = rf_last_trace_stats(c, &ms, nullptr)) != RF_OK) {
                            tune_apply(c, saved);
                            return s;
                        }
                        if (rep > 0) ms_min = std::min(ms_min, ms);  // the first run warms up
                    }
                    if (ms_min < best_ms) {
                        best_ms = ms_min;
                        best = TuneChoice{block, gpt, hist, stage, order};
                    }
                }
            }
        }
    c->have_results = false;
    tune_apply(c, best);
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        g_tune_cache[key] = best;
    }
    if (cache_path) {
        std::ofstream f(cache_path, std::ios::app);
        if (f) f << key << "|" << best.block << " " << best.gpt << " " << best.hist << " " << best.stage << " "
                 << best.order << "\n";
    }
    return RF_OK;
}

rf_status rf_get_launch_config(rf_ctx *c, int32_t *block, int32_t *rays_per_thread, int32_t *smem_hist,
                               int32_t *smem_table, int32_t *one_ray_at_a_time)
{
    if (!c) return RF_ERR_INVALID_ARG;
    if (c->cfg.precision == RF_PREC_MIXED) {  // the mixed kernel the next trace takes
        const bool small = use_small(c);
        if (block) *block = small ? kSmallThreads : kBatchBlock;
        if (rays_per_thread) *rays_per_thread = small ? 4 * small_gpt(c, false) : 4 * kBatchChunkDraws / kBatchBlock;
        if (smem_hist) *smem_hist = 1;
        if (smem_table) *smem_table = small || batch_resident(c) ? 1 : 0;
        if (one_ray_at_a_time) *one_ray_at_a_time = 0;
        return RF_OK;
    }
    if (block) *block = c->block > 0 ? c->block : (c->cfg.block_size > 0 ? c->cfg.block_size : kBlock);
    if (rays_per_thread) *rays_per_thread = 4 * (c->gpt > 0 ? c->gpt : (c->cfg.rays_per_thread == 8 ? 2 : 1));
    if (smem_hist) *smem_hist = c->hist >= 0 ? c->hist : 1;
    if (smem_table) *smem_table = c->stage >= 0 ? c->stage : 1;
    if (one_ray_at_a_time) *one_ray_at_a_time = c->order == 1 ? 1 : 0;
    return RF_OK;
}

rf_status rf_last_work_counts(rf_ctx *c, uint64_t *counts)
{
    if (!c || !counts) return RF_ERR_INVALID_ARG;
    for (int i = 0; i < 8; ++i) counts[i] = c->last_work[i];
    return RF_OK;
}

rf_status rf_last_refine_count(rf_ctx *c, uint64_t *refined)
{
    if (!c || !refined) return RF_ERR_INVALID_ARG;
    *refined = c->last_refined;
    return RF_OK;
}

}  // extern "C"
