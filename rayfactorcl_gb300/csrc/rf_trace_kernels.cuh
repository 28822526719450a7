// rf_trace_kernels.cuh -- the single-scene tracing kernels, templated on the
// arithmetic policy.  Included by one translation unit per policy, which
// instantiates launch_trace<M> and trace_blocks_per_sm<M>.
//
// Work decomposition (replaces one NDRange per emitter, RayFactorCL/main.cpp:
// 162-182): the rays of all emitters form segments; a segment is cut into
// chunks of block*gpt Philox draws (4 rays each, RayFactorGPU.cl:497-506);
// the grid is one wave of persistent blocks and block b owns a contiguous
// range of chunks, so its emitter changes rarely.  Every thread keeps its
// 4*gpt rays in registers and walks the surface table once, testing all of
// its rays against each surface, so a table entry is loaded once per 4*gpt
// ray tests and the type switch is warp-uniform.  Surfaces are visited in
// index order and a hit replaces the best only when strictly nearer, so the
// winner of every ray is the one RayFactorGPU.cl:445-472 picks.  Tallies go
// to a per-block shared-memory histogram of the emitter's row (warp-aggregated
// with match.any) and are flushed as 64-bit atomics, or straight to the
// 64-bit global row when the row does not fit.
#pragma once

#include "rf_device.cuh"

namespace rf {

__device__ __forceinline__ HitRec load_rec(const HitRec *tab, int j)
{
    const float4 *q = reinterpret_cast<const float4 *>(tab + j);
    HitRec h;
    h.r0 = __ldg(q);
    h.r1 = __ldg(q + 1);
    h.r2 = __ldg(q + 2);
    h.aux = __ldg(q + 3);
    return h;
}

// RayFactorGPU.cl:445-472 over global-memory records [start, end).
template <class M>
__device__ __forceinline__ int find_object(const HitRec *tab, int start, int end,
                                           const Ray<typename M::T> &w, typename M::T eps, bool sc)
{
    using T = typename M::T;
    int best = -1;
    T tbest = M::inf(), t = M::inf();
    for (int j = start; j < end; ++j) {
        const HitRec h = load_rec(tab, j);
        t = hit_any<M>(__float_as_int(h.aux.x), h, w, eps, sc, t);
        if (t < tbest) { tbest = t; best = j; }
    }
    return best;
}

// RayFactorGPU.cl:580-619: nearest bounding surface, immediate child search
// for settings == 1, otherwise a child search of the winner afterwards.
template <class M>
__device__ __forceinline__ int trace_bv(const TraceParams &p, const Ray<typename M::T> &w,
                                        typename M::T eps, bool sc)
{
    using T = typename M::T;
    T tbest = M::inf(), t = M::inf();
    int bvi = -1, obj = -1;
    const bool stale = (p.compat & RF_COMPAT_BV_STALE) != 0;
    for (int b = 0; b < p.nbv; ++b) {
        const HitRec hb = load_rec(p.bvtab, b);
        t = hit_any<M>(__float_as_int(hb.aux.x), hb, w, eps, sc, t);
        if (t < tbest) {
            const int4 info = __ldg(p.bvinfo + b);  // settings, start, end
            if (info.x == 1) {
                obj = find_object<M>(p.tab, info.y, info.z, w, eps, sc);
                if (obj != -1) { tbest = t; bvi = b; }
            } else {
                tbest = t;
                bvi = b;
                if (!stale) obj = -1;
            }
        }
    }
    if (bvi != -1 && obj == -1) {
        const int4 info = __ldg(p.bvinfo + bvi);
        obj = find_object<M>(p.tab, info.y, info.z, w, eps, sc);
    }
    return obj;
}

template <class M, int GPT, bool BV, bool REC, bool STAGE, bool SERIAL>
__global__ void __launch_bounds__(kBlock) trace_kernel(const TraceParams p)
{
    using T = typename M::T;
    constexpr int R = 4 * GPT;
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ rf_primitive s_emit;

    const int n = p.n;
    const int tid = threadIdx.x;
    constexpr bool stage = !BV && STAGE;  // surfaces in smem tiles, else through L1
    const bool tiled = stage && n > kTile;
    const int tab_cap = stage ? (tiled ? kTile : n) : 0;
    HitRec *s_tab = reinterpret_cast<HitRec *>(smem);
    int *s_hist = reinterpret_cast<int *>(smem + (size_t)tab_cap * sizeof(HitRec));
    const bool hist = !REC && p.use_smem_hist;
    const T eps = T(p.eps);
    const bool sc = (p.compat & RF_COMPAT_SPHERE) != 0;

    if (hist)
        for (int i = tid; i < n; i += blockDim.x) s_hist[i] = 0;
    if (stage && !tiled) {
        const float4 *src = reinterpret_cast<const float4 *>(p.tab);
        float4 *dst = reinterpret_cast<float4 *>(s_tab);
        for (int i = tid; i < 4 * n; i += blockDim.x) dst[i] = __ldg(src + i);
    }

    const int64_t c0 = (p.total_chunks * (int64_t)blockIdx.x) / gridDim.x;
    const int64_t c1 = (p.total_chunks * (int64_t)(blockIdx.x + 1)) / gridDim.x;
    int64_t seg_next = -1;
    Segment sg;
    sg.emitter = -1;
    int pending = 0;

    auto flush = [&](int emitter) {
        __syncthreads();
        unsigned long long *row = p.hits + (int64_t)emitter * n;
        for (int i = tid; i < n; i += blockDim.x) {
            const int v = s_hist[i];
            if (v) {
                atomicAdd(row + i, (unsigned long long)v);
                s_hist[i] = 0;
            }
        }
        __syncthreads();
    };

    for (int64_t c = c0; c < c1; ++c) {
        if (c >= seg_next) {  // block-uniform
            const int s = find_segment(p.seg, p.nseg, c);
            const Segment ns = p.seg[s];
            if (hist && sg.emitter >= 0 && ns.emitter != sg.emitter) {
                flush(sg.emitter);
                pending = 0;
            }
            sg = ns;
            seg_next = (s + 1 < p.nseg) ? p.seg[s + 1].chunk_begin : INT64_MAX;
            __syncthreads();
            if (tid < (int)(sizeof(rf_primitive) / 4))
                reinterpret_cast<float *>(&s_emit)[tid] =
                    reinterpret_cast<const float *>(p.emit + sg.emitter)[tid];
            __syncthreads();
        }
        if (hist && pending >= 4096) {  // keep the 32-bit bins far from overflow
            flush(sg.emitter);
            pending = 0;
        }
        ++pending;

        const int64_t gid0 = (sg.ray_begin >> 2) + (c - sg.chunk_begin) * (int64_t)(blockDim.x * GPT);
        Ray<T> ray[R];
#pragma unroll
        for (int g = 0; g < GPT; ++g) {
            const int64_t gid = gid0 + (int64_t)g * blockDim.x + tid;
            const uint4 u = stream_bits(p.compat, p.key1, p.scene_id, sg.emitter, gid);
            const float uf[4] = {u01(u.x), u01(u.y), u01(u.z), u01(u.w)};
#pragma unroll
            for (int v = 0; v < 4; ++v) {
                float r[4];
                rotate_uniforms(uf, v, r);
                ray[g * 4 + v] = emit_ray<M>(s_emit, r);
            }
        }

        int bi[R];
        if (BV) {
#pragma unroll
            for (int k = 0; k < R; ++k) bi[k] = trace_bv<M>(p, ray[k], eps, sc);
        } else if (SERIAL) {
            // One ray at a time against the table: a single copy of each surface
            // test in the instruction stream (the 4- or 8-ray unrolled tests with
            // the IEEE sequences of the exact mapping strain the instruction cache)
            // and half the registers (the rays wait in local memory).  Faster on
            // small scenes; the autotuner decides.
            T tb[R];
#pragma unroll
            for (int k = 0; k < R; ++k) { tb[k] = M::inf(); bi[k] = -1; }
            const int step = stage ? kTile : n;
            for (int t0 = 0; t0 < n; t0 += step) {
                const int cnt = min(step, n - t0);
                if (tiled) {
                    __syncthreads();
                    const float4 *src = reinterpret_cast<const float4 *>(p.tab + t0);
                    float4 *dst = reinterpret_cast<float4 *>(s_tab);
                    for (int i = tid; i < 4 * cnt; i += blockDim.x) dst[i] = __ldg(src + i);
                    __syncthreads();
                }
#pragma unroll 1
                for (int k = 0; k < R; ++k) {
                    const Ray<T> rk = ray[k];
                    T tbk = tb[k];
                    int bik = bi[k];
                    for (int jj = 0; jj < cnt; ++jj) {
                        const HitRec h = stage ? s_tab[jj] : load_rec(p.tab, t0 + jj);
                        T t;
                        switch (__float_as_int(h.aux.x)) {  // warp-uniform
                        case RF_DISC: t = disc_hit<M>(h, rk, eps); break;
                        case RF_ANNULUS: t = annulus_hit<M>(h, rk, eps); break;
                        case RF_RECTANGLE: t = rectangle_hit<M>(h, rk, eps); break;
                        case RF_CYLINDER: t = cylinder_hit<M>(h, rk, eps); break;
                        case RF_FRUSTUM: t = frustum_hit<M>(h, rk, eps); break;
                        case RF_SPHERE: t = sphere_hit<M>(h, rk, eps, sc); break;
                        default: t = M::inf(); break;  // validated away on the host
                        }
                        if (t < tbk) { tbk = t; bik = t0 + jj; }
                    }
                    tb[k] = tbk;
                    bi[k] = bik;
                }
            }
        } else {
            T tb[R];
#pragma unroll
            for (int k = 0; k < R; ++k) { tb[k] = M::inf(); bi[k] = -1; }
            const int step = stage ? kTile : n;
            for (int t0 = 0; t0 < n; t0 += step) {
                const int cnt = min(step, n - t0);
                if (tiled) {
                    __syncthreads();
                    const float4 *src = reinterpret_cast<const float4 *>(p.tab + t0);
                    float4 *dst = reinterpret_cast<float4 *>(s_tab);
                    for (int i = tid; i < 4 * cnt; i += blockDim.x) dst[i] = __ldg(src + i);
                    __syncthreads();
                }
                for (int jj = 0; jj < cnt; ++jj) {
                    const HitRec h = stage ? s_tab[jj] : load_rec(p.tab, t0 + jj);
                    const int j = t0 + jj;
                    switch (__float_as_int(h.aux.x)) {  // warp-uniform
#define RF_TEST_ALL(call)                                               \
    _Pragma("unroll") for (int k = 0; k < R; ++k)                       \
    {                                                                   \
        const T t = call;                                               \
        if (t < tb[k]) { tb[k] = t; bi[k] = j; }                        \
    }
                    case RF_DISC: RF_TEST_ALL((disc_hit<M>(h, ray[k], eps))) break;
                    case RF_ANNULUS: RF_TEST_ALL((annulus_hit<M>(h, ray[k], eps))) break;
                    case RF_RECTANGLE: RF_TEST_ALL((rectangle_hit<M>(h, ray[k], eps))) break;
                    case RF_CYLINDER: RF_TEST_ALL((cylinder_hit<M>(h, ray[k], eps))) break;
                    case RF_FRUSTUM: RF_TEST_ALL((frustum_hit<M>(h, ray[k], eps))) break;
                    case RF_SPHERE: RF_TEST_ALL((sphere_hit<M>(h, ray[k], eps, sc))) break;
                    default: break;  // validated away on the host
#undef RF_TEST_ALL
                    }
                }
            }
        }

        unsigned long long *grow = p.hits + (int64_t)sg.emitter * n;
#pragma unroll
        for (int k = 0; k < R; ++k) {
            const int64_t rid = (gid0 + (int64_t)(k >> 2) * blockDim.x + tid) * 4 + (k & 3);
            const bool valid = rid >= sg.ray_begin && rid < sg.ray_end;
            const int h = valid ? bi[k] : -1;
            if (REC) {
                if (valid) p.rec[rid - p.rec_base] = h;
            } else if (hist) {
                warp_tally(s_hist, h);
            } else {
                warp_tally_global(grow, h);
            }
        }
    }
    if (hist && sg.emitter >= 0) flush(sg.emitter);
}

template <class M, int GPT, bool BV, bool REC, bool STAGE, bool SERIAL>
static cudaError_t launch_one(const LaunchCfg &cfg, const TraceParams &p, cudaStream_t st)
{
    auto k = trace_kernel<M, GPT, BV, REC, STAGE, SERIAL>;
    if (cfg.smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cfg.smem);
        if (e != cudaSuccess) return e;
    }
    k<<<cfg.grid, cfg.block, cfg.smem, st>>>(p);
    return cudaGetLastError();
}

template <class M, int GPT, bool BV, bool REC, bool STAGE, bool SERIAL>
static int occupancy_one(const LaunchCfg &cfg)
{
    int nb = 0;
    auto k = trace_kernel<M, GPT, BV, REC, STAGE, SERIAL>;
    if (cfg.smem > 48 * 1024)
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cfg.smem);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, cfg.block, cfg.smem) != cudaSuccess)
        return 0;
    return nb;
}

#define RF_DISPATCH_S(FN, S, ...)                                                   \
    do {                                                                            \
        if (cfg.gpt == 2) {                                                         \
            if (cfg.stage) return FN<M, 2, false, false, true, S>(__VA_ARGS__);     \
            return FN<M, 2, false, false, false, S>(__VA_ARGS__);                   \
        }                                                                           \
        if (cfg.stage) return FN<M, 1, false, false, true, S>(__VA_ARGS__);         \
        return FN<M, 1, false, false, false, S>(__VA_ARGS__);                       \
    } while (0)
#define RF_DISPATCH(FN, ...)                                                        \
    do {                                                                            \
        if (cfg.rec) {                                                              \
            if (cfg.bv) return FN<M, 1, true, true, false, false>(__VA_ARGS__);     \
            return FN<M, 1, false, true, true, false>(__VA_ARGS__);                 \
        }                                                                           \
        if (cfg.bv) return FN<M, 1, true, false, false, false>(__VA_ARGS__);        \
        if (cfg.serial) RF_DISPATCH_S(FN, true, __VA_ARGS__);                       \
        RF_DISPATCH_S(FN, false, __VA_ARGS__);                                      \
    } while (0)

template <class M>
cudaError_t launch_trace(const LaunchCfg &cfg, const TraceParams &p, cudaStream_t st)
{
    RF_DISPATCH(launch_one, cfg, p, st);
}

template <class M>
int trace_blocks_per_sm(const LaunchCfg &cfg)
{
    RF_DISPATCH(occupancy_one, cfg);
}

#undef RF_DISPATCH
#undef RF_DISPATCH_S

}  // namespace rf
