// rf_mixed_small.cuh -- mixed-precision tracing of one small scene with the
// plain kernel's launch shape (RayFactorGPU.cl:481-527's method: every ray
// against every surface).
//
// Below a few tens of surfaces the batched kernel's sorting and culling cost
// more than the tests they save.  This kernel keeps the scene's tables in shared
// memory, gives each thread 4 or 8 rays (one or two Philox draws) and tests them
// together against each surface in index order, like the plain kernel, with the
// batched kernel's arithmetic: the same emission (emit_mixed), the same mixed
// tests with FP64 re-evaluation of ill-conditioned quadrics, the same skipped
// self-test of a planar emitter (self_skip) and the same per-ray resolution
// (resolve_brute) as its small-scene path.  A scene traced here therefore gets,
// ray for ray, the batched kernel's results for it.
#pragma once

#include "rf_batched.cuh"

namespace rf {

static_assert(kSmallThreads % 32 == 0, "whole warps");

template <int GPT, bool REC>
__global__ void __launch_bounds__(kSmallThreads, GPT == 1 ? 4 : 1) mixed_small_kernel(const TraceParams p)
{
    constexpr int R = 4 * GPT;
    __shared__ HitRec s_tab[kSmallMax];
    __shared__ int s_hist[kSmallMax];
    __shared__ rf_primitive s_emit;
    __shared__ float4 s_frame[kEmitFrameWords];

    const int n = p.n;
    const int tid = threadIdx.x, lane = tid & 31;
    const bool sc = (p.compat & RF_COMPAT_SPHERE) != 0;
    const float eps = p.eps;
    {
        const float4 *src = reinterpret_cast<const float4 *>(p.tab);
        float4 *dst = reinterpret_cast<float4 *>(s_tab);
        for (int i = tid; i < 4 * n; i += blockDim.x) dst[i] = __ldg(src + i);
        for (int i = tid; i < n; i += blockDim.x) s_hist[i] = 0;
    }
    const int64_t c0 = (p.total_chunks * (int64_t)blockIdx.x) / gridDim.x;
    const int64_t c1 = (p.total_chunks * (int64_t)(blockIdx.x + 1)) / gridDim.x;
    int64_t seg_next = -1;
    Segment sg;
    sg.emitter = -1;
    int pending = 0, nref = 0;

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
            if (!REC && sg.emitter >= 0 && ns.emitter != sg.emitter) {
                flush(sg.emitter);
                pending = 0;
            }
            sg = ns;
            seg_next = (s + 1 < p.nseg) ? p.seg[s + 1].chunk_begin : INT64_MAX;
            __syncthreads();
            if (tid < (int)(sizeof(rf_primitive) / 4))
                reinterpret_cast<float *>(&s_emit)[tid] = reinterpret_cast<const float *>(p.emit + sg.emitter)[tid];
            if (tid < kEmitFrameWords) s_frame[tid] = p.frame[(int64_t)sg.emitter * kEmitFrameWords + tid];
            __syncthreads();
        }
        if (!REC && pending >= 4096) {  // keep the 32-bit bins far from overflow
            flush(sg.emitter);
            pending = 0;
        }
        ++pending;

        const int64_t gid0 = (sg.ray_begin >> 2) + (c - sg.chunk_begin) * (int64_t)(blockDim.x * GPT);
        Ray<float> ray[R];
#pragma unroll
        for (int g = 0; g < GPT; ++g) {
            const int64_t gid = gid0 + (int64_t)g * blockDim.x + tid;
            const uint4 u = stream_bits(p.compat, p.key1, p.scene_id, sg.emitter, gid);
            const float uf[4] = {u01(u.x), u01(u.y), u01(u.z), u01(u.w)};
#pragma unroll
            for (int v = 0; v < 4; ++v) {
                float r[4];
                rotate_uniforms(uf, v, r);
                ray[g * 4 + v] = emit_mixed(s_emit, s_frame, r);
            }
        }
        float tb[R];
        int bi[R];
        uint32_t dmask = 0u;  // bit k: ray k deferred a test
#pragma unroll
        for (int k = 0; k < R; ++k) { tb[k] = MFast::inf(); bi[k] = -1; }
        const int skip = self_skip(s_emit, sg.emitter);  // block-uniform
        for (int j = 0; j < n; ++j) {
            if (j == skip) continue;
            const HitRec h = s_tab[j];
            const int type = __float_as_int(h.aux.x);
            // the same per-type tests as hit_mixed, each case expanded for the thread's rays
#define RF_MIXED_ALL(T)                                                        \
    _Pragma("unroll") for (int k = 0; k < R; ++k)                              \
    {                                                                          \
        bool defer = false;                                                    \
        const float t = hit_mixed(T, h, ray[k], eps, sc, defer);               \
        if (t < tb[k]) { tb[k] = t; bi[k] = j; }                               \
        dmask |= defer ? (1u << k) : 0u;                                       \
    }
            switch (type) {  // warp-uniform
            case RF_DISC: RF_MIXED_ALL(RF_DISC) break;
            case RF_ANNULUS: RF_MIXED_ALL(RF_ANNULUS) break;
            case RF_RECTANGLE: RF_MIXED_ALL(RF_RECTANGLE) break;
            case RF_CYLINDER: RF_MIXED_ALL(RF_CYLINDER) break;
            case RF_FRUSTUM: RF_MIXED_ALL(RF_FRUSTUM) break;
            case RF_SPHERE: RF_MIXED_ALL(RF_SPHERE) break;
            case kStackType: {  // one test for the segment stack j belongs to
                const int first = stack_first(h, j);
#pragma unroll
                for (int k = 0; k < R; ++k) {
                    bool defer = false;
                    int ring;
                    const float t = stack_mixed(h, ray[k], eps, defer, ring);
                    if (t < tb[k]) { tb[k] = t; bi[k] = first + ring; }
                    dmask |= defer ? (1u << k) : 0u;
                }
                j = stack_end(h, j) - 1;
                break;
            }
            case kPlateType: {  // one test for the plate j belongs to
#pragma unroll
                for (int k = 0; k < R; ++k) {
                    int idx;
                    const float t = plate_mixed(h, j, s_tab, true, ray[k], eps, idx);
                    if (t < tb[k]) { tb[k] = t; bi[k] = idx; }
                }
                j = stack_end(h, j) - 1;
                break;
            }
            default: break;  // validated away on the host
            }
#undef RF_MIXED_ALL
        }
        unsigned long long *grow = p.hits + (int64_t)sg.emitter * n;
#pragma unroll
        for (int k = 0; k < R; ++k) {
            const int64_t rid = (gid0 + (int64_t)(k >> 2) * blockDim.x + tid) * 4 + (k & 3);
            const bool valid = rid >= sg.ray_begin && rid < sg.ray_end;
            const int h = valid ? resolve_brute<true>(bi[k], (dmask >> k) & 1u, 0, n, true, s_tab, nullptr, ray[k], eps, sc,
                                                skip, nref)
                                : -1;
            if (REC) {
                if (valid) p.rec[rid - p.rec_base] = h;
            } else {
                warp_tally(s_hist, h);  // every lane
            }
        }
    }
    if (!REC && sg.emitter >= 0) flush(sg.emitter);
    int tot = nref;
#pragma unroll
    for (int o = 16; o; o >>= 1) tot += __shfl_xor_sync(0xffffffffu, tot, o);
    if (lane == 0 && tot && p.refined) atomicAdd(p.refined, (unsigned long long)tot);
}

}  // namespace rf
