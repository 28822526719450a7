// rf_kern_fast.cu -- single-scene kernels with the FP32 hardware
// approximations (the counterparts of OpenCL native_*), compiled with the
// default contraction of products and sums into FMA: the plain kernel and the
// small-scene mixed-precision kernel.
#include "rf_trace_kernels.cuh"
#include "rf_batched.cuh"
#include "rf_mixed_small.cuh"

namespace rf {
template cudaError_t launch_trace<MFast>(const LaunchCfg &, const TraceParams &, cudaStream_t);
template int trace_blocks_per_sm<MFast>(const LaunchCfg &);

template <int GPT, bool REC>
static cudaError_t launch_s(const TraceParams &p, int grid, cudaStream_t st)
{
    mixed_small_kernel<GPT, REC><<<grid, kSmallThreads, 0, st>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_mixed_small(const TraceParams &p, int gpt, bool rec, int grid, cudaStream_t st)
{
    if (p.n <= 0 || p.n > kSmallMax) return cudaErrorInvalidValue;
    if (rec) return launch_s<1, true>(p, grid, st);
    return gpt == 2 ? launch_s<2, false>(p, grid, st) : launch_s<1, false>(p, grid, st);
}

// Resident blocks per SM, queried once per process (every GPU of a run is the same part).
template <int GPT, bool REC>
static int occ_s()
{
    static const int nb = [] {
        int r = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, mixed_small_kernel<GPT, REC>, kSmallThreads, 0) !=
            cudaSuccess)
            r = 0;
        return r;
    }();
    return nb;
}

int mixed_small_blocks_per_sm(int gpt, bool rec)
{
    if (rec) return occ_s<1, true>();
    return gpt == 2 ? occ_s<2, false>() : occ_s<1, false>();
}

}  // namespace rf
