// rf_kern_fast.cu -- single-scene kernels with the FP32 hardware
// approximations (the counterparts of OpenCL native_*), compiled with the
// default contraction of products and sums into FMA.
#include "rf_trace_kernels.cuh"
#include "rf_batched.cuh"

namespace rf {
template cudaError_t launch_trace<MFast>(const LaunchCfg &, const TraceParams &, cudaStream_t);
template int trace_blocks_per_sm<MFast>(const LaunchCfg &);

static_assert(kBatchThreads * kBatchDraws == kBatchChunkDraws, "chunk size");

size_t batched_smem_bytes() { return sizeof(BatchSmem); }

template <bool REC, bool RES>
static cudaError_t launch_b(const TraceParams &p, int grid, cudaStream_t st)
{
    const size_t smem = sizeof(BatchSmem);
    cudaError_t e = cudaFuncSetAttribute(batched_kernel<REC, RES>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    batched_kernel<REC, RES><<<grid, kBatchThreads, smem, st>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_batched(const TraceParams &p, bool rec, bool resident, int grid, cudaStream_t st)
{
    if (rec) return resident ? launch_b<true, true>(p, grid, st) : launch_b<true, false>(p, grid, st);
    return resident ? launch_b<false, true>(p, grid, st) : launch_b<false, false>(p, grid, st);
}

template <bool REC, bool RES>
static int occ_b()
{
    const size_t smem = sizeof(BatchSmem);
    int nb = 0;
    cudaFuncSetAttribute(batched_kernel<REC, RES>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, batched_kernel<REC, RES>, kBatchThreads, smem);
    return nb;
}

int batched_blocks_per_sm(bool rec, bool resident)
{
    if (rec) return resident ? occ_b<true, true>() : occ_b<true, false>();
    return resident ? occ_b<false, true>() : occ_b<false, false>();
}

int batched_tile() { return kBatchTile; }

}  // namespace rf
