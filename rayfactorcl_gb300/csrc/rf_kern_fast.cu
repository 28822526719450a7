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

cudaError_t launch_batched(const TraceParams &p, bool rec, int grid, cudaStream_t st)
{
    const size_t smem = sizeof(BatchSmem);
    if (rec) {
        cudaError_t e = cudaFuncSetAttribute(batched_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        batched_kernel<true><<<grid, kBatchThreads, smem, st>>>(p);
    } else {
        cudaError_t e = cudaFuncSetAttribute(batched_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        batched_kernel<false><<<grid, kBatchThreads, smem, st>>>(p);
    }
    return cudaGetLastError();
}

int batched_blocks_per_sm(bool rec)
{
    const size_t smem = sizeof(BatchSmem);
    int nb = 0;
    if (rec) {
        cudaFuncSetAttribute(batched_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, batched_kernel<true>, kBatchThreads, smem);
    } else {
        cudaFuncSetAttribute(batched_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, batched_kernel<false>, kBatchThreads, smem);
    }
    return nb;
}
}  // namespace rf
