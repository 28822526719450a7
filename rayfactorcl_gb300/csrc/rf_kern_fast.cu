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

template <bool REC, bool RES, bool CNT>
static cudaError_t launch_b(const TraceParams &p, int grid, cudaStream_t st)
{
    const size_t smem = sizeof(BatchSmem);
    auto k = batched_kernel<REC, RES, CNT>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k<<<grid, kBatchThreads, smem, st>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_batched(const TraceParams &p, bool rec, bool resident, bool count, int grid, cudaStream_t st)
{
    if (rec) return resident ? launch_b<true, true, false>(p, grid, st) : launch_b<true, false, false>(p, grid, st);
    if (count) return resident ? launch_b<false, true, true>(p, grid, st) : launch_b<false, false, true>(p, grid, st);
    return resident ? launch_b<false, true, false>(p, grid, st) : launch_b<false, false, false>(p, grid, st);
}

template <bool REC, bool RES>
static int occ_b()
{
    const size_t smem = sizeof(BatchSmem);
    int nb = 0;
    auto k = batched_kernel<REC, RES, false>;
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, kBatchThreads, smem);
    return nb;
}

int batched_blocks_per_sm(bool rec, bool resident)
{
    if (rec) return resident ? occ_b<true, true>() : occ_b<true, false>();
    return resident ? occ_b<false, true>() : occ_b<false, false>();
}

cudaError_t launch_build_masks(const MaskInputs &in, uint32_t *out, cudaStream_t st)
{
    if (in.total_words <= 0) return cudaSuccess;
    const int64_t blocks = (in.total_words + 255) / 256;
    if (blocks > 0x7fffffff) return cudaErrorInvalidValue;
    build_masks_kernel<<<(unsigned)blocks, 256, 0, st>>>(in, out);
    return cudaGetLastError();
}

int batched_tile() { return kBatchTile; }

}  // namespace rf
