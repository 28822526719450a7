// rf_kern_fast.cu -- single-scene kernels with the FP32 hardware
// approximations (the counterparts of OpenCL native_*), compiled with the
// default contraction of products and sums into FMA.
#include "rf_trace_kernels.cuh"
#include "rf_batched.cuh"
#include "rf_mixed_small.cuh"

namespace rf {
template cudaError_t launch_trace<MFast>(const LaunchCfg &, const TraceParams &, cudaStream_t);
template int trace_blocks_per_sm<MFast>(const LaunchCfg &);

static_assert(kBatchThreads * kBatchDraws == kBatchChunkDraws, "chunk size");
static_assert(kBatchThreads == kBatchBlock, "block size");

size_t batched_smem_bytes() { return sizeof(BatchSmem); }

static_assert(sizeof(BatchSmem) <= 227 * 1024, "the batched kernel's shared memory exceeds a block's 227 KB");

template <bool REC, bool RES, bool CNT, bool BV = false>
static cudaError_t launch_b(const TraceParams &p, int grid, cudaStream_t st)
{
    const size_t smem = sizeof(BatchSmem);
    auto k = batched_kernel<REC, RES, CNT, BV>;
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

cudaError_t launch_batched_bv(const TraceParams &p, bool rec, bool count, int grid, cudaStream_t st)
{
    if (p.nbv <= 0 || p.nbv > kBatchMaxBV || p.n > kBatchTile) return cudaErrorInvalidValue;
    if (rec) return launch_b<true, true, false, true>(p, grid, st);
    return count ? launch_b<false, true, true, true>(p, grid, st) : launch_b<false, true, false, true>(p, grid, st);
}

template <bool REC, bool RES>
static int occ_b()
{
    const size_t smem = sizeof(BatchSmem);
    int nb = 0;
    auto k = batched_kernel<REC, RES, false, false>;
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

template <int GPT, bool REC>
static int occ_s()
{
    int nb = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, mixed_small_kernel<GPT, REC>, kSmallThreads, 0);
    return nb;
}

int mixed_small_blocks_per_sm(int gpt, bool rec)
{
    if (rec) return occ_s<1, true>();
    return gpt == 2 ? occ_s<2, false>() : occ_s<1, false>();
}

}  // namespace rf
