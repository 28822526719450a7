// rf_kern_batched.cu -- launchers of the batched mixed-precision persistent
// kernel (every instantiation: record / resident / counting / bounding-surface /
// segment-stack variants) and of the cell-mask builder.
#include "rf_trace_kernels.cuh"
#include "rf_batched.cuh"

namespace rf {

static_assert(kBatchThreads * kBatchDraws == kBatchChunkDraws, "chunk size");
static_assert(kBatchThreads == kBatchBlock, "block size");

size_t batched_smem_bytes() { return sizeof(BatchSmem); }

static_assert(sizeof(BatchSmem) <= 227 * 1024, "the batched kernel's shared memory exceeds a block's 227 KB");

template <bool REC, bool RES, bool CNT, bool BV, bool STK>
static cudaError_t launch_k(const TraceParams &p, int grid, cudaStream_t st)
{
    const size_t smem = sizeof(BatchSmem);
    auto k = batched_kernel<REC, RES, CNT, BV, STK>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k<<<grid, kBatchThreads, smem, st>>>(p);
    return cudaGetLastError();
}

template <bool BV, bool STK>
static cudaError_t launch_b(const TraceParams &p, bool rec, bool resident, bool count, int grid, cudaStream_t st)
{
    if constexpr (BV) {  // one resident scene
        if (rec) return launch_k<true, true, false, true, STK>(p, grid, st);
        return count ? launch_k<false, true, true, true, STK>(p, grid, st)
                     : launch_k<false, true, false, true, STK>(p, grid, st);
    } else {
        if (rec)
            return resident ? launch_k<true, true, false, false, STK>(p, grid, st)
                            : launch_k<true, false, false, false, STK>(p, grid, st);
        if (count)
            return resident ? launch_k<false, true, true, false, STK>(p, grid, st)
                            : launch_k<false, false, true, false, STK>(p, grid, st);
        return resident ? launch_k<false, true, false, false, STK>(p, grid, st)
                        : launch_k<false, false, false, false, STK>(p, grid, st);
    }
}

cudaError_t launch_batched(const TraceParams &p, bool rec, bool resident, bool count, bool stacks, int grid,
                           cudaStream_t st)
{
    return stacks ? launch_b<false, true>(p, rec, resident, count, grid, st)
                  : launch_b<false, false>(p, rec, resident, count, grid, st);
}

cudaError_t launch_batched_bv(const TraceParams &p, bool rec, bool count, bool stacks, int grid, cudaStream_t st)
{
    if (p.nbv <= 0 || p.nbv > kBatchMaxBV || p.n > kBatchTile) return cudaErrorInvalidValue;
    return stacks ? launch_b<true, true>(p, rec, true, count, grid, st) : launch_b<true, false>(p, rec, true, count, grid, st);
}

// Resident blocks per SM, queried once per process (every GPU of a run is the same
// part): the query costs microseconds on each launch otherwise.
template <bool REC, bool RES>
static int occ_b()
{
    static const int nb = [] {
        const size_t smem = sizeof(BatchSmem);
        int r = 0;
        auto k = batched_kernel<REC, RES, false, false, false>;
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, k, kBatchThreads, smem) != cudaSuccess) r = 0;
        return r;
    }();
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
