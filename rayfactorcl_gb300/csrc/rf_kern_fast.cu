// rf_kern_fast.cu -- single-scene kernels with the FP32 hardware
// approximations (the counterparts of OpenCL native_*), compiled with the
// default contraction of products and sums into FMA.
#include "rf_trace_kernels.cuh"

namespace rf {
template cudaError_t launch_trace<MFast>(const LaunchCfg &, const TraceParams &, cudaStream_t);
template int trace_blocks_per_sm<MFast>(const LaunchCfg &);
}  // namespace rf
