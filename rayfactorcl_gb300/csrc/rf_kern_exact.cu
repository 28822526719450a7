// rf_kern_exact.cu -- single-scene kernels with the IEEE FP32 op mapping
// (bit-exact with the CPU restatement) and in FP64.  Compiled with
// -fmad=false: a product followed by a sum in the source stays two roundings.
#include "rf_trace_kernels.cuh"

namespace rf {
template cudaError_t launch_trace<MExact>(const LaunchCfg &, const TraceParams &, cudaStream_t);
template int trace_blocks_per_sm<MExact>(const LaunchCfg &);
template cudaError_t launch_trace<MF64>(const LaunchCfg &, const TraceParams &, cudaStream_t);
template int trace_blocks_per_sm<MF64>(const LaunchCfg &);
}  // namespace rf
