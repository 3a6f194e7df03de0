// trace_exact.cu -- "exact" instantiation of the trace kernels.
// Compiled with --fmad=false: every operation rounds as the CPU restatement's does, so hit indices, bounce types and splat values match it bit for bit.
#define EAR_NS exact
#include "trace_impl.cuh"

namespace ear {
namespace {

cudaError_t trace_exact(const TraceArgs& a, int grid, size_t smem, bool debug, cudaStream_t s) {
  if (debug) {
    cudaFuncSetAttribute(exact::trace_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
    exact::trace_kernel<true><<<grid, exact::kTraceBlock, smem, s>>>(a);
  } else {
    cudaFuncSetAttribute(exact::trace_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
    exact::trace_kernel<false><<<grid, exact::kTraceBlock, smem, s>>>(a);
  }
  return cudaGetLastError();
}

cudaError_t occupancy_exact(bool debug, size_t smem, int* blocks_per_sm) {
  if (debug) {
    cudaFuncSetAttribute(exact::trace_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, exact::trace_kernel<true>,
                                                         exact::kTraceBlock, smem);
  }
  cudaFuncSetAttribute(exact::trace_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)smem);
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, exact::trace_kernel<false>,
                                                       exact::kTraceBlock, smem);
}

}  // namespace

const TraceOps kTraceExact = {trace_exact, occupancy_exact, exact::kTraceBlock};

}  // namespace ear
