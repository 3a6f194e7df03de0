// trace_fast.cu -- "fast" instantiation of the trace kernels.
// Compiled with FMA contraction allowed: statistically identical output, faster arithmetic; not bit-exact with the CPU restatement.
#define EAR_NS fast
#include "trace_impl.cuh"

namespace ear {
namespace {

cudaError_t trace_fast(const TraceArgs& a, int grid, size_t smem, bool debug, cudaStream_t s) {
  if (debug) {
    cudaFuncSetAttribute(fast::trace_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
    fast::trace_kernel<true><<<grid, fast::kTraceBlock, smem, s>>>(a);
  } else {
    cudaFuncSetAttribute(fast::trace_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
    fast::trace_kernel<false><<<grid, fast::kTraceBlock, smem, s>>>(a);
  }
  return cudaGetLastError();
}

cudaError_t occupancy_fast(bool debug, size_t smem, int* blocks_per_sm) {
  if (debug) {
    cudaFuncSetAttribute(fast::trace_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, fast::trace_kernel<true>,
                                                         fast::kTraceBlock, smem);
  }
  cudaFuncSetAttribute(fast::trace_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)smem);
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, fast::trace_kernel<false>,
                                                       fast::kTraceBlock, smem);
}

}  // namespace

const TraceOps kTraceFast = {trace_fast, occupancy_fast, fast::kTraceBlock};

}  // namespace ear
