// trace_fast.cu -- "fast" instantiation of the trace kernels.
// Compiled with FMA contraction allowed: statistically identical output, faster arithmetic; not bit-exact with the CPU restatement.
#define EAR_NS fast
#include "trace_impl.cuh"

namespace ear {
namespace {

template <int MODE>
cudaError_t launch(const TraceArgs& a, int grid, size_t smem, cudaStream_t s) {
  cudaFuncSetAttribute(fast::trace_kernel<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)smem);
  fast::trace_kernel<MODE><<<grid, fast::kTraceBlock, smem, s>>>(a);
  return cudaGetLastError();
}

template <int MODE>
cudaError_t occupancy(size_t smem, int* blocks_per_sm) {
  cudaFuncSetAttribute(fast::trace_kernel<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)smem);
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, fast::trace_kernel<MODE>,
                                                       fast::kTraceBlock, smem);
}

cudaError_t trace_fast(const TraceArgs& a, int grid, size_t smem, int mode, cudaStream_t s) {
  if (mode == kModeDebug) return launch<kModeDebug>(a, grid, smem, s);
  if (mode == kModeAdjoint) return launch<kModeAdjoint>(a, grid, smem, s);
  return launch<kModeForward>(a, grid, smem, s);
}

cudaError_t occupancy_fast(int mode, size_t smem, int* blocks_per_sm) {
  if (mode == kModeDebug) return occupancy<kModeDebug>(smem, blocks_per_sm);
  if (mode == kModeAdjoint) return occupancy<kModeAdjoint>(smem, blocks_per_sm);
  return occupancy<kModeForward>(smem, blocks_per_sm);
}

}  // namespace

const TraceOps kTraceFast = {trace_fast, occupancy_fast, fast::kTraceBlock};

}  // namespace ear
