// trace_exact.cu -- "exact" instantiation of the trace kernels.
// Compiled with --fmad=false: every operation rounds as the CPU restatement's does, so hit indices, bounce types and splat values match it bit for bit.
#define EAR_NS exact
#include "trace_impl.cuh"

namespace ear {
namespace {

template <int MODE>
cudaError_t launch(const TraceArgs& a, int grid, size_t smem, cudaStream_t s) {
  cudaFuncSetAttribute(exact::trace_kernel<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)smem);
  exact::trace_kernel<MODE><<<grid, exact::kTraceBlock, smem, s>>>(a);
  return cudaGetLastError();
}

template <int MODE>
cudaError_t occupancy(size_t smem, int* blocks_per_sm) {
  cudaFuncSetAttribute(exact::trace_kernel<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)smem);
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, exact::trace_kernel<MODE>,
                                                       exact::kTraceBlock, smem);
}

cudaError_t trace_exact(const TraceArgs& a, int grid, size_t smem, int mode, cudaStream_t s) {
  if (mode == kModeDebug) return launch<kModeDebug>(a, grid, smem, s);
  if (mode == kModeAdjoint) return launch<kModeAdjoint>(a, grid, smem, s);
  return launch<kModeForward>(a, grid, smem, s);
}

cudaError_t occupancy_exact(int mode, size_t smem, int* blocks_per_sm) {
  if (mode == kModeDebug) return occupancy<kModeDebug>(smem, blocks_per_sm);
  if (mode == kModeAdjoint) return occupancy<kModeAdjoint>(smem, blocks_per_sm);
  return occupancy<kModeForward>(smem, blocks_per_sm);
}

}  // namespace

const TraceOps kTraceExact = {trace_exact, occupancy_exact, exact::kTraceBlock};

}  // namespace ear
