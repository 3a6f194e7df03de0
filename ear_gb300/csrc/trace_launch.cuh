// trace_launch.cuh -- host launchers of one trace-kernel instantiation.
// Included at the end of trace_exact.cu / trace_fast.cu after trace_impl.cuh
// with EAR_NS naming the instantiation; defines ear::EAR_NS::kOps.
#pragma once

namespace ear {
namespace EAR_NS {
namespace {

template <int MODE>
cudaError_t launch(const TraceArgs& a, int grid, int block, size_t smem, cudaStream_t s) {
  if (block <= 0 || block > kTraceMaxBlock || block % 32) return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(trace_kernel<MODE>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  trace_kernel<MODE><<<grid, block, smem, s>>>(a);
  return cudaGetLastError();
}

template <int MODE>
cudaError_t occupancy(int block, size_t smem, int* blocks_per_sm) {
  cudaError_t e = cudaFuncSetAttribute(trace_kernel<MODE>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, trace_kernel<MODE>, block,
                                                       smem);
}

cudaError_t trace(const TraceArgs& a, int grid, int block, size_t smem, int mode, cudaStream_t s) {
  switch (mode) {
    case kModeDebug: return launch<kModeDebug>(a, grid, block, smem, s);
    case kModeAdjoint: return launch<kModeAdjoint>(a, grid, block, smem, s);
    case kModeBatch: return launch<kModeBatch>(a, grid, block, smem, s);
    default: return launch<kModeForward>(a, grid, block, smem, s);
  }
}

cudaError_t occ(int mode, int block, size_t smem, int* blocks_per_sm) {
  switch (mode) {
    case kModeDebug: return occupancy<kModeDebug>(block, smem, blocks_per_sm);
    case kModeAdjoint: return occupancy<kModeAdjoint>(block, smem, blocks_per_sm);
    case kModeBatch: return occupancy<kModeBatch>(block, smem, blocks_per_sm);
    default: return occupancy<kModeForward>(block, smem, blocks_per_sm);
  }
}

cudaError_t probe(const TraceArgs& a, int n, unsigned* blocked, cudaStream_t s) {
  occlusion_probe_kernel<<<(n + 255) / 256, 256, 0, s>>>(a, n, blocked);
  return cudaGetLastError();
}

}  // namespace

const TraceOps kOps = {trace, occ, probe, kTraceMaxBlock};

}  // namespace EAR_NS
}  // namespace ear
