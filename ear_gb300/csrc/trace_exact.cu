// trace_exact.cu -- "exact" instantiation of the trace kernels.
// Compiled with --fmad=false: every operation rounds as the CPU restatement's does, so hit indices, bounce types and splat values match it bit for bit.
#define EAR_NS exact
#include "trace_impl.cuh"
#include "trace_launch.cuh"

namespace ear {
const TraceOps kTraceExact = exact::kOps;
}  // namespace ear
