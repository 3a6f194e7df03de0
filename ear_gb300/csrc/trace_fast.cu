// trace_fast.cu -- "fast" instantiation of the trace kernels.
// Compiled with FMA contraction and approximate division allowed, powers on
// the special-function unit: statistically identical output, faster
// arithmetic; not bit-exact with the CPU restatement.
#define EAR_NS fast
#define EAR_FAST_TRIANGLE_TEST 1
#define EAR_FAST_MATH 1
#include "trace_impl.cuh"
#include "trace_launch.cuh"

namespace ear {
const TraceOps kTraceFast = fast::kOps;
}  // namespace ear
