// The step kernels compiled with -use_fast_math (FMA contraction,
// approximate division and square root): aqua::fast.  Same source as the
// exact kernels (step_kernels.cuh); results stay within the 1e-5 relative
// tolerance of the reference's per-step rates (tests/test_gpu_fast.py).
#include "aqua_internal.cuh"
#include "kernels.cuh"

namespace aqua {
namespace fast {
#define AQUA_FAST_ARITH 1
#include "step_kernels.cuh"
#undef AQUA_FAST_ARITH
}  // namespace fast
}  // namespace aqua
