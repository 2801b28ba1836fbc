// Mixed-precision lattice kernels, BF16 storage, round to nearest: FP32 arithmetic, compiled with
// FMA contraction.  One storage type per translation unit so that the forms
// compile in parallel.
#include "launchers.cuh"

namespace plbgpu {
const Launchers& launchersBf16() { return LaunchImpl<__nv_bfloat16>::table(); }
}  // namespace plbgpu
