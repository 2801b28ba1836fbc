// Mixed-precision lattice kernels, BF16 storage with stochastic rounding: FP32 arithmetic, compiled with
// FMA contraction.  One storage type per translation unit so that the forms
// compile in parallel.
#include "launchers.cuh"

namespace plbgpu {
const Launchers& launchersBf16Sr() { return LaunchImpl<bf16sr>::table(); }
}  // namespace plbgpu
