// Mixed-precision lattice kernels, FP16 storage: FP32 arithmetic, compiled with
// FMA contraction.  One storage type per translation unit so that the forms
// compile in parallel.
#include "launchers.cuh"

namespace plbgpu {
const Launchers& launchersFp16() { return LaunchImpl<__half>::table(); }
}  // namespace plbgpu
