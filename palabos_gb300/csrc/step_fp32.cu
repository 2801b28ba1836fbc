// Mixed-precision lattice kernels, FP32 storage: FP32 arithmetic, compiled with
// FMA contraction.  One storage type per translation unit so that the forms
// compile in parallel.
#include "launchers.cuh"

namespace plbgpu {
const Launchers& launchersFp32() { return LaunchImpl<float>::table(); }
}  // namespace plbgpu
