// Mixed-precision lattice kernels: FP32 arithmetic, f-bar stored in FP32,
// BF16 (round to nearest or stochastic rounding) or FP16.  Compiled with FMA contraction.
#include "launchers.cuh"

namespace plbgpu {
const Launchers& launchersFp32() { return LaunchImpl<float>::table(); }
const Launchers& launchersBf16() { return LaunchImpl<__nv_bfloat16>::table(); }
const Launchers& launchersFp16() { return LaunchImpl<__half>::table(); }
const Launchers& launchersBf16Sr() { return LaunchImpl<bf16sr>::table(); }
}  // namespace plbgpu
