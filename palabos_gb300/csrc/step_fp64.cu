// FP64 lattice kernels.  Compiled with --fmad=false: every multiply and add is
// rounded separately, in the reference's order, so the device reproduces the
// reference CPU path bit for bit.
#include "launchers.cuh"

namespace plbgpu {
const Launchers& launchersFp64() { return LaunchImpl<double>::table(); }
}  // namespace plbgpu
