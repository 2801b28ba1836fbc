// Time step of the fp32 storage form, even AA parity (see step_parity.cuh).
#include "step_parity.cuh"

namespace plbgpu {
template int stepParity<float, false>(const DevLattice&, bool, const StepParams<StoreT<float>::R>&, StatsAcc*,
                                        cudaStream_t, const SideStream*);
template int slabParity<float, false>(const DevLattice&, bool, const StepParams<StoreT<float>::R>&, StatsAcc*, int,
                                      int, cudaStream_t, const SideStream*);
}  // namespace plbgpu
