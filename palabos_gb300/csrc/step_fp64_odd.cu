// Time step of the fp64 storage form, odd AA parity (see step_parity.cuh).
#include "step_parity.cuh"

namespace plbgpu {
template int stepParity<double, true>(const DevLattice&, bool, const StepParams<StoreT<double>::R>&, StatsAcc*,
                                        cudaStream_t, const SideStream*);
template int slabParity<double, true>(const DevLattice&, bool, const StepParams<StoreT<double>::R>&, StatsAcc*, int,
                                      int, cudaStream_t, const SideStream*);
}  // namespace plbgpu
