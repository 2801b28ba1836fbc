// Time step of the fp16 storage form, odd AA parity (see step_parity.cuh).
#include "step_parity.cuh"

namespace plbgpu {
template int stepParity<__half, true>(const DevLattice&, bool, const StepParams<StoreT<__half>::R>&, StatsAcc*,
                                        cudaStream_t, const SideStream*);
template int slabParity<__half, true>(const DevLattice&, bool, const StepParams<StoreT<__half>::R>&, StatsAcc*, int,
                                      int, cudaStream_t, const SideStream*);
}  // namespace plbgpu
