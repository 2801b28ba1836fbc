// Time step of the bf16sr storage form, odd AA parity (see step_parity.cuh).
#include "step_parity.cuh"

namespace plbgpu {
template int stepParity<bf16sr, true>(const DevLattice&, bool, const StepParams<StoreT<bf16sr>::R>&, StatsAcc*,
                                        cudaStream_t, const SideStream*);
template int slabParity<bf16sr, true>(const DevLattice&, bool, const StepParams<StoreT<bf16sr>::R>&, StatsAcc*, int,
                                      int, cudaStream_t, const SideStream*);
}  // namespace plbgpu
