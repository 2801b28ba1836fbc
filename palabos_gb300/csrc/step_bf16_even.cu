// Time step of the bf16 storage form, even AA parity (see step_parity.cuh).
#include "step_parity.cuh"

namespace plbgpu {
template int stepParity<__nv_bfloat16, false>(const DevLattice&, bool, const StepParams<StoreT<__nv_bfloat16>::R>&, StatsAcc*,
                                        cudaStream_t, const SideStream*);
template int slabParity<__nv_bfloat16, false>(const DevLattice&, bool, const StepParams<StoreT<__nv_bfloat16>::R>&, StatsAcc*, int,
                                      int, cudaStream_t, const SideStream*);
}  // namespace plbgpu
