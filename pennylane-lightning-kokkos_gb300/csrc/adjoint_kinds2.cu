// adjoint_kinds2.cu — fused adjoint backward-step launchers for the two-wire
// gate kinds (the kernels are in adjoint_kernels.cuh; this
// translation unit exists so that they compile in parallel with adjoint.cu).
#include "adjoint_kernels.cuh"

namespace plk {

#define PLK_ADJ_INST(K)                                                                                               \
    template int launch_fused_kind<float, K>(plk_state, c2_t<float> *const *, int, int, const AdjArgs<float> &,           \
                                             double *, double);                                                        \
    template int launch_fused_kind<double, K>(plk_state, c2_t<double> *const *, int, int, const AdjArgs<double> &,        \
                                              double *, double);
PLK_ADJ_KINDS2(PLK_ADJ_INST)
#undef PLK_ADJ_INST

} // namespace plk
