// FP32 instantiation of the hot-path kernels: state, reconstruction,
// fluxes and RK stages in FP32; geometry, residual norm and forces in FP64.
#include "fvm_kernels_impl.cuh"

namespace fvm {
FVM_DEFINE_LAUNCHERS(float)
}  // namespace fvm
