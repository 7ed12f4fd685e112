// FP64 instantiation of the hot-path kernels (the plain method).  Compiled
// with --fmad=false: no multiply-add contraction, so the arithmetic is
// rounded exactly as the serial Fortran evaluates it.
#include "fvm_kernels_impl.cuh"

namespace fvm {
FVM_DEFINE_LAUNCHERS(double)
}  // namespace fvm
