// Kernel instantiations for the S2o2 stencil shape (one translation unit per
// shape so the build compiles them in parallel).
#include "solver_kernels.cuh"

namespace zfvm {
namespace dev {
ZFVM_DEFINE_SHAPE(s2o2, S2o2)
}  // namespace dev
}  // namespace zfvm
