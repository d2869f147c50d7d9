// Kernel instantiations for the S2o3 stencil shape (one translation unit per
// shape so the build compiles them in parallel).
#include "solver_kernels.cuh"

namespace zfvm {
namespace dev {
ZFVM_DEFINE_SHAPE(s2o3, S2o3)
}  // namespace dev
}  // namespace zfvm
