// Kernel instantiations for the S3o2 stencil shape (one translation unit per
// shape so the build compiles them in parallel).
#include "solver_kernels.cuh"

namespace zfvm {
namespace dev {
ZFVM_DEFINE_SHAPE(s3o2, S3o2)
}  // namespace dev
}  // namespace zfvm
