// Kernel instantiations for the S3o3 stencil shape (one translation unit per
// shape so the build compiles them in parallel).
#include "solver_kernels.cuh"

namespace zfvm {
namespace dev {
ZFVM_DEFINE_SHAPE(s3o3, S3o3)
}  // namespace dev
}  // namespace zfvm
