// Kernel instantiations for one stencil shape, one precision and either the
// single-solver kernels or the batched kernels of one block size.  The build
// compiles this file once per combination (ZFVM_SHAPE_NAME, ZFVM_SHAPE,
// ZFVM_MIXED, ZFVM_BATCH = 0 or the batch block size, set on the command
// line), so the kernel sets compile in parallel.
#include "solver_kernels.cuh"

#if !defined(ZFVM_SHAPE_NAME) || !defined(ZFVM_SHAPE) || !defined(ZFVM_MIXED) || !defined(ZFVM_BATCH)
#error "inst_shape.cu needs ZFVM_SHAPE_NAME, ZFVM_SHAPE, ZFVM_MIXED and ZFVM_BATCH"
#endif

// one level of indirection so the -D names expand before the macros paste them
#define ZFVM_SINGLE_X(n, S, M, sfx) ZFVM_DEFINE_SHAPE_SINGLE(n, S, M, sfx)
#define ZFVM_CFL_X(n, S) ZFVM_DEFINE_SHAPE_CFL(n, S)
#define ZFVM_BATCH_X(n, S, M, sfx, bs) ZFVM_DEFINE_SHAPE_BATCH(n, S, M, sfx, bs)

namespace zfvm {
namespace dev {
#if ZFVM_MIXED
#define ZFVM_SFX mix
#else
#define ZFVM_SFX f64
#endif
#if ZFVM_BATCH
ZFVM_BATCH_X(ZFVM_SHAPE_NAME, ZFVM_SHAPE, (ZFVM_MIXED != 0), ZFVM_SFX, ZFVM_BATCH)
#else
ZFVM_SINGLE_X(ZFVM_SHAPE_NAME, ZFVM_SHAPE, (ZFVM_MIXED != 0), ZFVM_SFX)
#if !ZFVM_MIXED
ZFVM_CFL_X(ZFVM_SHAPE_NAME, ZFVM_SHAPE)
#endif
#endif
}  // namespace dev
}  // namespace zfvm
