// Numerical fluxes and the ghost-cell boundary condition as standalone device
// calls, for callers that keep the reference's own loops around the GPU
// kernels' arithmetic:
//   zfvm_numerical_flux   HLLCBatten::flux (flux/hllc.hpp:142-176) or the
//                         Rusanov flux for n face states, with their wave speeds
//   zfvm_tracer_flux      HLLCBatten::tracer_flux (flux/hllc.hpp:178-197) or the
//                         Rusanov flux of an advected variable
//   zfvm_apply_boundary   BoundaryCondition::apply (boundary/boundary_condition.hpp:12-21)
//                         with the solver's ghost cells: FrozenBC rows
//                         (boundary/frozen_boundary_condition.cpp:39-55) and
//                         periodic images
// Each call is one batched launch over host arrays on its own stream (device
// scratch is allocated for the call); the face kernels of the solver evaluate
// the same device functions.
#include <cuda_runtime.h>

#include <string>

#include "solver_obj.hpp"

using namespace zfvm;
using namespace zfvm::dev;

namespace {

constexpr int kNV = 5;  // rho, normal momentum, two tangential momenta, E

__global__ void k_numerical_flux(int kind, double gamma, int64_t n, const double *uL, const double *uR, double *f,
                                 double *speeds) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double a[kNV], b[kNV], nf[kNV];
  for (int k = 0; k < kNV; ++k) a[k] = uL[i * kNV + k], b[k] = uR[i * kNV + k];
  double s0, s1, s2;
  if (kind == ZFVM_FLUX_HLLC) {
    const HllcWaves<double> w = hllc_waves<kNV>(a, b, gamma);
    hllc_flux<kNV>(a, b, gamma, nf);
    s0 = w.sL, s1 = w.s_star, s2 = w.sR;
  } else {
    rusanov_flux<kNV>(a, b, gamma, nf);
    // the symmetric fan of the local Lax-Friedrichs flux
    const double sm = rusanov_speed<kNV>(a, b, gamma);
    s0 = -sm, s1 = 0.0, s2 = sm;
  }
  for (int k = 0; k < kNV; ++k) f[i * kNV + k] = nf[k];
  if (speeds) speeds[3 * i] = s0, speeds[3 * i + 1] = s1, speeds[3 * i + 2] = s2;
}

__global__ void k_tracer_flux(int kind, int64_t n, const double *uL, const double *uR, const double *mqL,
                              const double *mqR, const double *speeds, double *f) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double vL = uL[i * kNV + 1] / uL[i * kNV], vR = uR[i * kNV + 1] / uR[i * kNV];
  if (kind == ZFVM_FLUX_HLLC) {
    HllcWaves<double> w{};
    w.vL = vL, w.vR = vR;
    w.sL = speeds[3 * i], w.s_star = speeds[3 * i + 1], w.sR = speeds[3 * i + 2];
    f[i] = hllc_tracer_flux(w, mqL[i], mqR[i]);
  } else {
    f[i] = rusanov_tracer_flux(speeds[3 * i + 2], vL, vR, mqL[i], mqR[i]);
  }
}

// Ghost rows: a frozen cell (its own source) takes its frozen row, a periodic
// image its source's row; interior rows stay.  Rows are the reference's
// cell-major (rho, m1, m2, m3, E) and n_avars-wide avars.
__global__ void k_apply_boundary(int n, const uint8_t *flags, const int *source, const double *frozen,
                                 const double *frozen_q, const double *in, const double *in_q, double *out,
                                 double *out_q, int na) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const bool ghost = flags[i] & kGhost;
  const int j = source[i];
  const bool frozen_row = ghost && j == i;
  for (int k = 0; k < 5; ++k) {
    const double x = frozen_row ? (frozen ? frozen[(size_t)i * 5 + k] : in[(size_t)i * 5 + k]) : in[(size_t)j * 5 + k];
    out[(size_t)i * 5 + k] = x;
  }
  for (int t = 0; t < na; ++t) {
    const double x =
        frozen_row ? (frozen_q ? frozen_q[(size_t)i * na + t] : in_q[(size_t)i * na + t]) : in_q[(size_t)j * na + t];
    out_q[(size_t)i * na + t] = x;
  }
}

struct Stream {
  cudaStream_t s = nullptr;
  Stream() { CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)); }
  ~Stream() {
    if (s) {
      cudaStreamSynchronize(s);
      cudaStreamDestroy(s);
    }
  }
};

template <class T>
void upload_async(DBuf<T> &b, const T *h, size_t n, cudaStream_t s) {
  b.alloc(n);
  if (n) CK(cudaMemcpyAsync(b.p, h, n * sizeof(T), cudaMemcpyHostToDevice, s));
}

}  // namespace

extern "C" int zfvm_numerical_flux(int32_t flux, double gamma, int64_t n, const double *uL, const double *uR,
                                   double *flux_out, double *speeds) {
  if (flux != ZFVM_FLUX_HLLC && flux != ZFVM_FLUX_RUSANOV) return fail(ZFVM_EINVAL, "unknown flux");
  if (!(gamma > 1.0)) return fail(ZFVM_EINVAL, "gamma must exceed 1");
  if (n < 0 || (n > 0 && (!uL || !uR || !flux_out))) return fail(ZFVM_EINVAL, "null argument");
  if (n == 0) return ZFVM_OK;
  SOLVER_GUARD_BEGIN
  Stream st;
  DBuf<double> a, b, f, sp;
  upload_async(a, uL, (size_t)n * kNV, st.s);
  upload_async(b, uR, (size_t)n * kNV, st.s);
  f.alloc((size_t)n * kNV);
  sp.alloc((size_t)n * 3);
  k_numerical_flux<<<(unsigned)((n + 127) / 128), 128, 0, st.s>>>(flux, gamma, n, a.p, b.p, f.p, sp.p);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(flux_out, f.p, (size_t)n * kNV * sizeof(double), cudaMemcpyDeviceToHost, st.s));
  if (speeds) CK(cudaMemcpyAsync(speeds, sp.p, (size_t)n * 3 * sizeof(double), cudaMemcpyDeviceToHost, st.s));
  CK(cudaStreamSynchronize(st.s));
  return ZFVM_OK;
  SOLVER_GUARD_END
}

extern "C" int zfvm_tracer_flux(int32_t flux, int64_t n, const double *uL, const double *uR, const double *mqL,
                                const double *mqR, const double *speeds, double *flux_out) {
  if (flux != ZFVM_FLUX_HLLC && flux != ZFVM_FLUX_RUSANOV) return fail(ZFVM_EINVAL, "unknown flux");
  if (n < 0 || (n > 0 && (!uL || !uR || !mqL || !mqR || !speeds || !flux_out))) return fail(ZFVM_EINVAL, "null argument");
  if (n == 0) return ZFVM_OK;
  SOLVER_GUARD_BEGIN
  Stream st;
  DBuf<double> a, b, qa, qb, sp, f;
  upload_async(a, uL, (size_t)n * kNV, st.s);
  upload_async(b, uR, (size_t)n * kNV, st.s);
  upload_async(qa, mqL, (size_t)n, st.s);
  upload_async(qb, mqR, (size_t)n, st.s);
  upload_async(sp, speeds, (size_t)n * 3, st.s);
  f.alloc((size_t)n);
  k_tracer_flux<<<(unsigned)((n + 127) / 128), 128, 0, st.s>>>(flux, n, a.p, b.p, qa.p, qb.p, sp.p, f.p);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(flux_out, f.p, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, st.s));
  CK(cudaStreamSynchronize(st.s));
  return ZFVM_OK;
  SOLVER_GUARD_END
}

extern "C" int zfvm_apply_boundary(zfvm_solver *s, const double *frozen_cvars, const double *frozen_avars,
                                   double *cvars, double *avars) {
  if (!s || !cvars || (s->na && !avars)) return fail(ZFVM_EINVAL, "null argument");
  SOLVER_GUARD_BEGIN
  const size_t n = (size_t)s->n_cells, na = (size_t)s->na;
  DBuf<double> in, out, fz, qin, qout, fzq;
  upload_async(in, cvars, n * 5, s->stream);
  out.alloc(n * 5);
  if (frozen_cvars) upload_async(fz, frozen_cvars, n * 5, s->stream);
  if (na) {
    upload_async(qin, avars, n * na, s->stream);
    qout.alloc(n * na);
    if (frozen_avars) upload_async(fzq, frozen_avars, n * na, s->stream);
  }
  k_apply_boundary<<<(unsigned)((n + 127) / 128), 128, 0, s->stream>>>((int)n, s->flags.p, s->src_map.p, fz.p, fzq.p,
                                                                       in.p, qin.p, out.p, qout.p, (int)na);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(cvars, out.p, n * 5 * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  if (na) CK(cudaMemcpyAsync(avars, qout.p, n * na * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  return ZFVM_OK;
  SOLVER_GUARD_END
}
