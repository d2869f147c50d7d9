// Device kernels of the GB300 rate-of-change and SSP-RK time stepping.
//
// One Runge-Kutta stage is three kernels:
//   k_reconstruct  one thread per cell: gather the stencil cell averages, the
//                  (optional) local hydrostatic equilibrium, CWENO-AO
//                  combination of the LSQ polynomials, evaluation at the
//                  cell's face quadrature points and the gravity source.
//   k_face_flux    one thread per face: numerical flux (HLLC / Rusanov) from
//                  the two face-point values, or the boundary flux.
//   k_update       one thread per cell: signed gather of the face fluxes,
//                  RK stage combination, CFL candidate of the new state.
// A one-thread k_clock kernel opens every step: it turns the CFL minimum of the
// previous step into dt, clips it to t_end and stops the loop when done, so the
// whole time loop runs from a CUDA graph without host round trips.
//
// The arithmetic is the reference's (ZisaFVM: reconstruction/cweno_ao.cpp,
// hybrid_weno.cpp, fvm_loops/flux_loop.hpp, gravity_source_loop.hpp,
// ode/runge_kutta.cpp, model/local_cfl_condition_impl.hpp), rearranged for the
// GPU: the LSQ solve uses a pseudo-inverse built on the host, the stencil values
// are reconstructed unscaled and the EulerScaling enters only the smoothness
// indicators, and the face-flux scatter is a deterministic cell-centric gather
// instead of OpenMP atomics.
//
// Two precisions share the kernels (template flag MIXED):
//   FP64   everything in double.
//   MIXED  the cell averages, the equilibrium (Newton solve, equilibrium
//          averages and point values), the RK accumulation and the CFL time
//          step stay FP64; the reconstruction of the deviation from the
//          equilibrium, the smoothness indicators / nonlinear weights and the
//          numerical flux run in FP32.  The flux is computed in deviation form
//          around the left cell's FP64 face state w:
//            F = F64(w) + [F32(w + dL, w + dR) - F32(w)],
//          which is exact in exact arithmetic (both fluxes are consistent) and
//          gives an exactly zero FP32 part on an unperturbed equilibrium.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <type_traits>

#include "grid.hpp"
#include "physics.cuh"

namespace zfvm {
namespace dev {

enum StatusBits : int { kStNonPhysical = 1, kStNewton = 2, kStNonFinite = 4 };

struct Clock {
  double t, dt, t_end, fixed_dt;
  unsigned long long cfl_min;  // bits of a positive double
  long long step, n_steps;
  int done, started, status, pad;
  // RejectLargeDensityChange (ode/step_rejection.cpp:17-56); reject_drho = 0
  // rejects nothing.  factor scales the CFL step; a rejected step is redone
  // from its saved start with factor * dt.
  double reject_drho, factor, min_factor;
  int rejected, good_prev, restore, retry;
  long long n_rejected;
};

// Close the running step and open the next one (mode 0) or only close it
// (mode 1): the TimeLoop of fvm_loops/time_loop.cpp:36-81 on the device clock.
__device__ __forceinline__ void clock_step(Clock *c, double cfl, int mode) {
  if (c->started) {
    c->started = 0;
    if (c->rejected) {
      // RejectLargeDensityChange::check (bad step) + TimeLoop::reject_step
      c->rejected = 0;
      c->good_prev = 0;
      c->factor = fmax(c->min_factor, fmin(0.5 * c->factor, 1.0));
      c->dt = c->factor * c->dt;
      c->retry = 1;
      c->restore = 1;
      c->n_rejected += 1;
    } else {
      c->t += c->dt;
      c->step += 1;
      c->restore = 0;
      if (c->reject_drho > 0.0) {
        if (c->good_prev) c->factor = fmax(c->min_factor, fmin(2.0 * c->factor, 1.0));
        c->good_prev = 1;
      }
    }
  } else {
    c->restore = 0;
  }
  if (mode == 1 || c->done) return;
  bool fin = (c->n_steps > 0 && c->step >= c->n_steps) ||
             (c->t_end > 0.0 && c->t_end - c->t <= 1e-12 * c->t_end) || c->status != 0;
  if (fin) {
    c->done = 1;
    return;
  }
  double dt;
  if (c->retry) {
    dt = c->dt;
    c->retry = 0;
  } else {
    dt = c->fixed_dt > 0.0 ? c->fixed_dt : cfl * __longlong_as_double((long long)c->cfl_min);
    if (c->reject_drho > 0.0) dt *= c->factor;
  }
  if (c->t_end > 0.0) dt = fmin(dt, c->t_end - c->t);
  c->dt = dt;
  c->cfl_min = 0x7ff0000000000000ull;
  c->started = 1;
}

// Device arrays shared by all kernels (struct of pointers, passed by value).
struct DevData {
  int n_cells, ld, n_edges, lde;
  const uint8_t *flags;
  const int *l2g;        // [MAXL][ld] through the periodic source map
  const double *pinv;    // [NP][ld]
  const float *pinv32;   // [NP][ld] (mixed precision)
  const uint8_t *bloc;   // [NB*RB][ld]
  const double *center;  // [ND][ld]
  const double *inv_len; // [ld]
  const double *mom;     // [NC][ld] (C_1 .. C_NC of the final polynomial)
  const int *cface;      // [NF][ld]  2 * edge + side, -1 when absent
  const double *inv_vol; // [ld]
  const double *r_eff;   // [ld] in-radius, minimum over the cell and its ghost images
  const int *fL, *fR;    // [lde]
  const uint8_t *fkL, *fkR, *factive;
  const double *fqx;     // [NQF][ND][lde]
  const double *fqw;     // [NQF][lde]
  const double *frame;   // [ND*ND][lde]: normal, tangent 1 (, tangent 2)
  const double *farea;   // [lde]
  // equilibrium / gravity
  const double *phi_cq;  // [NQC][ld] potential at the cell quadrature points
  const double *phi_m1;  // [ld] quadrature average of phi over the cell
  const double *phi_var; // [ld] quadrature average of (phi - phi_m1)^2
  const double *gphi_cq; // [NQC][ND][ld]
  const double *cqx;     // [NQC][ND][ld]
  const double *cqw;     // [NQC][ld]
  const double *phi_fq;  // [NQF][lde]
  // FP32 copies for the mixed form
  const float *frame32;  // [ND*ND][lde]
  const float *xfq32;    // [NF*NQF][ND][ld] scaled offsets (x - x_c) / l of the cell's face points
  const float *xcq32;    // [NQC][ND][ld] scaled offsets of the cell's quadrature points
  const float *mom32;    // [NC][ld]
  const float *fqw32;    // [NQF][lde] face quadrature weights
  const double *gphi_w;  // [ND][ld] sum_q w_q grad phi(x_q) over the cell
  const float *wg32;     // [NQC][ND][ld] w_q grad phi(x_q)
  const float2 *m1s;     // [ld] phi_m1 as an FP32 (hi, lo) pair
  const float2 *vars;    // [ld] phi_var as an FP32 (hi, lo) pair
  const float2 *phi_fq2; // [NQF][lde] phi at the face points as FP32 (hi, lo) pairs
  const double *heat_w;  // [NQC][ld] w_q * heating rate at x_q, or null (no heating)
  Clock *clock;
};

struct Params {
  double gamma;
  double lw[5];      // normalised linear weights
  double inv_lw0;    // 1 / lw[0]
  double epsilon, exponent;
  double cfl;
  double what_c[16]; // reference-cell volume weights (sum to one)
  int nqc, nqf;
  int flux_bc;       // 0 none, 1 constant, 2 isentropic
  int n_stages;
  int gamma2;        // gamma == 2: closed-form equilibrium cell averages (and, mixed, fit)
  double inv_gm1;    // 1 / (gamma - 1), computed once on the host
  double gm1;        // gamma - 1, computed once on the host
  int weno_ao;       // reconstruction: 0 CWENO-AO, 1 WENO-AO
  double a[4][4], b[4];
  // FP32 copies for the mixed form, rounded once on the host
  float lw32[5], inv_lw0_32, eps32, gamma32;
  int exp4;          // exponent == 4
  // equilibrium refresh schedule (LocalRCParams, local_reconstruction.hpp:18-21):
  // refresh every steps_per_recompute reconstructions, or sooner when the
  // scaled (rho, E_int) of the cell leave its equilibrium average by
  // recompute_threshold; 1 refreshes at every reconstruction
  int steps_per_recompute;
  double recompute_threshold;
};

struct StageArgs {
  const double *q;   // stage state
  double *fv;        // FP64: face values [NF*NQF*NV][ld]
  float *fv32;       // MIXED: polynomial part at the face points [NF*NQF*NV][ld]
  double *dev0;      // MIXED: cell-average deviation of every cell [NV][ld]
  double *nf;        // face fluxes [NV][lde]
  double *src;       // per-cell source [NV][ld]
  double *eqth;      // per-cell bound equilibrium (h_r, f, K, found) [4][ld]
  double *u0;        // state at the start of the step
  double *ux;        // next stage state
  double *k[4];      // stage tendencies
  double *tend_out;  // when non-null: write the tendency and do no RK update
  // MIXED: per-face flux G [NV][lde] and per-side corrections mL, mR [ND][lde]
  // (tend_L += -G + mL, tend_R += G + mR), FP32 source [NV][ld], FP32 stage
  // tendencies [NV][ld]
  float *g32, *mL32, *mR32, *src32, *k32[4];
  // MIXED: the stage state as FP32 (hi, lo) pairs [NV][ld] (hi + lo carries 48
  // bits of the FP64 value), and the pairs the update writes with its state
  const float2 *qs;
  float2 *qs_next;
  // MIXED: FP32 copy of dev0 [NV][ld]; with gamma = 2 the bound equilibrium
  // (h_r, f, K) as FP32 (hi, lo) pairs [3][ld]
  float *dev032;
  float2 *eq32;
  // when non-null: every reconstructed cell's polynomial record [PolyRecord][ld]
  double *poly_out;
  // step rejection: the last stage saves the step's start state here [NV][ld]
  double *uprev;
  // equilibrium refresh schedule (only with steps_per_recompute > 1): the
  // reconstructions since the last refresh [ld], and per cell the scale
  // (rho, E_int) and the equilibrium's own cell average (rho, E_int) of the
  // last refresh [4][ld]; eqth then holds the equilibrium between stages
  int *sched_count;
  double *sched;
  double coef[4];    // RK row of this stage: a[stage + 1][.] or b[.] at the last stage
  float coef32[4];   // the same row rounded to FP32 (mixed form)
  int stage;
};

template <int NDIM_, int R0_, int C0_, int NB_, int RB_, int CB_, int NQF_, int NQC_>
struct Shape {
  static constexpr int ND = NDIM_, NV = NDIM_ + 2, NF = NDIM_ + 1;
  static constexpr int R0 = R0_, C0 = C0_, NB = NB_, RB = RB_, CB = CB_;
  static constexpr int NC = C0_ > CB_ ? C0_ : CB_;
  static constexpr int NP = R0_ * C0_ + NB_ * RB_ * CB_;
  static constexpr int MAXL = R0_ + 1 + NB_ * RB_;
  static constexpr int NQF = NQF_, NQC = NQC_;
};

__host__ __device__ __forceinline__ double powd(double x, double y) {
  if (y == 1.0) return x;
  if (y == 2.0) return x * x;
  return pow(x, y);
}

// Non-constant monomials of the scaled offset X in poly_index order
// (math/poly2d_impl.hpp:176-183), minus the normalized moments.
template <int ND, int NC, class R>
__host__ __device__ __forceinline__ void basis(const R *X, const R *C, R *phi) {
  if (ND == 2) {
    const R x = X[0], y = X[1];
    R m[5] = {x, y, x * x, x * y, y * y};
#pragma unroll
    for (int c = 0; c < NC; ++c) phi[c] = m[c] - C[c];
  } else {
    const R x = X[0], y = X[1], z = X[2];
    R m[9] = {x, y, z, x * x, x * y, x * z, y * y, y * z, z * z};
#pragma unroll
    for (int c = 0; c < NC; ++c) phi[c] = m[c] - C[c];
  }
}

// Isentropic equilibrium (model/isentropic_equilibrium.hpp:27-63 with
// IdealGasEOS::rhoE(EnthalpyEntropy), ideal_gas_eos.hpp:162-168):
//   h(x) = h_ref + phi_ref - phi(x),  rho = ((gamma-1)/gamma h / K)^(1/(gamma-1)),
//   E = K rho^gamma / (gamma-1).
// The reference evaluates `1.0 / K * (gamma - 1.0) / gamma * h` left to right, so
// the factor in front of h depends on K only and is computed once per
// equilibrium; the result is bit-identical.
struct EqEval {
  double gamma, gm1, inv_gm1;
  struct Bound {
    double hr, f, K;
    __host__ __device__ __forceinline__ void at(const EqEval &ev, double phi, double &rho, double &E) const {
      double h = hr - phi;
      rho = powd(f * h, ev.inv_gm1);
      double p = K * powd(rho, ev.gamma);
      E = ev.gm1 == 1.0 ? p : p / ev.gm1;
    }
  };
  __host__ __device__ __forceinline__ Bound bind(double h_ref, double K, double phi_ref) const {
    return Bound{h_ref + phi_ref, 1.0 / K * gm1 / gamma, K};
  }
};

// Quadrature average of the equilibrium over a cell.  For gamma = 2 the
// density is linear and the energy quadratic in phi, so the average follows
// exactly from the cell's <phi> and <(phi - <phi>)^2>:
//   rho_bar = f (h_r - <phi>),  E_bar = K f^2 ((h_r - <phi>)^2 + var phi).
// Otherwise the quadrature-point sum with the reference-cell weights.  (The
// reference sums w_q f(x_q) over the volume-scaled weights and divides by the
// volume; in the FP64 form that order costs two FP64 divisions per average and
// made the reconstruction 2.9x slower, for last-bit differences of the size
// the reference's own atomic flux sums change from run to run.)
template <int NQC>
__device__ __forceinline__ void eq_cell_average(const EqEval &ev, const Params &P, const DevData &d,
                                                const EqEval::Bound &b, int j, double &rb, double &Eb) {
  if (P.gamma2) {
    const double t = b.hr - d.phi_m1[j];
    rb = b.f * t;
    Eb = b.K * (b.f * b.f) * (t * t + d.phi_var[j]);
    return;
  }
  double r, e;
  b.at(ev, d.phi_cq[j], r, e);
  rb = P.what_c[0] * r;
  Eb = P.what_c[0] * e;
#pragma unroll
  for (int q = 1; q < NQC; ++q) {
    b.at(ev, d.phi_cq[q * d.ld + j], r, e);
    rb += P.what_c[q] * r;
    Eb += P.what_c[q] * e;
  }
}

// LocalEquilibriumBase::solve_exact + quasi_newton (local_equilibrium_impl.hpp:40-94,
// math/quasi_newton.hpp:12-50, rolling_convergence_rate.hpp): finite-difference
// Jacobian, atol = 1e-13 * guess, at most 20 iterations.  Returns 0 when the
// equilibrium was found, 1 when it was not (the reference then extrapolates
// zeros), 2 when the iteration diverged (the reference aborts).
template <int NQC>
__device__ int solve_equilibrium(const EqEval &ev, const Params &P, const DevData &d, int i, double phi_ref,
                                 double rho_bar, double E_bar, double &h_out, double &K_out) {
  const double gamma = ev.gamma;
  const double p_g = E_bar * ev.gm1;
  const double h0 = gamma / ev.gm1 * p_g / rho_bar;
  const double K0 = p_g / powd(rho_bar, gamma);
  const double atol0 = 1e-13 * h0, atol1 = 1e-13 * K0;
  // EqEval::bind's factor (gamma - 1) / (gamma K), in bind's own operation
  // order: it depends on K only, so the evaluations that vary h reuse it
  auto factor = [&](double K) { return 1.0 / K * ev.gm1 / ev.gamma; };
  auto f = [&](double h, double K, double fk, double &f0, double &f1) {
    double rb, Eb;
    eq_cell_average<NQC>(ev, P, d, EqEval::Bound{h + phi_ref, fk, K}, i, rb, Eb);
    f0 = rho_bar - rb;
    f1 = E_bar - Eb;
  };
  double x0 = h0, x1 = K0, fx0, fx1;
  double fk = factor(x1);
  f(x0, x1, fk, fx0, fx1);
  double dx0 = 2.0 * atol0 + 1.0, dx1 = 2.0 * atol1 + 1.0;
  double hist0[3] = {0, 0, 0}, hist1[3] = {0, 0, 0};
  int iter = 0;
  while (!(fabs(dx0) <= atol0 && fabs(dx1) <= atol1) && iter < 20) {
    double eps0 = 1e-6 * fabs(x0), eps1 = 1e-6 * fabs(x1);
    double a0, a1, b0, b1;
    f(x0 + 0.5 * eps0, x1, fk, a0, a1);
    f(x0 - 0.5 * eps0, x1, fk, b0, b1);
    double d00 = (a0 - b0) / eps0, d01 = (a1 - b1) / eps0;
    const double k_up = x1 + 0.5 * eps1, k_dn = x1 - 0.5 * eps1;
    f(x0, k_up, factor(k_up), a0, a1);
    f(x0, k_dn, factor(k_dn), b0, b1);
    double d10 = (a0 - b0) / eps1, d11 = (a1 - b1) / eps1;
    double inv_det = 1.0 / (d00 * d11 - d01 * d10);
    dx0 = inv_det * (d11 * fx0 - d10 * fx1);
    dx1 = inv_det * (-d01 * fx0 + d00 * fx1);
    x0 -= dx0;
    x1 -= dx1;
    fk = factor(x1);
    f(x0, x1, fk, fx0, fx1);
    hist0[0] = hist0[1], hist0[1] = hist0[2], hist0[2] = dx0;
    hist1[0] = hist1[1], hist1[1] = hist1[2], hist1[2] = dx1;
    if (iter >= 4) {
      bool conv = (hist0[2] <= atol0) && (hist1[2] <= atol1);
      if (!conv) {
        double r0 = log(fabs(hist0[2]) / fabs(hist0[1])) / log(fabs(hist0[1]) / fabs(hist0[0]));
        double r1 = log(fabs(hist1[2]) / fabs(hist1[1])) / log(fabs(hist1[1]) / fabs(hist1[0]));
        if (!(r0 >= 0.0 && r1 >= 0.0)) {
          h_out = h0;
          K_out = K0;
          return 2;
        }
      }
    }
    ++iter;
  }
  if (iter == 20 && !(fabs(dx0) <= 1000.0 * atol0 && fabs(dx1) <= 1000.0 * atol1)) {
    h_out = h0;
    K_out = K0;
    return 1;
  }
  h_out = x0;
  K_out = x1;
  return 0;
}

__device__ __forceinline__ void set_status(Clock *c, int bits) { atomicOr(&c->status, bits); }

// Exported reconstruction of one cell (GlobalReconstruction::operator()(i, x)):
// u(x) = dev0 + sum_c coef[c] (monomial_c((x - xc) / len) - C_c)  (+ the bound
// equilibrium at x for rho and E).  Layout, one [ld] row each:
//   dev0[NV] | coef[NC][NV] | xc[ND] | 1/len | C[NC] | h_r, f, K, found | valid
template <class S>
struct PolyRecord {
  static constexpr int DEV = 0, COEF = S::NV, XC = COEF + S::NC * S::NV, IL = XC + S::ND, MOM = IL + 1,
                       EQ = MOM + S::NC, VALID = EQ + 4, SIZE = VALID + 1;
};

// ------------------------------------------------------------- load paths
// A kernel's per-cell operands that only the thread of that cell reads (its
// stencil operator, its quadrature offsets, its slots of the index tables) are
// read once and bypass L1 (ld.global.nc.L1::no_allocate): the L1 that the
// shared-memory carve-out leaves then holds the stencil gathers, which
// neighbouring threads reuse.  Gathered operands that no thread of the running
// kernel writes take the read-only path (ld.global.nc).  Both leave the L2
// policy alone: between the stages of a run the operators stay L2-resident
// when they fit.
__device__ __forceinline__ float ld_once(const float *p) {
  float v;
  asm("ld.global.nc.L1::no_allocate.f32 %0, [%1];" : "=f"(v) : "l"(p));
  return v;
}
__device__ __forceinline__ double ld_once(const double *p) {
  double v;
  asm("ld.global.nc.L1::no_allocate.f64 %0, [%1];" : "=d"(v) : "l"(p));
  return v;
}
__device__ __forceinline__ int ld_once(const int *p) {
  int v;
  asm("ld.global.nc.L1::no_allocate.s32 %0, [%1];" : "=r"(v) : "l"(p));
  return v;
}
template <class T>
__device__ __forceinline__ T ld_gather(const T *p) {
  return __ldg(p);
}

// ------------------------------------------------- FP32 pair ("double-float")
// Unevaluated sums hi + lo of two FP32 numbers, with the error-free
// transformations of Knuth (two-sum, TAOCP vol. 2, 4.2.2) and Dekker (two-product,
// 1971; here with a fused multiply-add).  About 48 significant bits on the
// FP32 pipe, which on this GPU issues 64 times faster than the FP64 pipe.
struct DF {
  float hi, lo;
};
__device__ __forceinline__ DF df_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return DF{s, e};
}
__device__ __forceinline__ DF df_fast(float a, float b) {  // |a| >= |b| or a == 0
  const float s = __fadd_rn(a, b);
  return DF{s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ DF df_add(DF x, DF y) {
  DF s = df_two_sum(x.hi, y.hi);
  return df_fast(s.hi, __fadd_rn(s.lo, __fadd_rn(x.lo, y.lo)));
}
__device__ __forceinline__ DF df_sub(DF x, DF y) { return df_add(x, DF{-y.hi, -y.lo}); }
__device__ __forceinline__ DF df_mul(DF x, DF y) {
  const float p = __fmul_rn(x.hi, y.hi);
  float e = __fmaf_rn(x.hi, y.hi, -p);
  e = __fmaf_rn(x.hi, y.lo, e);
  e = __fmaf_rn(x.lo, y.hi, e);
  return df_fast(p, e);
}
__device__ __forceinline__ DF df_of(float2 v) { return DF{v.x, v.y}; }
// x - y for two pairs whose hi parts lie within a factor of two of each other
// (neighbouring cell averages, or a difference and the equilibrium variation
// it nearly cancels): the hi difference is then exact (Sterbenz's lemma), so
// the result needs no renormalisation.  Outside that range the hi difference
// is rounded once, a relative error of 2^-24 of a difference that is then
// large -- the precision the result is rounded to anyway.
__device__ __forceinline__ DF df_sub_close(DF x, DF y) { return DF{__fsub_rn(x.hi, y.hi), __fsub_rn(x.lo, y.lo)}; }
__device__ __forceinline__ float df_round(DF x) { return __fadd_rn(x.hi, x.lo); }
// FP64 value as an FP32 pair (FP64 pipe: used once per cell, not per stencil row)
__device__ __forceinline__ DF df_split(double x) {
  const float hi = __double2float_rn(x);
  return DF{hi, __double2float_rn(x - (double)hi)};
}

// --------------------------------------------------------- reconstruction
// The 2D mixed well-balanced reconstruction, whose stencil rows cost FP32-pair
// arithmetic, keeps the row differences in dynamic shared memory: (MAXL - 1)
// rows x NV floats per thread.  Elsewhere rows are cheap and the L1 cache is
// worth more than the shared memory.
template <class S, int EQ, bool MIXED>
constexpr bool kRowsInShared = MIXED && EQ && S::ND == 2;
template <class S, int EQ, bool MIXED>
constexpr size_t recon_smem_bytes(int threads) {
  return kRowsInShared<S, EQ, MIXED> ? (size_t)(S::MAXL - 1) * S::NV * threads * sizeof(float) : 0;
}

// Heating (model/heating.hpp:29-45) in the mixed form: sum_q w_q rate(x_q)
// rho(x_q) with rho = equilibrium (FP64) + cell deviation (FP64) + polynomial
// part (FP32); the caller divides by the volume.
template <class S, int EQ, bool MIXED, class PolyX>
__device__ __forceinline__ double heating(const DevData &d, const EqEval &ev, const EqEval::Bound &eqb, bool found,
                                          const double *dev0, const PolyX &poly_X, int i) {
  using R = std::conditional_t<MIXED, float, double>;
  constexpr int ND = S::ND, NV = S::NV;
  const int ld = d.ld;
  double h = 0.0;
  R hp = R(0);
#pragma unroll
  for (int qq = 0; qq < S::NQC; ++qq) {
    const double hw = d.heat_w[qq * ld + i];
    double r_eq = 0.0, E_eq = 0.0;
    if (EQ && found) eqb.at(ev, d.phi_cq[qq * ld + i], r_eq, E_eq);
    h += hw * (r_eq + dev0[0]);
    R X[ND], pv[NV];
#pragma unroll
    for (int k = 0; k < ND; ++k) X[k] = R(d.xcq32[(qq * ND + k) * ld + i]);
    poly_X(X, pv);
    hp += R(hw) * pv[0];
  }
  return h + double(hp);
}

template <class S, int EQ, int SRC, bool MIXED, bool EXPORT = false>
__device__ __forceinline__ void recon_cell(const DevData &d, const Params &P, const StageArgs &a, const int i) {
  using R = std::conditional_t<MIXED, float, double>;
  constexpr int NV = S::NV, ND = S::ND, NF = S::NF, NC = S::NC;
  if (i >= d.n_cells) return;
  if (d.clock->done) return;
  const uint8_t fl = d.flags[i];
  if (!(fl & (kInterior | kGhostL1))) return;
  const int ld = d.ld;
  const double *__restrict__ q = a.q;
  const double gamma = P.gamma;
  EqEval ev{gamma, gamma - 1.0, P.inv_gm1};

  const int j0 = ld_once(&d.l2g[i]);
  if constexpr (kRowsInShared<S, EQ, MIXED>) {
    // all stencil indices first, as independent loads in flight during the
    // FP64 work below, parked in the first slot of their own row until the
    // row is computed
    extern __shared__ float rows_park[];
#pragma unroll
    for (int l = 1; l < S::MAXL; ++l)
      rows_park[((l - 1) * NV) * blockDim.x + threadIdx.x] = __int_as_float(ld_once(&d.l2g[l * ld + i]));
  }
  double u0[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) u0[v] = q[v * ld + j0];
  const double rho = u0[0];
  // mixed form: one FP64 reciprocal of rho serves the kinetic energy and the
  // equilibrium fit (FP64 divisions cost the 1/64-rate FP64 pipe ~10 slots each)
  double eint, inv_rho = 0.0;
  if constexpr (MIXED) {
    inv_rho = 1.0 / rho;
    double m2 = 0.0;
#pragma unroll
    for (int v = 1; v < NV - 1; ++v) m2 += u0[v] * u0[v];
    eint = u0[NV - 1] - 0.5 * m2 * inv_rho;
  } else {
    eint = u0[NV - 1] - kinetic_energy<NV>(u0);
  }
  if (!(rho > 0.0) || !(eint > 0.0)) {
    set_status(d.clock, kStNonPhysical);
    return;
  }
  // LocalReconstruction::recompute_equilibrium (local_reconstruction.hpp:87-100):
  // with a schedule the equilibrium and the scaling of the last refresh stay
  // until steps_per_recompute reconstructions have passed, or until the
  // scaled distance of (rho, E_int) from the equilibrium's own cell average
  // reaches recompute_threshold
  bool refresh = true;
  double rho_s = rho, eint_s = eint;
  if (EQ && a.sched_count) {
    const int cnt = a.sched_count[i];
    if (cnt % P.steps_per_recompute != 0) {
      rho_s = a.sched[i];
      eint_s = a.sched[ld + i];
      const double d0 = (rho - a.sched[2 * ld + i]) / rho_s, d1 = (eint - a.sched[3 * ld + i]) / eint_s;
      // the reference's norm, each product and the sum rounded on their own
      refresh = sqrt(__dadd_rn(__dmul_rn(d0, d0), __dmul_rn(d1, d1))) >= P.recompute_threshold;
      if (refresh) rho_s = rho, eint_s = eint;
    }
    a.sched_count[i] = refresh ? 1 : cnt + 1;
  }
  // EulerScaling (model/characteristic_scale.hpp:23-32): {rho, c, c, c, E_int}
  R inv_s2[NV];
  {
    const R rr = R(rho_s), ee = R(eint_s), g = MIXED ? R(P.gamma32) : R(gamma);
    const R cs = sqrt(g * (ee * (g - R(1))) / rr);
    inv_s2[0] = R(1) / (rr * rr);
#pragma unroll
    for (int v = 1; v < NV - 1; ++v) inv_s2[v] = R(1) / (cs * cs);
    inv_s2[NV - 1] = R(1) / (ee * ee);
  }

  // local equilibrium of this cell from its own average
  double eh = 0.0, eK = 0.0, phi_ref = 0.0;
  bool found = false;
  // closed form for gamma = 2 (mixed form): the cell average of the
  // equilibrium is rho_bar = T / (2K), E_bar = (T^2 + var phi) / (4K) with
  // T = h_r - <phi>, so K = (E_bar + sqrt(E_bar^2 - rho_bar^2 var)) / (2 rho_bar^2)
  // and T = 2 K rho_bar: the exact root the FP64 form's Newton iteration
  // converges to within its tolerance.
  // With T = 2 K rho_bar = (E_bar + sqrt(disc)) / rho_bar: K = T / (2 rho_bar),
  // h_r = T + <phi> and f = (gamma - 1) / (gamma K) = rho_bar / T.
  bool closed = false;
  double f_closed = 0.0;
  if (EQ && !refresh) {
    // the equilibrium of the last refresh, as it was bound then
    phi_ref = d.phi_cq[i];
  } else if (EQ && MIXED && P.gamma2) {
    phi_ref = d.phi_cq[i];
    const double m1 = d.phi_m1[i], var = d.phi_var[i];
    const double disc = eint * eint - rho * rho * var;
    if (disc >= 0.0) {
      const double T = (eint + sqrt(disc)) * inv_rho;
      eK = 0.5 * T * inv_rho;
      eh = T + m1 - phi_ref;
      f_closed = rho / T;
      found = eK > 0.0;
      closed = true;
    }
  }
  if (EQ && refresh && !closed) {
    phi_ref = d.phi_cq[i];
    int st = solve_equilibrium<S::NQC>(ev, P, d, i, phi_ref, rho, eint, eh, eK);
    found = st == 0;
    if (st == 2) set_status(d.clock, kStNewton);
  }
  EqEval::Bound eqb;
  if (EQ && !refresh) {
    eqb = EqEval::Bound{a.eqth[i], a.eqth[ld + i], a.eqth[2 * ld + i]};
    found = a.eqth[3 * ld + i] != 0.0;
  } else {
    eqb = closed ? EqEval::Bound{eh + phi_ref, f_closed, eK} : ev.bind(eh, eK, phi_ref);
  }
  if (EQ && refresh) {
    a.eqth[i] = eqb.hr;
    a.eqth[ld + i] = eqb.f;
    a.eqth[2 * ld + i] = eqb.K;
    a.eqth[3 * ld + i] = found ? 1.0 : 0.0;
    if (a.sched_count) {
      // the scale and the equilibrium's own cell average (rhoEbar_cache(0),
      // zero when no equilibrium was found) of this refresh
      double rc = 0.0, Ec = 0.0;
      if (found) eq_cell_average<S::NQC>(ev, P, d, eqb, j0, rc, Ec);
      a.sched[i] = rho_s;
      a.sched[ld + i] = eint_s;
      a.sched[2 * ld + i] = rc;
      a.sched[3 * ld + i] = Ec;
    }
  }
  // deviation of a stencil cell's average from this cell's equilibrium (FP64)
  auto load_dev = [&](int j, double *out) {
#pragma unroll
    for (int v = 0; v < NV; ++v) out[v] = q[v * ld + j];
    if (EQ && found) {
      double rb, Eb;
      eq_cell_average<S::NQC>(ev, P, d, eqb, j, rb, Eb);
      out[0] -= rb;
      out[NV - 1] -= Eb;
    }
  };
  double dev0[NV];
  if (EQ) {
    // the own cell goes through the same path so padded rows cancel exactly
    load_dev(j0, dev0);
  } else {
#pragma unroll
    for (int v = 0; v < NV; ++v) dev0[v] = u0[v];
  }
  float dev0f[NV];  // mixed form: the deviation rounded to FP32 once
  DF f_split{0.f, 0.f};
  if (MIXED) {
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      a.dev0[v * ld + i] = dev0[v];
      dev0f[v] = float(dev0[v]);
      a.dev032[v * ld + i] = dev0f[v];
    }
    if (EQ && P.gamma2) {
      const DF hr = df_split(eqb.hr), K = df_split(eqb.K);
      f_split = df_split(eqb.f);
      a.eq32[i] = make_float2(hr.hi, hr.lo);
      a.eq32[ld + i] = make_float2(f_split.hi, f_split.lo);
      // K > 0 whenever the equilibrium was found; -1 marks a cell without one,
      // so the face kernel tells them apart with one FP32 comparison
      a.eq32[2 * ld + i] = found ? make_float2(K.hi, K.lo) : make_float2(-1.f, 0.f);
    }
  }
  // dev_j - dev_0 for a stencil cell j.  In the mixed form with gamma = 2 the
  // equilibrium averages are differenced analytically,
  //   d rho = (q_j - q_0) - f (<phi>_0 - <phi>_j),
  //   d E   = (q_j - q_0) - K f^2 ((<phi>_0 - <phi>_j)(2 h_r - <phi>_j - <phi>_0) + var_j - var_0),
  // so the O(h) equilibrium variation cancels against the O(h) state variation
  // in 48-bit FP32-pair arithmetic, never in plain FP32.
  const bool diff_form = MIXED && EQ && found && P.gamma2;
  // Mixed form: the stencil rows come from the FP32 (hi, lo) pairs of the
  // state, <phi> and var(phi); the differences and the analytic equilibrium
  // differences are formed in FP32-pair arithmetic and rounded once to FP32.
  DF own_q[NV], own_m1{0.f, 0.f}, own_var{0.f, 0.f}, df_f{0.f, 0.f}, df_kf2{0.f, 0.f}, df_2t{0.f, 0.f};
  if (MIXED && (!EQ || diff_form)) {
#pragma unroll
    for (int v = 0; v < NV; ++v) own_q[v] = df_of(ld_gather(&a.qs[v * ld + j0]));
    if (diff_form) {
      own_m1 = df_of(ld_gather(&d.m1s[j0]));
      own_var = df_of(ld_gather(&d.vars[j0]));
      df_f = f_split;
      df_kf2 = df_split(eqb.K * (eqb.f * eqb.f));
      df_2t = df_split(2.0 * (eqb.hr - d.phi_m1[j0]));
    }
  }
  auto row_diff = [&](int j, R *dq) {
    if (MIXED && !EQ) {
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        const float2 x = ld_gather(&a.qs[v * ld + j]);
        dq[v] = R(__fadd_rn(__fsub_rn(x.x, own_q[v].hi), __fsub_rn(x.y, own_q[v].lo)));
      }
    } else if (MIXED && diff_form) {
      // rho_eq(j) - rho_eq(0) = f dm,
      // E_eq(j) - E_eq(0) = K f^2 (dm (2 (h_r - <phi>_0) + dm) + var_j - var_0),
      // dm = <phi>_0 - <phi>_j
      // <phi> may differ by more than a factor of two near the centre of the
      // potential: full two-sum there
      const DF dm = df_sub(own_m1, df_of(ld_gather(&d.m1s[j])));
#pragma unroll
      for (int v = 1; v < NV - 1; ++v) {
        const float2 x = ld_gather(&a.qs[v * ld + j]);
        dq[v] = R(__fadd_rn(__fsub_rn(x.x, own_q[v].hi), __fsub_rn(x.y, own_q[v].lo)));
      }
      dq[0] = R(df_round(df_sub_close(df_sub_close(df_of(ld_gather(&a.qs[j])), own_q[0]), df_mul(df_f, dm))));
      // 2 (h_r - <phi>_0) + dm with |dm| << |2 (h_r - <phi>_0)|
      const float sh = __fadd_rn(df_2t.hi, dm.hi);
      const DF sum{sh, __fadd_rn(__fsub_rn(dm.hi, __fsub_rn(sh, df_2t.hi)), __fadd_rn(df_2t.lo, dm.lo))};
      const DF t = df_add(df_mul(dm, sum), df_sub_close(df_of(ld_gather(&d.vars[j])), own_var));
      const DF dE = df_sub_close(df_sub_close(df_of(ld_gather(&a.qs[(NV - 1) * ld + j])), own_q[NV - 1]), df_mul(df_kf2, t));
      dq[NV - 1] = R(df_round(dE));
    } else {
      double dq64[NV];
      load_dev(j, dq64);
#pragma unroll
      for (int v = 0; v < NV; ++v) dq[v] = R(dq64[v] - dev0[v]);
    }
  };

  // LSQ fits: coefficients 1..C of every stencil, unscaled
  R b0[S::C0][NV];
#pragma unroll
  for (int c = 0; c < S::C0; ++c)
#pragma unroll
    for (int v = 0; v < NV; ++v) b0[c][v] = R(0);
  R bb[S::NB][S::CB][NV];
#pragma unroll
  for (int k = 0; k < S::NB; ++k)
#pragma unroll
    for (int c = 0; c < S::CB; ++c)
#pragma unroll
      for (int v = 0; v < NV; ++v) bb[k][c][v] = R(0);
  if constexpr (kRowsInShared<S, EQ, MIXED>) {
    // The one-sided stencils mostly reuse cells of the central one (the
    // combined 2D stencil averages about 11 cells for 19 rows), so every
    // distinct stencil cell is differenced once into shared memory,
    // rows[((l - 1) * NV + v) * blockDim.x + thread], and all fits read it there.
    extern __shared__ float rows_smem[];
    const int bd = blockDim.x, tid = threadIdx.x;
    // (the stencil indices are parked in the rows' first slots)
#pragma unroll 2
    for (int l = 1; l < S::MAXL; ++l) {
      const int j = __float_as_int(rows_smem[((l - 1) * NV) * bd + tid]);
      R dq[NV];
      if (j != j0) {
        row_diff(j, dq);
      } else {
#pragma unroll
        for (int v = 0; v < NV; ++v) dq[v] = R(0);
      }
#pragma unroll
      for (int v = 0; v < NV; ++v) rows_smem[((l - 1) * NV + v) * bd + tid] = dq[v];
    }
    // fully unrolled: the operator's loads of every row can be in flight together
#pragma unroll
    for (int r = 0; r < S::R0; ++r) {
#pragma unroll
      for (int c = 0; c < S::C0; ++c) {
        const R pc = R(ld_once(&d.pinv32[(c * S::R0 + r) * ld + i]));
#pragma unroll
        for (int v = 0; v < NV; ++v) b0[c][v] += pc * rows_smem[(r * NV + v) * bd + tid];
      }
    }
#pragma unroll
    for (int k = 0; k < S::NB; ++k)
#pragma unroll
      for (int r = 0; r < S::RB; ++r) {
        const int l = d.bloc[(k * S::RB + r) * ld + i];
        R dq[NV];
#pragma unroll
        for (int v = 0; v < NV; ++v) dq[v] = l > 0 ? rows_smem[((l - 1) * NV + v) * bd + tid] : R(0);
#pragma unroll
        for (int c = 0; c < S::CB; ++c) {
          const R pc = R(ld_once(&d.pinv32[(S::R0 * S::C0 + (k * S::CB + c) * S::RB + r) * ld + i]));
#pragma unroll
          for (int v = 0; v < NV; ++v) bb[k][c][v] += pc * dq[v];
        }
      }
  } else if constexpr (MIXED && S::ND == 2) {
    // all stencil indices first, as independent loads, so the gathers of a
    // row do not wait on the load of its index (in 3D the extra registers
    // cost a block per SM, which costs more than the wait)
    int jc[S::R0], jb[S::NB * S::RB];
#pragma unroll
    for (int r = 0; r < S::R0; ++r) jc[r] = ld_once(&d.l2g[(r + 1) * ld + i]);
#pragma unroll
    for (int kr = 0; kr < S::NB * S::RB; ++kr) jb[kr] = d.l2g[d.bloc[kr * ld + i] * ld + i];
#pragma unroll 2
    for (int r = 0; r < S::R0; ++r) {
      R dq[NV];
      row_diff(jc[r], dq);
#pragma unroll
      for (int c = 0; c < S::C0; ++c) {
        const R pc = R(ld_once(&d.pinv32[(c * S::R0 + r) * ld + i]));
#pragma unroll
        for (int v = 0; v < NV; ++v) b0[c][v] += pc * dq[v];
      }
    }
#pragma unroll
    for (int k = 0; k < S::NB; ++k) {
#pragma unroll
      for (int r = 0; r < S::RB; ++r) {
        R dq[NV];
        row_diff(jb[k * S::RB + r], dq);
#pragma unroll
        for (int c = 0; c < S::CB; ++c) {
          const R pc = R(ld_once(&d.pinv32[(S::R0 * S::C0 + (k * S::CB + c) * S::RB + r) * ld + i]));
#pragma unroll
          for (int v = 0; v < NV; ++v) bb[k][c][v] += pc * dq[v];
        }
      }
    }
  } else {
#pragma unroll 2
    for (int r = 0; r < S::R0; ++r) {
      R dq[NV];
      row_diff(ld_once(&d.l2g[(r + 1) * ld + i]), dq);
#pragma unroll
      for (int c = 0; c < S::C0; ++c) {
        const R pc = MIXED ? R(ld_once(&d.pinv32[(c * S::R0 + r) * ld + i])) : R(ld_once(&d.pinv[(c * S::R0 + r) * ld + i]));
#pragma unroll
        for (int v = 0; v < NV; ++v) b0[c][v] += pc * dq[v];
      }
    }
#pragma unroll
    for (int k = 0; k < S::NB; ++k) {
#pragma unroll
      for (int r = 0; r < S::RB; ++r) {
        const int l = d.bloc[(k * S::RB + r) * ld + i];
        R dq[NV];
        row_diff(ld_once(&d.l2g[l * ld + i]), dq);
#pragma unroll
        for (int c = 0; c < S::CB; ++c) {
          const int pi = (S::R0 * S::C0 + (k * S::CB + c) * S::RB + r) * ld + i;
          const R pc = MIXED ? R(ld_once(&d.pinv32[pi])) : R(ld_once(&d.pinv[pi]));
#pragma unroll
          for (int v = 0; v < NV; ++v) bb[k][c][v] += pc * dq[v];
        }
      }
    }
  }

  // CWENO-AO: p_c = (p_opt - sum_k g_k p_k) / g_c   (cweno_ao.cpp:35-53);
  // WENO-AO hybridizes p_opt itself (weno_ao.cpp:14-24)
  R pf[NC][NV];
#pragma unroll
  for (int c = 0; c < NC; ++c)
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      R x = c < S::C0 ? b0[c][v] : R(0);
      if (!P.weno_ao) {
#pragma unroll
        for (int k = 0; k < S::NB; ++k)
          if (c < S::CB) x -= (MIXED ? R(P.lw32[k + 1]) : R(P.lw[k + 1])) * bb[k][c][v];
        x *= MIXED ? R(P.inv_lw0_32) : R(P.inv_lw0);
      }
      pf[c][v] = x;
    }
  // smoothness indicators in the scaled variables (poly2d_impl.hpp:325-337)
  auto indicator = [&](auto coef, int ncoef) {
    R m = R(0);
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      R s = R(0);
      for (int c = 0; c < ncoef; ++c) s += coef(c, v) * coef(c, v);
      m = fmax(m, s * inv_s2[v]);
    }
    return m;
  };
  R alpha[S::NB + 1];
  auto weight = [&](R IS, R g) {
    const bool e4 = MIXED ? P.exp4 != 0 : P.exponent == 4.0;
    R pw = e4 ? (IS * IS) * (IS * IS) : R(pow(double(IS), P.exponent));
    return g / ((MIXED ? R(P.eps32) : R(P.epsilon)) + pw);
  };
  auto lw = [&](int k) { return MIXED ? R(P.lw32[k]) : R(P.lw[k]); };
  alpha[0] = weight(indicator([&](int c, int v) { return pf[c][v]; }, S::C0), lw(0));
#pragma unroll
  for (int k = 0; k < S::NB; ++k)
    alpha[k + 1] = weight(indicator([&](int c, int v) { return bb[k][c][v]; }, S::CB), lw(k + 1));
  R al_tot = R(0);
#pragma unroll
  for (int k = 0; k <= S::NB; ++k) al_tot += alpha[k];
  // eno_hybridize (hybrid_weno.cpp:109-128)
  {
    const R w0 = alpha[0] / al_tot;
#pragma unroll
    for (int c = 0; c < NC; ++c)
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        R x = w0 * pf[c][v];
#pragma unroll
        for (int k = 0; k < S::NB; ++k)
          if (c < S::CB) x += (alpha[k + 1] / al_tot) * bb[k][c][v];
        pf[c][v] = x;
      }
  }

  double xc[ND];
  R C[NC];
  double il = 0.0;
  if (!MIXED) {
#pragma unroll
    for (int k = 0; k < ND; ++k) xc[k] = d.center[k * ld + i];
    il = d.inv_len[i];
  }
#pragma unroll
  for (int c = 0; c < NC; ++c) C[c] = MIXED ? R(ld_once(&d.mom32[c * ld + i])) : R(d.mom[c * ld + i]);
  if constexpr (EXPORT) {
    using PR = PolyRecord<S>;
    double *o = a.poly_out;
#pragma unroll
    for (int v = 0; v < NV; ++v) o[(PR::DEV + v) * ld + i] = dev0[v];
#pragma unroll
    for (int c = 0; c < NC; ++c)
#pragma unroll
      for (int v = 0; v < NV; ++v) o[(PR::COEF + c * NV + v) * ld + i] = double(pf[c][v]);
#pragma unroll
    for (int k = 0; k < ND; ++k) o[(PR::XC + k) * ld + i] = d.center[k * ld + i];
    o[PR::IL * ld + i] = d.inv_len[i];
#pragma unroll
    for (int c = 0; c < NC; ++c) o[(PR::MOM + c) * ld + i] = d.mom[c * ld + i];
    o[PR::EQ * ld + i] = eqb.hr;
    o[(PR::EQ + 1) * ld + i] = eqb.f;
    o[(PR::EQ + 2) * ld + i] = eqb.K;
    o[(PR::EQ + 3) * ld + i] = (EQ && found) ? 1.0 : 0.0;
    o[PR::VALID * ld + i] = 1.0;
  }
  // non-constant part of the limited polynomial at the scaled offset X
  auto poly_X = [&](const R *X, R *pv) {
    R phi[NC];
    basis<ND, NC>(X, C, phi);
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      R s = R(0);
#pragma unroll
      for (int c = 0; c < NC; ++c) s += pf[c][v] * phi[c];
      pv[v] = s;
    }
  };
  auto poly_at = [&](const double *x, R *pv) {
    R X[ND];
#pragma unroll
    for (int k = 0; k < ND; ++k) X[k] = R((x[k] - xc[k]) * il);
    poly_X(X, pv);
  };

  double s_acc[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) s_acc[v] = 0.0;

  // values at the face quadrature points of this cell
#pragma unroll
  for (int f = 0; f < NF; ++f) {
    const int cf = d.cface[f * ld + i];
    if (cf < 0) continue;
    const int e = cf >> 1;
    const double sgn = (cf & 1) ? -1.0 : 1.0;
#pragma unroll
    for (int qq = 0; qq < S::NQF; ++qq) {
      R pv[NV];
      if (MIXED) {
        R X[ND];
#pragma unroll
        for (int k = 0; k < ND; ++k) X[k] = R(ld_once(&d.xfq32[((f * S::NQF + qq) * ND + k) * ld + i]));
        poly_X(X, pv);
      } else {
        double x[ND];
#pragma unroll
        for (int k = 0; k < ND; ++k) x[k] = d.fqx[(qq * ND + k) * d.lde + e];
        poly_at(x, pv);
      }
      double r_eq = 0.0, E_eq = 0.0;
      if (EQ && found && !MIXED) {
        eqb.at(ev, d.phi_fq[qq * d.lde + e], r_eq, E_eq);
        if (SRC) {
          // surface part of the well-balanced source: p_eq n_out
          const double p_eq = E_eq * ev.gm1;
          const double w = d.fqw[qq * d.lde + e];
#pragma unroll
          for (int k = 0; k < ND; ++k) s_acc[1 + k] += w * (p_eq * sgn * d.frame[k * d.lde + e]);
        }
      }
      const size_t slot = (size_t)((f * S::NQF + qq) * NV) * ld + i;
      if (MIXED) {
#pragma unroll
        for (int v = 0; v < NV; ++v) a.fv32[slot + (size_t)v * ld] = float(pv[v]);
      } else {
        double u[NV];
#pragma unroll
        for (int v = 0; v < NV; ++v) u[v] = dev0[v] + double(pv[v]);
        u[0] += r_eq;
        u[NV - 1] += E_eq;
#pragma unroll
        for (int v = 0; v < NV; ++v) a.fv[slot + (size_t)v * ld] = u[v];
      }
    }
  }

  if (SRC && MIXED) {
    // volume part, split into the FP64 cell-average deviation times
    // sum_q w_q grad phi_q and the FP32 polynomial part
    // (0, -rho' grad phi, -m . grad phi) with rho', m deviation-sized: FP32
    R acc[NV], G[ND];
#pragma unroll
    for (int v = 0; v < NV; ++v) acc[v] = R(0);
#pragma unroll
    for (int k = 0; k < ND; ++k) G[k] = R(0);
#pragma unroll
    for (int qq = 0; qq < S::NQC; ++qq) {
      R X[ND], wg[ND], pv[NV];
#pragma unroll
      for (int k = 0; k < ND; ++k) {
        X[k] = R(ld_once(&d.xcq32[(qq * ND + k) * ld + i]));
        wg[k] = R(ld_once(&d.wg32[(qq * ND + k) * ld + i]));
        G[k] += wg[k];
      }
      poly_X(X, pv);
      R mg = R(0);
#pragma unroll
      for (int k = 0; k < ND; ++k) {
        acc[1 + k] -= pv[0] * wg[k];
        mg += pv[1 + k] * wg[k];
      }
      acc[NV - 1] -= mg;
    }
    // the surface part p_eq n_out cancels face by face against the flux
    // baseline and is accounted for in k_face_flux
    R mg0 = R(0);
    const R d0 = dev0f[0];
#pragma unroll
    for (int k = 0; k < ND; ++k) {
      acc[1 + k] -= d0 * G[k];
      mg0 += dev0f[1 + k] * G[k];
    }
    acc[NV - 1] -= mg0;
    const double iv = d.inv_vol[i];
    const R ivr = R(iv);
    if (d.heat_w) acc[NV - 1] += R(heating<S, EQ, MIXED>(d, ev, eqb, found, dev0, poly_X, i));
#pragma unroll
    for (int v = 0; v < NV; ++v) a.src32[v * ld + i] = float(acc[v] * ivr);
  } else if (SRC) {
    // volume part: (0, -rho' grad phi, -m . grad phi), rho' = delta (well-balanced)
    // or the full reconstruction (gravity_source_loop.hpp:60-84,121-148)
#pragma unroll
    for (int qq = 0; qq < S::NQC; ++qq) {
      double x[ND], g[ND];
#pragma unroll
      for (int k = 0; k < ND; ++k) {
        x[k] = d.cqx[(qq * ND + k) * ld + i];
        g[k] = d.gphi_cq[(qq * ND + k) * ld + i];
      }
      R pv[NV];
      poly_at(x, pv);
      double du[NV];
#pragma unroll
      for (int v = 0; v < NV; ++v) du[v] = dev0[v] + double(pv[v]);
      const double r = du[0];
      const double w = d.cqw[qq * ld + i];
      double mg = 0.0;
#pragma unroll
      for (int k = 0; k < ND; ++k) {
        s_acc[1 + k] += w * (-r * g[k]);
        mg += du[1 + k] * g[k];
      }
      s_acc[NV - 1] += w * (-mg);
      if (d.heat_w) {
        // Heating (model/heating.hpp:29-45): rho(x_q) * rate(x_q), rho the full reconstruction
        double r_eq = 0.0, E_eq = 0.0;
        if (EQ && found) eqb.at(ev, d.phi_cq[qq * ld + i], r_eq, E_eq);
        s_acc[NV - 1] += d.heat_w[qq * ld + i] * (r_eq + r);
      }
    }
    const double iv = d.inv_vol[i];
#pragma unroll
    for (int v = 0; v < NV; ++v) a.src[v * ld + i] = s_acc[v] * iv;
  }
}

template <class S, int EQ, int SRC, bool MIXED>
__global__ void __launch_bounds__(128) k_reconstruct(const DevData d, const Params P, StageArgs a) {
  recon_cell<S, EQ, SRC, MIXED>(d, P, a, blockIdx.x * blockDim.x + threadIdx.x);
}

// The mixed reconstruction is latency-bound: its builds are held to the
// register count that fits kMixedReconBlocks blocks of 128 threads per SM
// (2D: 96 registers, five blocks -- the well-balanced one also holds 5 x 38.9 KB
// of stencil rows in shared memory; 3D order 2: 128, four; 3D order 3: 168,
// three; the 3D well-balanced builds 168, three, where some 200 bytes of
// spills cost less than the third block gains: 384,000 tetrahedra 0.539 ->
// 0.442 ms per launch against their unbounded 222 registers and two blocks).
template <class S, int EQ>
constexpr int kMixedReconBlocks = S::ND == 2 ? 5 : (EQ ? 3 : (S::C0 <= 3 ? 4 : 3));

template <class S, int EQ, int SRC, bool MIXED>
__global__ void __launch_bounds__(128, kMixedReconBlocks<S, EQ>) k_reconstruct_mixed(const DevData d, const Params P,
                                                                                 StageArgs a) {
  recon_cell<S, EQ, SRC, MIXED>(d, P, a, blockIdx.x * blockDim.x + threadIdx.x);
}

template <class S, int EQ, int SRC, bool MIXED>
constexpr auto recon_kernel() {
  if constexpr (MIXED)
    return &k_reconstruct_mixed<S, EQ, SRC, MIXED>;
  else
    return &k_reconstruct<S, EQ, SRC, MIXED>;
}

// ------------------------------------------------------------- face flux
template <int NV, int ND, class T>
__device__ __forceinline__ void to_face(const T *u, const double *fr, int lde, int e, T *w) {
  w[0] = u[0];
  w[NV - 1] = u[NV - 1];
#pragma unroll
  for (int a = 0; a < ND; ++a) {
    T s = T(0);
#pragma unroll
    for (int k = 0; k < ND; ++k) s += u[1 + k] * T(fr[(a * ND + k) * lde + e]);
    w[1 + a] = s;
  }
}

template <int NV, int ND>
__device__ __forceinline__ void from_face(double *f, const double *fr, int lde, int e) {
  double m[ND];
#pragma unroll
  for (int k = 0; k < ND; ++k) {
    double s = 0.0;
#pragma unroll
    for (int a = 0; a < ND; ++a) s += f[1 + a] * fr[(a * ND + k) * lde + e];
    m[k] = s;
  }
#pragma unroll
  for (int k = 0; k < ND; ++k) f[1 + k] = m[k];
}

template <int NV, int ND>
__device__ __forceinline__ void to_face32(const float *u, const float *fr, int lde, int e, float *w) {
  w[0] = u[0];
  w[NV - 1] = u[NV - 1];
#pragma unroll
  for (int a = 0; a < ND; ++a) {
    float s = 0.0f;
#pragma unroll
    for (int k = 0; k < ND; ++k) s += u[1 + k] * fr[(a * ND + k) * lde + e];
    w[1 + a] = s;
  }
}

template <int NV, int ND>
__device__ __forceinline__ void from_face32(float *f, const float *fr, int lde, int e) {
  float m[ND];
#pragma unroll
  for (int k = 0; k < ND; ++k) {
    float s = 0.0f;
#pragma unroll
    for (int a = 0; a < ND; ++a) s += f[1 + a] * fr[(a * ND + k) * lde + e];
    m[k] = s;
  }
#pragma unroll
  for (int k = 0; k < ND; ++k) f[1 + k] = m[k];
}

template <int NV, int FLUX, class T>
__device__ __forceinline__ void numerical_flux(const T *uL, const T *uR, T gamma, T *f) {
  if (FLUX == 0)
    hllc_flux<NV>(uL, uR, gamma, f);
  else
    rusanov_flux<NV>(uL, uR, gamma, f);
}

__device__ __forceinline__ EqEval::Bound eq_bound(const StageArgs &a, int ld, int c) {
  return EqEval::Bound{a.eqth[c], a.eqth[ld + c], a.eqth[2 * ld + c]};
}
__device__ __forceinline__ bool eq_found(const StageArgs &a, int ld, int c) { return a.eqth[3 * ld + c] != 0.0; }

// Face state of one side in the MIXED form: FP64 base (cell-average deviation
// plus the equilibrium at the point) and the FP32 polynomial part.
template <class S, int EQ>
__device__ __forceinline__ void mixed_base(const DevData &d, const StageArgs &a, const EqEval &ev, int c, double phi,
                                           double *base) {
  const int ld = d.ld;
#pragma unroll
  for (int v = 0; v < S::NV; ++v) base[v] = a.dev0[v * ld + c];
  if (EQ && eq_found(a, ld, c)) {
    double r, E;
    eq_bound(a, ld, c).at(ev, phi, r, E);
    base[0] += r;
    base[S::NV - 1] += E;
  }
}

template <class S, int FLUX, int EQ, bool MIXED>
__device__ __forceinline__ void face_one(const DevData &d, const Params &P, const StageArgs &a, const int e) {
  constexpr int NV = S::NV, ND = S::ND;
  if (e >= d.n_edges) return;
  if (d.clock->done) return;
  if (!d.factive[e]) return;
  const int lde = d.lde, ld = d.ld;
  const int L = d.fL[e], R = d.fR[e];
  EqEval ev{P.gamma, P.gm1, P.inv_gm1};
  double nf[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) nf[v] = 0.0;
  if (R >= 0) {
    const int kL = d.fkL[e], kR = d.fkR[e];
    double nf_rot[NV];  // contributions still in the face frame
#pragma unroll
    for (int v = 0; v < NV; ++v) nf_rot[v] = 0.0;
    float g32[NV], mL[ND], mR[ND];
    bool any64 = false;  // some point added to the FP64 accumulators
#pragma unroll
    for (int v = 0; v < NV; ++v) g32[v] = 0.f;
#pragma unroll
    for (int k = 0; k < ND; ++k) mL[k] = mR[k] = 0.f;
#pragma unroll
    for (int qq = 0; qq < S::NQF; ++qq) {
      bool rotated = true;
      const size_t sL = (size_t)((kL * S::NQF + qq) * NV) * ld + L;
      const size_t sR = (size_t)((kR * S::NQF + qq) * NV) * ld + R;
      double f[NV];
      if (!MIXED) {
        double uL[NV], uR[NV], wL[NV], wR[NV];
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          uL[v] = a.fv[sL + (size_t)v * ld];
          uR[v] = a.fv[sR + (size_t)v * ld];
        }
        to_face<NV, ND>(uL, d.frame, lde, e, wL);
        to_face<NV, ND>(uR, d.frame, lde, e, wR);
        numerical_flux<NV, FLUX>(wL, wR, P.gamma, f);
      } else if (EQ && (P.gamma2 ? (a.eq32[2 * ld + L].x >= 0.f && a.eq32[2 * ld + R].x >= 0.f)
                                 : (eq_found(a, ld, L) && eq_found(a, ld, R)))) {
        // perturbation form around the left cell's equilibrium at the point:
        // F = (0, p_w n, 0) + [F32(w + dL, w + dR) - F32(w)] in the face frame
        // base w = the left equilibrium at the point; the right side carries
        // the difference of the two equilibria there
        float rwL, EwL, drho, dE;
        if (P.gamma2) {
          // gamma = 2: rho = f (h_r - phi), E = K rho^2, in FP32-pair arithmetic
          const DF phi = df_of(d.phi_fq2[qq * lde + e]);
          const DF rL = df_mul(df_of(a.eq32[ld + L]), df_sub(df_of(a.eq32[L]), phi));
          const DF rR = df_mul(df_of(a.eq32[ld + R]), df_sub(df_of(a.eq32[R]), phi));
          const DF EL = df_mul(df_of(a.eq32[2 * ld + L]), df_mul(rL, rL));
          const DF ER = df_mul(df_of(a.eq32[2 * ld + R]), df_mul(rR, rR));
          const DF dr = df_sub(rR, rL), dEE = df_sub(ER, EL);
          rwL = rL.hi;
          EwL = EL.hi;
          drho = __fadd_rn(dr.hi, dr.lo);
          dE = __fadd_rn(dEE.hi, dEE.lo);
        } else {
          const double phi = d.phi_fq[qq * lde + e];
          double rwL64, EwL64, rwR64, EwR64;
          eq_bound(a, ld, L).at(ev, phi, rwL64, EwL64);
          eq_bound(a, ld, R).at(ev, phi, rwR64, EwR64);
          rwL = float(rwL64);
          EwL = float(EwL64);
          drho = float(rwR64 - rwL64);
          dE = float(EwR64 - EwL64);
        }
        float cL[NV], cR[NV], dL[NV], dR[NV], df[NV];
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          cL[v] = a.dev032[v * ld + L];
          cR[v] = a.dev032[v * ld + R];
        }
        cR[0] += drho;
        cR[NV - 1] += dE;
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          cL[v] += a.fv32[sL + (size_t)v * ld];
          cR[v] += a.fv32[sR + (size_t)v * ld];
        }
        to_face32<NV, ND>(cL, d.frame32, lde, e, dL);
        to_face32<NV, ND>(cR, d.frame32, lde, e, dR);
        const float gamma32 = P.gamma32;
        if (FLUX == 0)
          hllc_flux_dev<NV>(dL, dR, rwL, EwL, gamma32, df);
        else
          rusanov_flux_dev<NV>(dL, dR, rwL, EwL, gamma32, df);
        from_face32<NV, ND>(df, d.frame32, lde, e);
        // the baseline p_wL n cancels the left cell's own surface source term
        // exactly; the right cell keeps (p_wL - p_eqR) n
        const float wq = d.fqw32[qq * lde + e];
        const float dpn = -dE * (gamma32 - 1.f) * wq;
#pragma unroll
        for (int v = 0; v < NV; ++v) g32[v] += wq * df[v];
#pragma unroll
        for (int k = 0; k < ND; ++k) mR[k] += dpn * d.frame32[k * lde + e];
        continue;
      } else if (!EQ) {
        // plain FP32 flux of the FP32 face states
        float uL[NV], uR[NV], wL[NV], wR[NV], f32[NV];
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          uL[v] = a.dev032[v * ld + L] + a.fv32[sL + (size_t)v * ld];
          uR[v] = a.dev032[v * ld + R] + a.fv32[sR + (size_t)v * ld];
        }
        to_face32<NV, ND>(uL, d.frame32, lde, e, wL);
        to_face32<NV, ND>(uR, d.frame32, lde, e, wR);
        numerical_flux<NV, FLUX>(wL, wR, P.gamma32, f32);
        from_face32<NV, ND>(f32, d.frame32, lde, e);
        const float wq = d.fqw32[qq * lde + e];
#pragma unroll
        for (int v = 0; v < NV; ++v) g32[v] += wq * f32[v];
        continue;
      } else {
        // a side without equilibrium: FP64 flux of base + polynomial part
        const double phi = d.phi_fq[qq * lde + e];
        double bL[NV], bR[NV], wL[NV], wR[NV];
        mixed_base<S, EQ>(d, a, ev, L, phi, bL);
        mixed_base<S, EQ>(d, a, ev, R, phi, bR);
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          bL[v] += double(a.fv32[sL + (size_t)v * ld]);
          bR[v] += double(a.fv32[sR + (size_t)v * ld]);
        }
        to_face<NV, ND>(bL, d.frame, lde, e, wL);
        to_face<NV, ND>(bR, d.frame, lde, e, wR);
        numerical_flux<NV, FLUX>(wL, wR, P.gamma, f);
        // surface source terms of the sides that have an equilibrium
        double rq, Eq;
        const float wq32 = d.fqw32[qq * lde + e];
        if (eq_found(a, ld, L)) {
          eq_bound(a, ld, L).at(ev, phi, rq, Eq);
#pragma unroll
          for (int k = 0; k < ND; ++k) mL[k] += float(Eq * ev.gm1) * wq32 * d.frame32[k * lde + e];
        }
        if (eq_found(a, ld, R)) {
          eq_bound(a, ld, R).at(ev, phi, rq, Eq);
#pragma unroll
          for (int k = 0; k < ND; ++k) mR[k] -= float(Eq * ev.gm1) * wq32 * d.frame32[k * lde + e];
        }
      }
      any64 = true;
      const double wq = d.fqw[qq * lde + e];
      if (rotated) {
#pragma unroll
        for (int v = 0; v < NV; ++v) nf_rot[v] += wq * f[v];
      } else {
#pragma unroll
        for (int v = 0; v < NV; ++v) nf[v] += wq * f[v];
      }
    }
    if (!MIXED || any64) {
      from_face<NV, ND>(nf_rot, d.frame, lde, e);
#pragma unroll
      for (int v = 0; v < NV; ++v) nf[v] += nf_rot[v];
    }
    if (MIXED) {
#pragma unroll
      for (int v = 0; v < NV; ++v) a.g32[v * lde + e] = any64 ? g32[v] + float(nf[v]) : g32[v];
#pragma unroll
      for (int k = 0; k < ND; ++k) {
        a.mL32[k * lde + e] = mL[k];
        a.mR32[k * lde + e] = mR[k];
      }
      return;
    }
  } else if (P.flux_bc == 1) {
    // FluxBC (boundary/flux_bc.hpp:25-42): physical flux of the cell average
    double u[NV], w[NV], f[NV];
    const int j = d.l2g[L];
#pragma unroll
    for (int v = 0; v < NV; ++v) u[v] = a.q[v * ld + j];
    to_face<NV, ND>(u, d.frame, lde, e, w);
    euler_flux<NV>(w, pressure<NV>(w, P.gamma), f);
    from_face<NV, ND>(f, d.frame, lde, e);
    const double area = d.farea[e];
#pragma unroll
    for (int v = 0; v < NV; ++v) nf[v] = area * f[v];
  } else if (P.flux_bc == 2 && MIXED) {
    // EquilibriumFluxBC: F = p_eq n on the face equals the cell's own surface
    // source term there, so the pair contributes nothing
  } else if (P.flux_bc == 2) {
    // EquilibriumFluxBC (boundary/equilibrium_flux_bc.hpp:36-62): the equilibrium
    // of the boundary cell extrapolated to the face; zero velocity, so F = p n.
    if (eq_found(a, ld, L)) {
      const EqEval::Bound b = eq_bound(a, ld, L);
      double pn = 0.0;
#pragma unroll
      for (int qq = 0; qq < S::NQF; ++qq) {
        double r, E;
        b.at(ev, d.phi_fq[qq * lde + e], r, E);
        pn += d.fqw[qq * lde + e] * (E * ev.gm1);
      }
#pragma unroll
      for (int k = 0; k < ND; ++k) nf[1 + k] = pn * d.frame[k * lde + e];
    }
  }
  if constexpr (MIXED) {
    // boundary face: flux of the cell average (FluxBC); with an equilibrium and
    // no FluxBC the cell's surface source term on this face remains
    float mLb[ND];
#pragma unroll
    for (int k = 0; k < ND; ++k) mLb[k] = 0.f;
    if (EQ && P.flux_bc != 2 && eq_found(a, ld, L)) {
      const EqEval::Bound b = eq_bound(a, ld, L);
#pragma unroll
      for (int qq = 0; qq < S::NQF; ++qq) {
        double r, E;
        b.at(ev, d.phi_fq[qq * lde + e], r, E);
        const float pw = float(E * ev.gm1 * d.fqw[qq * lde + e]);
#pragma unroll
        for (int k = 0; k < ND; ++k) mLb[k] += pw * d.frame32[k * lde + e];
      }
    }
#pragma unroll
    for (int v = 0; v < NV; ++v) a.g32[v * lde + e] = float(nf[v]);
#pragma unroll
    for (int k = 0; k < ND; ++k) {
      a.mL32[k * lde + e] = mLb[k];
      a.mR32[k * lde + e] = 0.f;
    }
  } else {
#pragma unroll
    for (int v = 0; v < NV; ++v) a.nf[v * lde + e] = nf[v];
  }
}

// Blocks of 128 threads per SM the face kernel is held to: the mixed
// well-balanced fluxes are latency-bound on their gathers and gain from more
// resident warps even with the spills a tight bound brings (2D: 48 registers,
// ten blocks, 0.40-0.74 KB of spills per thread; 3D: 64 registers, eight
// blocks).  Measured per launch: batched C4 ensemble of 48 disks 0.204 ms at
// the compiler's 118 registers and four blocks, 0.180 at 96 and five, 0.120
// now; 384,000 tetrahedra 0.138 ms at 126 registers and four blocks, 0.098
// now.  The mixed form without well-balancing takes the same bounds (C3 vortex
// tube, 2,058,000 tetrahedra: 0.272 -> 0.250 ms); the FP64 form, bound by its
// FP64 pipe, keeps the compiler's choice.
template <class S, int EQ, bool MIXED>
constexpr int kFaceBlocks = MIXED ? (S::ND == 2 ? 10 : 8) : 1;

template <class S, int FLUX, int EQ, bool MIXED>
__global__ void __launch_bounds__(128, (kFaceBlocks<S, EQ, MIXED>)) k_face_flux(const DevData d, const Params P, StageArgs a) {
  face_one<S, FLUX, EQ, MIXED>(d, P, a, blockIdx.x * blockDim.x + threadIdx.x);
}

// ---------------------------------------------------------------- update
template <int NV>
__device__ __forceinline__ double cfl_candidate(const double *u, double gamma, double r) {
  double m2 = 0.0;
#pragma unroll
  for (int k = 1; k < NV - 1; ++k) m2 += u[k] * u[k];
  double v2 = m2 / (u[0] * u[0]);
  double p = pressure<NV>(u, gamma);
  double c = sqrt(gamma * p / u[0]);
  return r / (sqrt(v2) + c);
}

// The mixed form's CFL candidate r / (|m| / rho + sqrt(gamma p / rho)),
// p = (gamma - 1) (E - |m|^2 / (2 rho)), in FP32 from the FP32 high parts of
// the new state: the time step carries FP32 precision, far more than the CFL
// bound needs, and the FP64 square roots and divisions leave the FP64 pipe.
template <int NV>
__device__ __forceinline__ float cfl_candidate_f32(const float *u, float gamma, float r) {
  float m2 = 0.f;
#pragma unroll
  for (int k = 1; k < NV - 1; ++k) m2 += u[k] * u[k];
  const float ir = 1.f / u[0];
  const float p = (u[NV - 1] - 0.5f * m2 * ir) * (gamma - 1.f);
  return r / (sqrtf(m2) * ir + sqrtf(gamma * p * ir));
}

__device__ __forceinline__ void block_min_to_clock(double cand, Clock *clock) {
  // positive doubles order like their bit patterns; NaN bits sort above +inf
  unsigned long long bits = __double_as_longlong(cand);
  if (!(cand >= 0.0)) bits = 0x7ff0000000000000ull;  // ignored: status flags the state
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long other = __shfl_xor_sync(0xffffffffu, bits, o);
    bits = other < bits ? other : bits;
  }
  __shared__ unsigned long long warp_min[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) warp_min[wid] = bits;
  __syncthreads();
  if (wid == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    bits = lane < nw ? warp_min[lane] : 0x7ff0000000000000ull;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      unsigned long long other = __shfl_xor_sync(0xffffffffu, bits, o);
      bits = other < bits ? other : bits;
    }
    if (lane == 0) atomicMin(&clock->cfl_min, bits);
  }
}

// One cell of the stage update; returns the CFL candidate of the new state at
// the last stage (+inf otherwise).
template <class S, bool MIXED>
__device__ __forceinline__ double update_cell(const DevData &d, const Params &P, const StageArgs &a, const int i) {
  constexpr int NV = S::NV, NF = S::NF, ND = S::ND;
  const bool last = a.stage == P.n_stages - 1;
  double cand = INFINITY;
  if (!d.clock->done && i < d.n_cells && (d.flags[i] & kInterior)) {
    const int ld = d.ld, lde = d.lde;
    double tend[NV];
    float t32[NV];  // mixed form: the tendency in FP32
    if (MIXED) {
      // deviation-sized terms only: FP32 sums
#pragma unroll
      for (int v = 0; v < NV; ++v) t32[v] = 0.f;
#pragma unroll
      for (int f = 0; f < NF; ++f) {
        const int cf = d.cface[f * ld + i];
        if (cf < 0) continue;
        const int e = cf >> 1;
        const bool right = cf & 1;
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          const float x = a.g32[v * lde + e];
          t32[v] += right ? x : -x;
        }
        const float *m = right ? a.mR32 : a.mL32;
#pragma unroll
        for (int k = 0; k < ND; ++k) t32[1 + k] += m[k * lde + e];
      }
      const float iv = float(d.inv_vol[i]);
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        t32[v] *= iv;
        if (a.src32) t32[v] += a.src32[v * ld + i];
        tend[v] = double(t32[v]);
      }
    } else {
#pragma unroll
      for (int v = 0; v < NV; ++v) tend[v] = 0.0;
#pragma unroll
      for (int f = 0; f < NF; ++f) {
        const int cf = d.cface[f * ld + i];
        if (cf < 0) continue;
        const int e = cf >> 1;
        const bool right = cf & 1;
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          const double x = a.nf[v * lde + e];
          tend[v] += right ? x : -x;
        }
      }
      const double iv = d.inv_vol[i];
#pragma unroll
      for (int v = 0; v < NV; ++v) tend[v] *= iv;
      if (a.src) {
#pragma unroll
        for (int v = 0; v < NV; ++v) tend[v] += a.src[v * ld + i];
      }
    }
    if (a.tend_out) {
#pragma unroll
      for (int v = 0; v < NV; ++v) a.tend_out[v * ld + i] = tend[v];
    } else {
      const int s = a.stage;
      const double dt = d.clock->dt;
      double un[NV];
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        if (MIXED) {
          // FP32 stage tendencies combined in FP32; the cell average itself
          // accumulates in FP64
          float dudt = 0.f;
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            if (j > s) break;
            const float c = a.coef32[j];
            if (c != 0.f) dudt += c * (j == s ? t32[v] : a.k32[j][v * ld + i]);
          }
          un[v] = a.u0[v * ld + i] + dt * double(dudt);
        } else {
          double dudt = 0.0;
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            if (j > s) break;
            const double c = a.coef[j];
            if (c != 0.0) dudt += c * (j == s ? tend[v] : a.k[j][v * ld + i]);
          }
          un[v] = a.u0[v * ld + i] + dt * dudt;
        }
      }
      float cand32 = INFINITY;  // mixed form: CFL candidate from the FP32 high parts
      if (MIXED) {
        float hi[NV];
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          const DF x = df_split(un[v]);
          a.qs_next[v * ld + i] = make_float2(x.hi, x.lo);
          hi[v] = x.hi;
        }
        if (last) cand32 = cfl_candidate_f32<NV>(hi, P.gamma32, float(d.r_eff[i]));
      }
      if (!last) {
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          if (MIXED)
            a.k32[s][v * ld + i] = t32[v];
          else
            a.k[s][v * ld + i] = tend[v];
          a.ux[v * ld + i] = un[v];
        }
      } else {
        if (a.uprev) {
          // RejectLargeDensityChange::check: |rho_1 - rho_0| > drho_crit rho_0 in any cell
          const double rho0 = a.u0[i];
#pragma unroll
          for (int v = 0; v < NV; ++v) a.uprev[v * ld + i] = a.u0[v * ld + i];
          if (fabs(un[0] - rho0) > d.clock->reject_drho * rho0) atomicOr(&d.clock->rejected, 1);
        }
#pragma unroll
        for (int v = 0; v < NV; ++v) a.u0[v * ld + i] = un[v];
        cand = MIXED ? double(cand32) : cfl_candidate<NV>(un, P.gamma, d.r_eff[i]);
        bool finite = true;
#pragma unroll
        for (int v = 0; v < NV; ++v) finite = finite && isfinite(un[v]);
        if (!finite) set_status(d.clock, kStNonFinite);
      }
    }
  } else if (last && !a.tend_out && !d.clock->done && i < d.n_cells && (d.flags[i] & kFrozen)) {
    // a frozen ghost cell keeps its state; LocalCFL still counts it
    double w[NV];
    float w32[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) w[v] = a.u0[v * d.ld + i], w32[v] = float(w[v]);
    cand = MIXED ? double(cfl_candidate_f32<NV>(w32, P.gamma32, float(d.r_eff[i])))
                 : cfl_candidate<NV>(w, P.gamma, d.r_eff[i]);
  }
  return cand;
}

template <class S, bool MIXED>
__global__ void __launch_bounds__(128) k_update(const DevData d, const Params P, StageArgs a) {
  const double cand = update_cell<S, MIXED>(d, P, a, blockIdx.x * blockDim.x + threadIdx.x);
  if (a.stage == P.n_stages - 1 && !a.tend_out) block_min_to_clock(cand, d.clock);
}

template <class S>
__global__ void __launch_bounds__(128) k_cfl(const DevData d, const Params P, const double *u, int mixed) {
  constexpr int NV = S::NV;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double cand = INFINITY;
  if (i < d.n_cells && (d.flags[i] & (kInterior | kFrozen))) {
    double w[NV];
    float w32[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) w[v] = u[v * d.ld + i], w32[v] = float(w[v]);
    // the mixed form's candidate is the one its update computes, so a state
    // set from the host (a restart) continues with the same time steps
    cand = mixed ? double(cfl_candidate_f32<NV>(w32, P.gamma32, float(d.r_eff[i])))
                 : cfl_candidate<NV>(w, P.gamma, d.r_eff[i]);
  }
  block_min_to_clock(cand, d.clock);
}

// TimeLoop::reject_step: put back the saved start of a rejected step (interior
// cells; ghost cells never change) and, in the mixed form, its FP32 pairs.
template <int NV>
__global__ void k_restore(const Clock *clock, const uint8_t *flags, const double *uprev, double *u0, float2 *pairs,
                          int n, int ld) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || !clock->restore || !(flags[i] & kInterior)) return;
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    const double x = uprev[(size_t)v * ld + i];
    u0[(size_t)v * ld + i] = x;
    if (pairs) {
      const DF p = df_split(x);
      pairs[(size_t)v * ld + i] = make_float2(p.hi, p.lo);
    }
  }
}

// ------------------------------------------------- multi-instance kernels
// A batch packs many independent solves (meshes of any size) into one launch
// per phase: a persistent grid walks a list of 128-item tiles, each tile
// belonging to one instance, whose argument structs live in device memory.
// Every instance keeps its own clock (its own CFL time step and end time).
struct BatchInst {
  DevData d;
  Params P;
  StageArgs a[3];
};

struct Tile {
  int slot, begin;
};

// The batched kernels run blocks of BS threads over tiles of BS cells or
// faces (BS = 64, 128 or 256, picked per group by the autotuner).  The mixed
// reconstruction keeps the single-solver kernel's register budget per thread:
// its per-shape bound of blocks per SM scaled to the block size.
template <class S, int EQ, int BS>
constexpr int kBatchReconBlocks = (kMixedReconBlocks<S, EQ> * 128 + BS - 1) / BS;

template <class S, int EQ, int SRC, bool MIXED, int BS>
__global__ void __launch_bounds__(BS) km_reconstruct(const BatchInst *__restrict__ inst,
                                                     const Tile *__restrict__ tiles, int n_tiles, int stage) {
  for (int t = blockIdx.x; t < n_tiles; t += gridDim.x) {
    const Tile tl = tiles[t];
    const BatchInst &I = inst[tl.slot];
    recon_cell<S, EQ, SRC, MIXED>(I.d, I.P, I.a[stage], tl.begin + threadIdx.x);
  }
}

template <class S, int EQ, int SRC, bool MIXED, int BS>
__global__ void __launch_bounds__(BS, (kBatchReconBlocks<S, EQ, BS>)) km_reconstruct_mixed(
    const BatchInst *__restrict__ inst, const Tile *__restrict__ tiles, int n_tiles, int stage) {
  for (int t = blockIdx.x; t < n_tiles; t += gridDim.x) {
    const Tile tl = tiles[t];
    const BatchInst &I = inst[tl.slot];
    recon_cell<S, EQ, SRC, MIXED>(I.d, I.P, I.a[stage], tl.begin + threadIdx.x);
  }
}

template <class S, int EQ, int SRC, bool MIXED, int BS>
constexpr auto batch_recon_kernel() {
  if constexpr (MIXED)
    return &km_reconstruct_mixed<S, EQ, SRC, MIXED, BS>;
  else
    return &km_reconstruct<S, EQ, SRC, MIXED, BS>;
}

// The batched face kernel takes the single-solver kernel's register budget per
// thread (kFaceBlocks 128-thread blocks per SM, scaled to the block size).
template <class S, int EQ, bool MIXED, int BS>
constexpr int kBatchFaceBlocks = (kFaceBlocks<S, EQ, MIXED> * 128 + BS - 1) / BS;

template <class S, int FLUX, int EQ, bool MIXED, int BS>
__global__ void __launch_bounds__(BS, (kBatchFaceBlocks<S, EQ, MIXED, BS>)) km_face_flux(const BatchInst *__restrict__ inst,
                                                   const Tile *__restrict__ tiles, int n_tiles, int stage) {
  for (int t = blockIdx.x; t < n_tiles; t += gridDim.x) {
    const Tile tl = tiles[t];
    const BatchInst &I = inst[tl.slot];
    face_one<S, FLUX, EQ, MIXED>(I.d, I.P, I.a[stage], tl.begin + threadIdx.x);
  }
}

template <class S, bool MIXED, int BS>
__global__ void __launch_bounds__(BS) km_update(const BatchInst *__restrict__ inst, const Tile *__restrict__ tiles,
                                                int n_tiles, int stage) {
  for (int t = blockIdx.x; t < n_tiles; t += gridDim.x) {
    const Tile tl = tiles[t];
    const BatchInst &I = inst[tl.slot];
    const double cand = update_cell<S, MIXED>(I.d, I.P, I.a[stage], tl.begin + threadIdx.x);
    // block-uniform: the whole tile belongs to one instance
    if (stage == I.P.n_stages - 1) block_min_to_clock(cand, I.d.clock);
    __syncthreads();
  }
}

struct BatchCfg {
  bool eq, src, mixed;
  int flux;
  int block = 128;                         // threads per block = cells or faces per tile
  int grid_recon, grid_face, grid_update;  // persistent grid sizes (autotuned; 0: one block per tile)
  cudaStream_t stream;
  cudaEvent_t *ev = nullptr;  // optional: 4 events recorded around the three stage kernels
};

template <class S, bool MIXED, int BS>
void launch_batch_stage_p(const BatchInst *inst, const Tile *cell_tiles, int n_ct, const Tile *face_tiles, int n_ft,
                          int stage, const BatchCfg &c) {
  const int gr = c.grid_recon > 0 ? c.grid_recon : n_ct, gf = c.grid_face > 0 ? c.grid_face : n_ft,
            gu = c.grid_update > 0 ? c.grid_update : n_ct;
  if (c.ev) cudaEventRecord(c.ev[0], c.stream);
  if (c.eq && c.src)
    batch_recon_kernel<S, 1, 1, MIXED, BS>()<<<gr, BS, recon_smem_bytes<S, 1, MIXED>(BS), c.stream>>>(inst, cell_tiles,
                                                                                                     n_ct, stage);
  else if (c.eq)
    batch_recon_kernel<S, 1, 0, MIXED, BS>()<<<gr, BS, recon_smem_bytes<S, 1, MIXED>(BS), c.stream>>>(inst, cell_tiles,
                                                                                                     n_ct, stage);
  else if (c.src)
    batch_recon_kernel<S, 0, 1, MIXED, BS>()<<<gr, BS, recon_smem_bytes<S, 0, MIXED>(BS), c.stream>>>(inst, cell_tiles,
                                                                                                     n_ct, stage);
  else
    batch_recon_kernel<S, 0, 0, MIXED, BS>()<<<gr, BS, recon_smem_bytes<S, 0, MIXED>(BS), c.stream>>>(inst, cell_tiles,
                                                                                                     n_ct, stage);
  if (c.ev) cudaEventRecord(c.ev[1], c.stream);
  if (c.flux == 0) {
    if (c.eq)
      km_face_flux<S, 0, 1, MIXED, BS><<<gf, BS, 0, c.stream>>>(inst, face_tiles, n_ft, stage);
    else
      km_face_flux<S, 0, 0, MIXED, BS><<<gf, BS, 0, c.stream>>>(inst, face_tiles, n_ft, stage);
  } else {
    if (c.eq)
      km_face_flux<S, 1, 1, MIXED, BS><<<gf, BS, 0, c.stream>>>(inst, face_tiles, n_ft, stage);
    else
      km_face_flux<S, 1, 0, MIXED, BS><<<gf, BS, 0, c.stream>>>(inst, face_tiles, n_ft, stage);
  }
  if (c.ev) cudaEventRecord(c.ev[2], c.stream);
  km_update<S, MIXED, BS><<<gu, BS, 0, c.stream>>>(inst, cell_tiles, n_ct, stage);
  if (c.ev) cudaEventRecord(c.ev[3], c.stream);
}

// Occupancy-limited block counts of the three batch kernels (for the autotuner).
// (it also lifts the reconstruction kernels' dynamic shared-memory limit above
// the 48 KB default where a block size needs it: the autotuner calls it for
// every block size before it captures a launch with that size)
template <class S, bool MIXED, int BS>
void batch_occupancy_p(int *blocks_per_sm) {
  auto occ = [](const void *k, size_t smem = 0) {
    if (smem > 48 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int b = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k, BS, smem);
    return b;
  };
  occ((const void *)batch_recon_kernel<S, 1, 0, MIXED, BS>(), recon_smem_bytes<S, 1, MIXED>(BS));
  blocks_per_sm[0] = occ((const void *)batch_recon_kernel<S, 1, 1, MIXED, BS>(), recon_smem_bytes<S, 1, MIXED>(BS));
  blocks_per_sm[1] = occ((const void *)km_face_flux<S, 0, 1, MIXED, BS>);
  blocks_per_sm[2] = occ((const void *)km_update<S, MIXED, BS>);
}

// ------------------------------------------------------------ launching
}  // namespace dev
}  // namespace zfvm

#include "tracer_kernels.cuh"

namespace zfvm {
namespace dev {

struct LaunchCfg {
  int n_cells, n_edges;
  bool eq, src, mixed;
  int flux;
  cudaStream_t stream;
  cudaEvent_t *ev;  // optional: 4 events recorded around the three stage kernels
};

// 2D CWENO-AO order 3: central 11 cells (A 10x5), three one-sided 4 cells (A 3x2)
using S2o3 = Shape<2, 10, 5, 3, 3, 2, 2, 4>;
// 2D order 2 ({2,2,2,2}, overfit {3,2,2,2}): central 7 (6x2), one-sided 5 (4x2)
using S2o2 = Shape<2, 6, 2, 3, 4, 2, 2, 4>;
// 3D order 3 (overfit {2,1.5,...}): central 19 (18x9), one-sided 5 (4x3);
// degree-2 rules: 3 points per face, 4 per tetrahedron
using S3o3 = Shape<3, 18, 9, 4, 4, 3, 3, 4>;
// 3D order 2 (overfit {3,2,...}): central 10 (9x3), one-sided 7 (6x3)
using S3o2 = Shape<3, 9, 3, 4, 6, 3, 3, 4>;

template <class S, bool MIXED>
void launch_stage_p(const DevData &D, const Params &P, StageArgs &a, const LaunchCfg &c) {
  const int nb = (c.n_cells + 127) / 128, nbe = (c.n_edges + 127) / 128;
  if (c.ev) cudaEventRecord(c.ev[0], c.stream);
  if (c.eq && c.src)
    recon_kernel<S, 1, 1, MIXED>()<<<nb, 128, recon_smem_bytes<S, 1, MIXED>(128), c.stream>>>(D, P, a);
  else if (c.eq)
    recon_kernel<S, 1, 0, MIXED>()<<<nb, 128, recon_smem_bytes<S, 1, MIXED>(128), c.stream>>>(D, P, a);
  else if (c.src)
    recon_kernel<S, 0, 1, MIXED>()<<<nb, 128, recon_smem_bytes<S, 0, MIXED>(128), c.stream>>>(D, P, a);
  else
    recon_kernel<S, 0, 0, MIXED>()<<<nb, 128, recon_smem_bytes<S, 0, MIXED>(128), c.stream>>>(D, P, a);
  if (c.ev) cudaEventRecord(c.ev[1], c.stream);
  if (c.flux == 0) {
    if (c.eq)
      k_face_flux<S, 0, 1, MIXED><<<nbe, 128, 0, c.stream>>>(D, P, a);
    else
      k_face_flux<S, 0, 0, MIXED><<<nbe, 128, 0, c.stream>>>(D, P, a);
  } else {
    if (c.eq)
      k_face_flux<S, 1, 1, MIXED><<<nbe, 128, 0, c.stream>>>(D, P, a);
    else
      k_face_flux<S, 1, 0, MIXED><<<nbe, 128, 0, c.stream>>>(D, P, a);
  }
  if (c.ev) cudaEventRecord(c.ev[2], c.stream);
  k_update<S, MIXED><<<nb, 128, 0, c.stream>>>(D, P, a);
  if (c.ev) cudaEventRecord(c.ev[3], c.stream);
}

// Reconstruction with the polynomial export (zfvm_reconstruct); a separate
// instantiation so the stage kernels carry none of it.
template <class S, int EQ, int SRC, bool MIXED>
__global__ void __launch_bounds__(128) k_reconstruct_export(const DevData d, const Params P, StageArgs a) {
  recon_cell<S, EQ, SRC, MIXED, true>(d, P, a, blockIdx.x * blockDim.x + threadIdx.x);
}

template <class S, bool MIXED>
void launch_export_p(const DevData &D, const Params &P, StageArgs &a, const LaunchCfg &c) {
  const int nb = (c.n_cells + 127) / 128;
  if (c.eq && c.src)
    k_reconstruct_export<S, 1, 1, MIXED><<<nb, 128, recon_smem_bytes<S, 1, MIXED>(128), c.stream>>>(D, P, a);
  else if (c.eq)
    k_reconstruct_export<S, 1, 0, MIXED><<<nb, 128, recon_smem_bytes<S, 1, MIXED>(128), c.stream>>>(D, P, a);
  else if (c.src)
    k_reconstruct_export<S, 0, 1, MIXED><<<nb, 128, recon_smem_bytes<S, 0, MIXED>(128), c.stream>>>(D, P, a);
  else
    k_reconstruct_export<S, 0, 0, MIXED><<<nb, 128, recon_smem_bytes<S, 0, MIXED>(128), c.stream>>>(D, P, a);
}

template <class S>
void launch_cfl_t(const DevData &D, const Params &P, const double *u, const LaunchCfg &c) {
  const int nb = (c.n_cells + 127) / 128;
  k_cfl<S><<<nb, 128, 0, c.stream>>>(D, P, u, c.mixed ? 1 : 0);
}

// Instantiation: inst_shape.cu is compiled once per (shape, precision, single
// solver or batch) so the sixteen kernel sets build in parallel; the shape-level
// entry points below pick the precision at run time.
#define ZFVM_DECLARE_SHAPE_BATCH_BS(name, sfx, bs)                                                         \
  void launch_batch_stage_##name##_##sfx##_b##bs(const BatchInst *inst, const Tile *ct, int n_ct, const Tile *ft, \
                                                 int n_ft, int stage, const BatchCfg &c);                         \
  void batch_occupancy_##name##_##sfx##_b##bs(int *blocks_per_sm);
#define ZFVM_DECLARE_SHAPE_PREC(name, sfx)                                                                \
  void launch_stage_##name##_##sfx(const DevData &D, const Params &P, StageArgs &a, const LaunchCfg &c);  \
  void launch_export_##name##_##sfx(const DevData &D, const Params &P, StageArgs &a, const LaunchCfg &c); \
  void launch_tracer_##name##_##sfx(const DevData &D, const Params &P, StageArgs &a, TracerArgs &ta,      \
                                    const LaunchCfg &c);                                                  \
  ZFVM_DECLARE_SHAPE_BATCH_BS(name, sfx, 64)                                                              \
  ZFVM_DECLARE_SHAPE_BATCH_BS(name, sfx, 128)                                                             \
  ZFVM_DECLARE_SHAPE_BATCH_BS(name, sfx, 256)                                                             \
  inline void launch_batch_stage_##name##_##sfx(const BatchInst *inst, const Tile *ct, int n_ct, const Tile *ft, \
                                                int n_ft, int stage, const BatchCfg &c) {                 \
    if (c.block == 64)                                                                                    \
      launch_batch_stage_##name##_##sfx##_b64(inst, ct, n_ct, ft, n_ft, stage, c);                        \
    else if (c.block == 256)                                                                              \
      launch_batch_stage_##name##_##sfx##_b256(inst, ct, n_ct, ft, n_ft, stage, c);                       \
    else                                                                                                  \
      launch_batch_stage_##name##_##sfx##_b128(inst, ct, n_ct, ft, n_ft, stage, c);                       \
  }                                                                                                       \
  inline void batch_occupancy_##name##_##sfx(int block, int *blocks_per_sm) {                             \
    if (block == 64)                                                                                      \
      batch_occupancy_##name##_##sfx##_b64(blocks_per_sm);                                                \
    else if (block == 256)                                                                                \
      batch_occupancy_##name##_##sfx##_b256(blocks_per_sm);                                               \
    else                                                                                                  \
      batch_occupancy_##name##_##sfx##_b128(blocks_per_sm);                                               \
  }
#define ZFVM_DECLARE_SHAPE(name)                                                                          \
  ZFVM_DECLARE_SHAPE_PREC(name, f64)                                                                      \
  ZFVM_DECLARE_SHAPE_PREC(name, mix)                                                                      \
  void launch_cfl_##name(const DevData &D, const Params &P, const double *u, const LaunchCfg &c);         \
  inline void launch_stage_##name(const DevData &D, const Params &P, StageArgs &a, const LaunchCfg &c) {  \
    c.mixed ? launch_stage_##name##_mix(D, P, a, c) : launch_stage_##name##_f64(D, P, a, c);              \
  }                                                                                                       \
  inline void launch_export_##name(const DevData &D, const Params &P, StageArgs &a, const LaunchCfg &c) { \
    c.mixed ? launch_export_##name##_mix(D, P, a, c) : launch_export_##name##_f64(D, P, a, c);            \
  }                                                                                                       \
  inline void launch_tracer_##name(const DevData &D, const Params &P, StageArgs &a, TracerArgs &ta,       \
                                   const LaunchCfg &c) {                                                  \
    c.mixed ? launch_tracer_##name##_mix(D, P, a, ta, c) : launch_tracer_##name##_f64(D, P, a, ta, c);    \
  }                                                                                                       \
  inline void launch_batch_stage_##name(const BatchInst *inst, const Tile *ct, int n_ct, const Tile *ft,  \
                                        int n_ft, int stage, const BatchCfg &c) {                         \
    c.mixed ? launch_batch_stage_##name##_mix(inst, ct, n_ct, ft, n_ft, stage, c)                         \
            : launch_batch_stage_##name##_f64(inst, ct, n_ct, ft, n_ft, stage, c);                        \
  }                                                                                                       \
  inline void batch_occupancy_##name(const BatchCfg &c, int *blocks_per_sm) {                             \
    c.mixed ? batch_occupancy_##name##_mix(c.block, blocks_per_sm)                                        \
            : batch_occupancy_##name##_f64(c.block, blocks_per_sm);                                       \
  }
// the single-solver kernels of one shape and precision (the FP64 unit also
// holds the shape's CFL pass)
#define ZFVM_DEFINE_SHAPE_SINGLE(name, S, MIXED, sfx)                                                      \
  void launch_stage_##name##_##sfx(const DevData &D, const Params &P, StageArgs &a, const LaunchCfg &c) {  \
    launch_stage_p<S, MIXED>(D, P, a, c);                                                                  \
  }                                                                                                        \
  void launch_export_##name##_##sfx(const DevData &D, const Params &P, StageArgs &a, const LaunchCfg &c) { \
    launch_export_p<S, MIXED>(D, P, a, c);                                                                 \
  }                                                                                                        \
  void launch_tracer_##name##_##sfx(const DevData &D, const Params &P, StageArgs &a, TracerArgs &ta,       \
                                    const LaunchCfg &c) {                                                  \
    launch_tracer_p<S, MIXED>(D, P, a, ta, c.n_cells, c.n_edges, c.eq, c.flux, c.stream);                  \
  }
#define ZFVM_DEFINE_SHAPE_CFL(name, S)                                                                     \
  void launch_cfl_##name(const DevData &D, const Params &P, const double *u, const LaunchCfg &c) {          \
    launch_cfl_t<S>(D, P, u, c);                                                                           \
  }
// the batched (persistent, multi-instance) kernels of one shape, precision and block size
#define ZFVM_DEFINE_SHAPE_BATCH(name, S, MIXED, sfx, bs)                                                   \
  void launch_batch_stage_##name##_##sfx##_b##bs(const BatchInst *inst, const Tile *ct, int n_ct,          \
                                                 const Tile *ft, int n_ft, int stage, const BatchCfg &c) { \
    launch_batch_stage_p<S, MIXED, bs>(inst, ct, n_ct, ft, n_ft, stage, c);                                \
  }                                                                                                        \
  void batch_occupancy_##name##_##sfx##_b##bs(int *blocks_per_sm) { batch_occupancy_p<S, MIXED, bs>(blocks_per_sm); }

ZFVM_DECLARE_SHAPE(s2o3)
ZFVM_DECLARE_SHAPE(s2o2)
ZFVM_DECLARE_SHAPE(s3o3)
ZFVM_DECLARE_SHAPE(s3o2)

}  // namespace dev
}  // namespace zfvm
