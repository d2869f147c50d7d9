// GB300 rate-of-change and SSP-RK time stepping: host side of the solver.
//
// One Runge-Kutta stage is three kernels (solver_kernels.cuh):
//   k_reconstruct  one thread per cell: stencil gather, local equilibrium,
//                  CWENO-AO combination, face-point values and gravity source;
//   k_face_flux    one thread per face: HLLC / Rusanov or the boundary flux;
//   k_update       one thread per cell: signed flux gather, RK stage
//                  combination and the CFL candidate of the new state.
// A one-thread k_clock kernel opens every step: it turns the CFL minimum of the
// previous step into dt, clips it to t_end and stops the loop when done, so the
// whole time loop replays from a CUDA graph without host round trips.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "mesh_obj.hpp"
#include "solver_kernels.cuh"

namespace zfvm {
namespace dev {

// mode 0: open a step; mode 1: close the last step only
__global__ void k_clock(Clock *c, double cfl, int mode) { clock_step(c, cfl, mode); }

// The whole clock from the host, passed by value as a launch argument: stream
// ordered like a copy, but with no host buffer to keep alive and no implicit
// synchronisation (a copy from pageable memory waits for the stream).
__global__ void k_clock_set(Clock *c, Clock v) { *c = v; }

// A new run's end condition, set on the device so no host round trip is needed.
__global__ void k_clock_reset(Clock *c, long long n_steps, double t_end, double fixed_dt, double reject_drho) {
  c->done = 0;
  c->started = 0;
  c->step = 0;
  c->n_steps = n_steps;
  c->t_end = t_end;
  c->fixed_dt = fixed_dt;
  c->reject_drho = reject_drho;
}

// state SoA (NV x ld) -> AoS (n x 5); the 2D layout drops the third momentum
__global__ void k_soa_to_aos(const double *soa, double *aos, int n, int ld, int nv, const int *src) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int j = src[i];
  double r[5] = {0, 0, 0, 0, 0};
  for (int v = 0; v < nv - 1; ++v) r[v] = soa[v * ld + j];
  r[4] = soa[(nv - 1) * ld + j];
  for (int v = 0; v < 5; ++v) aos[i * 5 + v] = r[v];
}

// TimeLoop::reject_step for the advected variables of interior cells.
__global__ void k_tracer_restore(const Clock *clock, const uint8_t *flags, const double *uprev, double *u0, int n,
                                 int ld, int na) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || !clock->restore || !(flags[i] & kInterior)) return;
  for (int t = 0; t < na; ++t) u0[(size_t)t * ld + i] = uprev[(size_t)t * ld + i];
}

// A state from the host in one pass: AoS rows -> the step state u0 and the
// stage state ux (SoA), and in the mixed form the FP32 (hi, lo) pairs of both.
__global__ void k_state_in(const double *aos, double *u0, double *ux, float2 *pairs, int n, int ld, int nv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const size_t half = (size_t)nv * ld;
  for (int v = 0; v < nv; ++v) {
    const double x = aos[i * 5 + (v == nv - 1 ? 4 : v)];
    u0[(size_t)v * ld + i] = x;
    ux[(size_t)v * ld + i] = x;
    if (pairs) {
      const float hi = __double2float_rn(x);
      const float2 p = make_float2(hi, __double2float_rn(x - (double)hi));
      pairs[(size_t)v * ld + i] = p;
      pairs[half + (size_t)v * ld + i] = p;
    }
  }
}

}  // namespace dev
}  // namespace zfvm

// ======================================================================= host
using namespace zfvm;
using namespace zfvm::dev;

#include "solver_obj.hpp"

using zfvm::CudaError;
using zfvm::DBuf;

namespace {

struct ShapeKey {
  int nd, R0, C0, NB, RB, CB, nqf, nqc;
};

template <class S>
bool matches(const ShapeKey &k) {
  return k.nd == S::ND && k.R0 == S::R0 && k.C0 == S::C0 && k.NB == S::NB && k.RB == S::RB &&
         k.CB == S::CB && k.nqf == S::NQF && k.nqc == S::NQC;
}


}  // namespace

StageArgs stage_args(zfvm_solver *s, int stage, double *tend_out) {
  StageArgs a{};
  a.q = stage == 0 ? s->u0.p : s->ux.p;
  a.fv = s->fv.p;
  a.fv32 = s->fv32.p;
  a.dev0 = s->dev0.p;
  a.dev032 = s->dev032.p;
  a.eq32 = s->eq32.p;
  a.uprev = s->uprev.p;
  a.sched_count = s->sched_count.p;
  a.sched = s->sched.p;
  a.nf = s->nfb.p;
  a.src = s->has_src ? s->srcb.p : nullptr;
  a.eqth = s->has_eq ? s->eqth.p : nullptr;
  a.u0 = s->u0.p;
  a.ux = s->ux.p;
  for (int k = 0; k < 4; ++k) a.k[k] = s->kbuf.p ? s->kbuf.p + (size_t)k * s->nv * s->ld : nullptr;
  a.tend_out = tend_out;
  a.g32 = s->g32.p;
  a.mL32 = s->mL32.p;
  a.mR32 = s->mR32.p;
  a.src32 = s->src32.p;
  for (int k = 0; k < 4; ++k) a.k32[k] = s->kbuf32.p ? s->kbuf32.p + (size_t)k * s->nv * s->ld : nullptr;
  a.stage = stage;
  const bool last = stage == s->P.n_stages - 1;
  for (int j = 0; j < 4; ++j) {
    a.coef[j] = last ? s->P.b[j] : (stage + 1 < 4 ? s->P.a[stage + 1][j] : 0.0);
    a.coef32[j] = (float)a.coef[j];
  }
  if (s->qsplit.p) {
    const size_t half = (size_t)s->nv * s->ld;
    a.qs = s->qsplit.p + (stage == 0 ? 0 : half);
    a.qs_next = s->qsplit.p + (last ? 0 : half);
  }
  return a;
}

TracerArgs tracer_args(zfvm_solver *s, int stage, double *tend_out) {
  TracerArgs t{};
  t.na = s->na;
  t.q = stage == 0 ? s->tq0.p : s->tqx.p;
  t.fv = s->tfv.p;
  t.nf = s->tnf.p;
  t.u0 = s->tq0.p;
  t.ux = s->tqx.p;
  for (int k = 0; k < 4; ++k) t.k[k] = s->tk.p ? s->tk.p + (size_t)k * s->na * s->ld : nullptr;
  t.tend_out = tend_out;
  t.uprev = s->tprev.p;
  return t;
}

namespace {

LaunchCfg launch_cfg(zfvm_solver *s) {
  return LaunchCfg{s->n_cells, s->n_edges,  s->has_eq, s->has_src, s->mixed,
                   s->scheme.flux == ZFVM_FLUX_HLLC ? 0 : 1, s->stream, nullptr};
}

void dispatch_stage(zfvm_solver *s, StageArgs &a, cudaEvent_t *ev = nullptr) {
  LaunchCfg c = launch_cfg(s);
  c.ev = ev;
  switch (s->shape_id) {
    case 0: launch_stage_s2o3(s->D, s->P, a, c); break;
    case 1: launch_stage_s2o2(s->D, s->P, a, c); break;
    case 2: launch_stage_s3o3(s->D, s->P, a, c); break;
    case 3: launch_stage_s3o2(s->D, s->P, a, c); break;
  }
  CK(cudaGetLastError());
}

// the advected variables' three kernels of a stage, after the stage's own
void dispatch_tracers(zfvm_solver *s, StageArgs &a, double *tend_out, cudaStream_t stream = nullptr) {
  if (!s->na) return;
  TracerArgs ta = tracer_args(s, a.stage, tend_out);
  LaunchCfg c = launch_cfg(s);
  if (stream) c.stream = stream;
  switch (s->shape_id) {
    case 0: launch_tracer_s2o3(s->D, s->P, a, ta, c); break;
    case 1: launch_tracer_s2o2(s->D, s->P, a, ta, c); break;
    case 2: launch_tracer_s3o3(s->D, s->P, a, ta, c); break;
    case 3: launch_tracer_s3o2(s->D, s->P, a, ta, c); break;
  }
  CK(cudaGetLastError());
}

void launch_cfl(zfvm_solver *s) {
  LaunchCfg c = launch_cfg(s);
  switch (s->shape_id) {
    case 0: launch_cfl_s2o3(s->D, s->P, s->u0.p, c); break;
    case 1: launch_cfl_s2o2(s->D, s->P, s->u0.p, c); break;
    case 2: launch_cfl_s3o3(s->D, s->P, s->u0.p, c); break;
    case 3: launch_cfl_s3o2(s->D, s->P, s->u0.p, c); break;
  }
  CK(cudaGetLastError());
}

// after every clock launch when step rejection is on: put back the start of a
// rejected step (a no-op launch otherwise)
void enqueue_restore(zfvm_solver *s, cudaStream_t stream = nullptr) {
  if (!s->uprev.p) return;
  if (!stream) stream = s->stream;
  const int nb = (s->n_cells + 127) / 128;
  if (s->nv == 4)
    k_restore<4><<<nb, 128, 0, stream>>>(s->clock.p, s->flags.p, s->uprev.p, s->u0.p, s->qsplit.p, s->n_cells, s->ld);
  else
    k_restore<5><<<nb, 128, 0, stream>>>(s->clock.p, s->flags.p, s->uprev.p, s->u0.p, s->qsplit.p, s->n_cells, s->ld);
  if (s->na)
    k_tracer_restore<<<nb, 128, 0, stream>>>(s->clock.p, s->flags.p, s->tprev.p, s->tq0.p, s->n_cells, s->ld, s->na);
  CK(cudaGetLastError());
}

void close_step(zfvm_solver *s) {
  k_clock<<<1, 1, 0, s->stream>>>(s->clock.p, s->P.cfl, 1);
  CK(cudaGetLastError());
  enqueue_restore(s);
}

void enqueue_step(zfvm_solver *s) {
  k_clock<<<1, 1, 0, s->stream>>>(s->clock.p, s->P.cfl, 0);
  CK(cudaGetLastError());
  enqueue_restore(s);
  for (int st = 0; st < s->P.n_stages; ++st) {
    StageArgs a = stage_args(s, st, nullptr);
    dispatch_stage(s, a);
    dispatch_tracers(s, a, nullptr);
  }
}

}  // namespace

void solver_restore_on(zfvm_solver *s, cudaStream_t stream) { enqueue_restore(s, stream); }

void solver_dispatch_stage(zfvm_solver *s, StageArgs &a) { dispatch_stage(s, a); }

void solver_tracers_on(zfvm_solver *s, int stage, cudaStream_t stream) {
  StageArgs a = stage_args(s, stage, nullptr);
  dispatch_tracers(s, a, nullptr, stream);
}

void solver_close_step(zfvm_solver *s) { close_step(s); }

int status_to_code(int st, std::string &msg) {
  if (st & kStNewton) {
    msg = "local equilibrium solve is not converging";
    return ZFVM_ENEWTON;
  }
  if (st & kStNonPhysical) {
    msg = "non-physical state (rho <= 0 or E_int <= 0) in the scaling";
    return ZFVM_ENONPHYSICAL;
  }
  if (st & kStNonFinite) {
    msg = "non-finite state after a step";
    return ZFVM_ENONPHYSICAL;
  }
  return ZFVM_OK;
}

Clock fresh_clock(const zfvm_solver *s, double t) {
  Clock c{};
  c.t = t;
  c.cfl_min = 0x7ff0000000000000ull;
  c.reject_drho = s->scheme.step_rejection_drho;
  c.factor = 1.0;
  c.min_factor = std::pow(2.0, -(double)std::max(0, s->scheme.step_rejection_max_exponent));
  c.good_prev = 1;
  return c;
}

Clock read_clock(zfvm_solver *s) {
  Clock c;
  CK(cudaMemcpyAsync(&c, s->clock.p, sizeof(Clock), cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  return c;
}

void write_clock(zfvm_solver *s, const Clock &c) {
  k_clock_set<<<1, 1, 0, s->stream>>>(s->clock.p, c);
  CK(cudaGetLastError());
}

namespace {

int build_solver(zfvm_solver *s) {
  zfvm_mesh *m = s->mesh;
  const Grid &g = m->grid;
  const StencilFamilies &fam = m->fam;
  const auto &sc = s->scheme;
  s->nd = g.n_dims;
  s->nv = g.n_dims + 2;
  s->nf = g.n_dims + 1;
  s->nqf = g.n_face_qp;
  s->nqc = g.n_cell_qp;
  // the counts and padded lengths below are ints; the table check further down
  // sets the real limit
  if (g.n_cells >= INT32_MAX - 64 || g.n_edges >= INT32_MAX - 64)
    return fail(ZFVM_EINVAL, "mesh too large for one solver; split it into instances of a batch");
  s->n_cells = (int)g.n_cells;
  s->n_edges = (int)g.n_edges;
  s->ld = (int)((g.n_cells + 31) / 32 * 32);
  s->lde = (int)((g.n_edges + 31) / 32 * 32);
  const int ld = s->ld, lde = s->lde, nd = s->nd, nv = s->nv, nf = s->nf;
  const index_t n = g.n_cells;

  // ---- shape of the stencil family
  const auto &sp = m->sparams;
  const int ns = (int)sp.orders.size();
  if (ns < 2 || sp.biased[0] != 0) return fail(ZFVM_EINVAL, "the first stencil must be the central one");
  for (int k = 2; k < ns; ++k)
    if (sp.orders[k] != sp.orders[1] || sp.overfit[k] != sp.overfit[1] || !sp.biased[k])
      return fail(ZFVM_EINVAL, "all one-sided stencils must share order and overfit factor");
  ShapeKey key;
  key.nd = nd;
  key.R0 = (int)required_stencil_size(sp.orders[0] - 1, sp.overfit[0], nd) - 1;
  key.C0 = poly_dof(sp.orders[0] - 1, nd) - 1;
  key.NB = ns - 1;
  key.RB = (int)required_stencil_size(sp.orders[1] - 1, sp.overfit[1], nd) - 1;
  key.CB = poly_dof(sp.orders[1] - 1, nd) - 1;
  key.nqf = s->nqf;
  key.nqc = s->nqc;
  if (matches<S2o3>(key))
    s->shape_id = 0;
  else if (matches<S2o2>(key))
    s->shape_id = 1;
  else if (matches<S3o3>(key))
    s->shape_id = 2;
  else if (matches<S3o2>(key))
    s->shape_id = 3;
  else
    return fail(ZFVM_EINVAL, "unsupported stencil / quadrature shape for the GPU kernels");
  const int R0 = key.R0, C0 = key.C0, NB = key.NB, RB = key.RB, CB = key.CB;
  const int NC = std::max(C0, CB), NP = R0 * C0 + NB * RB * CB, MAXL = R0 + 1 + NB * RB;
  // The kernels form 32-bit offsets row * ld + i into the per-cell tables (and
  // row * lde + e into the per-face ones); the tallest per-cell table is the
  // pseudo-inverses (NP rows) or the exported polynomial records.
  {
    const int64_t rows = std::max<int64_t>({(int64_t)NP, (int64_t)MAXL, (int64_t)nf * s->nqf * nv,
                                            (int64_t)s->nqc * nd, (int64_t)nv + (int64_t)NC * nv + nd + NC + 6});
    const int64_t face_rows = std::max<int64_t>({(int64_t)s->nqf * nd, (int64_t)nd * nd, (int64_t)nv});
    if (rows * ld >= INT32_MAX || face_rows * lde >= INT32_MAX)
      return fail(ZFVM_EINVAL, "mesh of " + std::to_string(g.n_cells) + " cells exceeds the kernels' 32-bit table offsets (" +
                                   std::to_string(INT32_MAX / rows) + " cells at most for this stencil shape); "
                                   "split it into instances of a batch");
  }

  // ---- scheme parameters
  if (sc.rk_stages < 1 || sc.rk_stages > 3) return fail(ZFVM_EINVAL, "rk_stages must be 1, 2 or 3");
  if (sc.steps_per_recompute < 1) return fail(ZFVM_EINVAL, "steps_per_recompute must be at least 1");
  s->has_eq = sc.equilibrium == ZFVM_EQ_ISENTROPIC;
  s->mixed = sc.precision == ZFVM_MIXED;
  s->has_src = sc.gravity != ZFVM_GRAVITY_NONE;
  if (s->has_eq && !s->has_src) return fail(ZFVM_EINVAL, "isentropic well-balancing needs gravity");
  if (sc.heating_rate != 0.0 && !s->has_src) return fail(ZFVM_EINVAL, "heating needs a gravity source here");
  if (sc.gravity < ZFVM_GRAVITY_NONE || sc.gravity > ZFVM_GRAVITY_RADIAL_TABLE)
    return fail(ZFVM_EINVAL, "unknown gravity kind");
  if (sc.flux_bc == ZFVM_FLUX_BC_ISENTROPIC && !s->has_eq)
    return fail(ZFVM_EINVAL, "isentropic flux boundary needs isentropic well-balancing");
  Params &P = s->P;
  P.gamma = sc.gamma;
  double tot = 0.0;
  for (int k = 0; k < ns; ++k) tot += sc.linear_weights[k];
  for (int k = 0; k < ns; ++k) P.lw[k] = sc.linear_weights[k] / tot;
  P.inv_lw0 = 1.0 / P.lw[0];
  P.epsilon = sc.epsilon;
  P.exponent = sc.exponent;
  P.cfl = sc.cfl_number;
  P.nqc = s->nqc;
  P.nqf = s->nqf;
  P.flux_bc = sc.flux_bc;
  P.n_stages = sc.rk_stages;
  P.gamma2 = sc.gamma == 2.0 ? 1 : 0;
  P.inv_gm1 = 1.0 / (sc.gamma - 1.0);
  P.gm1 = sc.gamma - 1.0;
  if (sc.reconstruction != ZFVM_RC_CWENO_AO && sc.reconstruction != ZFVM_RC_WENO_AO)
    return fail(ZFVM_EINVAL, "unknown reconstruction mode");
  if (sc.step_rejection_drho < 0.0) return fail(ZFVM_EINVAL, "negative step_rejection_drho");
  if (sc.n_avars < 0 || sc.n_avars > ZFVM_MAX_AVARS)
    return fail(ZFVM_EINVAL, "n_avars must be 0 .. " + std::to_string(ZFVM_MAX_AVARS));
  s->na = sc.n_avars;
  P.weno_ao = sc.reconstruction == ZFVM_RC_WENO_AO ? 1 : 0;
  for (int k = 0; k < 5; ++k) P.lw32[k] = (float)P.lw[k];
  P.inv_lw0_32 = (float)P.inv_lw0;
  P.eps32 = (float)P.epsilon;
  P.gamma32 = (float)P.gamma;
  P.exp4 = P.exponent == 4.0 ? 1 : 0;
  P.steps_per_recompute = sc.steps_per_recompute;
  P.recompute_threshold = sc.recompute_threshold;
  std::memset(P.a, 0, sizeof(P.a));
  std::memset(P.b, 0, sizeof(P.b));
  if (sc.rk_stages == 1) {
    P.b[0] = 1.0;
  } else if (sc.rk_stages == 2) {
    P.a[1][0] = 1.0;
    P.b[0] = 0.5, P.b[1] = 0.5;
  } else {
    // SSP3 tableau (ode/runge_kutta.cpp:213-224)
    P.a[1][0] = 1.0;
    P.a[2][0] = 0.25, P.a[2][1] = 0.25;
    P.b[0] = 1.0 / 6, P.b[1] = 1.0 / 6, P.b[2] = 2.0 / 3;
  }
  {
    RefRule cr = nd == 2 ? triangle_rule(m->quad.volume) : tetra_rule(m->quad.volume);
    for (size_t q = 0; q < cr.w.size() && q < 16; ++q) P.what_c[q] = cr.w[q];
  }

  // ---- per-cell arrays
  std::vector<uint8_t> h_flags(ld, 0), h_bloc((size_t)NB * RB * ld, 0);
  std::vector<int> h_l2g((size_t)MAXL * ld, 0), h_cface((size_t)nf * ld, -1), h_src(ld, 0);
  // the pseudo-inverses in FP64 (the FP64 form, and the advected variables of
  // either form) and in FP32 (the mixed form), written straight into the
  // precision each needs
  const bool want64 = !s->mixed || s->na > 0, want32 = s->mixed;
  std::vector<double> h_pinv;
  std::vector<float> h_pinv32;
  if (want64) h_pinv.resize((size_t)NP * ld, 0.0);
  if (want32) h_pinv32.resize((size_t)NP * ld, 0.f);
  auto put_pinv = [&](size_t at, double v) {
    if (want64) h_pinv[at] = v;
    if (want32) h_pinv32[at] = (float)v;
  };
  std::vector<double> h_center((size_t)nd * ld, 0.0), h_il(ld, 0.0), h_mom((size_t)NC * ld, 0.0), h_iv(ld, 0.0),
      h_reff(ld, 1e300);
  // cells in parallel (each writes its own column of every table); the first
  // inconsistency found is reported after the loop
  std::string setup_err;
  bool setup_bad = false;
  auto bad = [&](const char *msg) {
#pragma omp critical(zfvm_setup_error)
    if (!setup_bad) setup_bad = true, setup_err = msg;
  };
#pragma omp parallel for schedule(static)
  for (index_t i = 0; i < n; ++i) {
    h_flags[i] = g.flags[i] | (((g.flags[i] & kGhost) && g.source[i] == i) ? kFrozen : 0);
    h_src[i] = (int)g.source[i];
    h_iv[i] = 1.0 / g.volumes[i];
    h_il[i] = 1.0 / g.char_length[i];
    for (int k = 0; k < nd; ++k) h_center[k * ld + i] = g.cell_centers[i][k];
    for (int c = 3; c <= NC; ++c) h_mom[(c - 1) * ld + i] = g.moments[i * g.n_moments + c];
    for (int f = 0; f < nf; ++f) {
      index_t e = g.edge_indices[i * nf + f];
      int side = g.left[e] == i ? 0 : 1;
      h_cface[f * ld + i] = (int)(2 * e + side);
    }
    const bool active = (g.flags[i] & kInterior) || (g.flags[i] & kGhostL1);
    if (!active) continue;
    if (fam.k_high[i] != 0) {
      bad("cell whose highest-order stencil is not the central one");
      continue;
    }
    const int nl = fam.n_l2g[i];
    if (nl > MAXL) {
      bad("combined stencil larger than the kernel's capacity");
      continue;
    }
    for (int l = 0; l < MAXL; ++l) {
      index_t gl = l < nl ? fam.l2g[i * kMaxL2G + l] : i;
      h_l2g[(size_t)l * ld + i] = (int)g.source[gl];
    }
    // central stencil: local indices are 0..size-1 by construction
    {
      const int k = 0;
      const size_t id = i * kMaxStencils + k;
      const int sz = fam.size[id];
      bool layout_ok = true;
      for (int r = 0; r < sz; ++r) layout_ok = layout_ok && fam.local[id * kMaxStencilSize + r] == r;
      const int rows = m->pinv_rows[id], cols = m->pinv_cols[id];
      if (!layout_ok) {
        bad("unexpected central stencil layout");
        continue;
      }
      if (rows > R0 || cols > C0) {
        bad("central stencil larger than the kernel shape");
        continue;
      }
      for (int c = 0; c < cols; ++c)
        for (int r = 0; r < rows; ++r) put_pinv(((size_t)c * R0 + r) * ld + i, m->pinv[id][(size_t)c * rows + r]);
    }
    for (int k = 1; k < ns; ++k) {
      const size_t id = i * kMaxStencils + k;
      const int rows = m->pinv_rows[id], cols = m->pinv_cols[id];
      if (rows > RB || cols > CB) {
        bad("one-sided stencil larger than the kernel shape");
        break;
      }
      for (int r = 0; r < RB; ++r)
        h_bloc[((size_t)(k - 1) * RB + r) * ld + i] =
            r < rows ? (uint8_t)fam.local[id * kMaxStencilSize + r + 1] : 0;
      for (int c = 0; c < cols; ++c)
        for (int r = 0; r < rows; ++r)
          put_pinv(((size_t)R0 * C0 + ((k - 1) * CB + c) * RB + r) * ld + i, m->pinv[id][(size_t)c * rows + r]);
    }
  }
  if (setup_bad) return fail(ZFVM_EINVAL, setup_err);
  // a periodic image's in-radius bounds its source's CFL length
  for (index_t i = 0; i < n; ++i) h_reff[g.source[i]] = std::min(h_reff[g.source[i]], g.inradii[i]);
  // ---- faces
  const int nqf = s->nqf;
  std::vector<int> h_fL(lde, 0), h_fR(lde, -1);
  std::vector<uint8_t> h_fkL(lde, 0), h_fkR(lde, 0), h_fact(lde, 0);
  std::vector<double> h_fqx((size_t)nqf * nd * lde, 0.0), h_fqw((size_t)nqf * lde, 0.0),
      h_frame((size_t)nd * nd * lde, 0.0), h_farea(lde, 0.0);
#pragma omp parallel for schedule(static)
  for (index_t e = 0; e < g.n_edges; ++e) {
    index_t L = g.left[e], R = g.right[e];
    h_fL[e] = (int)L;
    h_fR[e] = (int)R;
    for (int f = 0; f < nf; ++f) {
      if (g.edge_indices[L * nf + f] == e) h_fkL[e] = (uint8_t)f;
      if (R >= 0 && g.edge_indices[R * nf + f] == e) h_fkR[e] = (uint8_t)f;
    }
    bool Lint = g.flags[L] & kInterior, Rint = R >= 0 && (g.flags[R] & kInterior);
    if (R >= 0)
      h_fact[e] = Lint || Rint;
    else
      // mixed well-balanced form: a boundary face also carries the cell's
      // surface source term, so it is visited without a flux boundary
      h_fact[e] = Lint && (sc.flux_bc != ZFVM_FLUX_BC_NONE ||
                           (sc.precision == ZFVM_MIXED && sc.equilibrium == ZFVM_EQ_ISENTROPIC));
    for (int q = 0; q < nqf; ++q) {
      h_fqw[(size_t)q * lde + e] = g.face_qw[e * nqf + q];
      for (int k = 0; k < nd; ++k) h_fqx[((size_t)q * nd + k) * lde + e] = g.face_qx[e * nqf + q][k];
    }
    Vec3 fr[3] = {g.face_normal[e], g.face_t1[e], g.face_t2[e]};
    for (int a2 = 0; a2 < nd; ++a2)
      for (int k = 0; k < nd; ++k) h_frame[((size_t)a2 * nd + k) * lde + e] = fr[a2][k];
    h_farea[e] = g.face_area[e];
  }
  // ---- gravity potential and its gradient at the quadrature points
  const int nqc = s->nqc;
  std::vector<double> h_phi_cq, h_phi_m1, h_phi_var, h_gphi_cq, h_cqx, h_cqw, h_phi_fq;
  try {
    s->pot = RadialPotential::from_scheme(sc);
  } catch (const SetupError &e) {
    return fail(ZFVM_EINVAL, e.what());  // a configuration error, not a failed set-up
  }
  if (s->has_src) {
    const RadialPotential &pot = s->pot;
    bool uncovered = false;
#pragma omp parallel for schedule(static) reduction(|| : uncovered)
    for (index_t i = 0; i < n; ++i)
      for (int q = 0; q < nqc; ++q) uncovered = uncovered || !pot.covers(norm(g.cell_qx[i * nqc + q]));
#pragma omp parallel for schedule(static) reduction(|| : uncovered)
    for (index_t e = 0; e < g.n_edges; ++e)
      for (int q = 0; q < g.n_face_qp; ++q) uncovered = uncovered || !pot.covers(norm(g.face_qx[e * g.n_face_qp + q]));
    if (uncovered) return fail(ZFVM_EINVAL, "the tabulated potential ends before the mesh does");
    auto phi = [&](const Vec3 &x) { return pot.phi(x); };
    auto gphi = [&](const Vec3 &x, int dir) { return pot.dphi_dx(x, dir); };
    h_phi_cq.assign((size_t)nqc * ld, 0.0);
    h_phi_m1.assign(ld, 0.0);
    h_phi_var.assign(ld, 0.0);
    h_gphi_cq.assign((size_t)nqc * nd * ld, 0.0);
    h_cqx.assign((size_t)nqc * nd * ld, 0.0);
    h_cqw.assign((size_t)nqc * ld, 0.0);
    h_phi_fq.assign((size_t)nqf * lde, 0.0);
#pragma omp parallel for schedule(static)
    for (index_t i = 0; i < n; ++i)
      for (int q = 0; q < nqc; ++q) {
        const Vec3 &x = g.cell_qx[i * nqc + q];
        h_phi_cq[(size_t)q * ld + i] = phi(x);
        h_cqw[(size_t)q * ld + i] = g.cell_qw[i * nqc + q];
        for (int k = 0; k < nd; ++k) {
          h_gphi_cq[((size_t)q * nd + k) * ld + i] = gphi(x, k);
          h_cqx[((size_t)q * nd + k) * ld + i] = x[k];
        }
      }
    // <phi> and <(phi - <phi>)^2> with the reference-cell weights
#pragma omp parallel for schedule(static)
    for (index_t i = 0; i < n; ++i) {
      double m1 = P.what_c[0] * h_phi_cq[i];
      for (int q = 1; q < nqc; ++q) m1 += P.what_c[q] * h_phi_cq[(size_t)q * ld + i];
      double var = 0.0;
      for (int q = 0; q < nqc; ++q) {
        double dphi = h_phi_cq[(size_t)q * ld + i] - m1;
        var += P.what_c[q] * (dphi * dphi);
      }
      h_phi_m1[i] = m1;
      h_phi_var[i] = var;
    }
#pragma omp parallel for schedule(static)
    for (index_t e = 0; e < g.n_edges; ++e)
      for (int q = 0; q < nqf; ++q) h_phi_fq[(size_t)q * lde + e] = phi(g.face_qx[e * nqf + q]);
  }

  CK(cudaGetDevice(&s->device));
  CK(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
  CK(cudaEventCreateWithFlags(&s->ev_in, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&s->ev_sync, cudaEventDisableTiming));
  s->flags.upload(h_flags);
  s->bloc.upload(h_bloc);
  s->l2g.upload(h_l2g);
  s->cface.upload(h_cface);
  s->src_map.upload(h_src);
  s->src_host.assign(h_src.begin(), h_src.begin() + n);
  if (want64) s->pinv.upload(h_pinv);
  s->center.upload(h_center);
  s->inv_len.upload(h_il);
  s->mom.upload(h_mom);
  s->inv_vol.upload(h_iv);
  s->r_eff.upload(h_reff);
  s->fL.upload(h_fL);
  s->fR.upload(h_fR);
  s->fkL.upload(h_fkL);
  s->fkR.upload(h_fkR);
  s->factive.upload(h_fact);
  s->fqx.upload(h_fqx);
  s->fqw.upload(h_fqw);
  s->frame.upload(h_frame);
  s->farea.upload(h_farea);
  if (s->has_src) {
    s->phi_cq.upload(h_phi_cq);
    s->phi_m1.upload(h_phi_m1);
    s->phi_var.upload(h_phi_var);
    s->gphi_cq.upload(h_gphi_cq);
    s->cqx.upload(h_cqx);
    s->cqw.upload(h_cqw);
    s->phi_fq.upload(h_phi_fq);
    if (sc.heating_rate != 0.0) {
      // make_heating_source (model/heating.hpp:52-77): rate on r0 <= |x| <= r1
      std::vector<double> hw((size_t)nqc * ld, 0.0);
      for (index_t i = 0; i < n; ++i)
        for (int q = 0; q < nqc; ++q) {
          const double r = norm(g.cell_qx[i * nqc + q]);
          const bool in = sc.heating_r0 <= r && r <= sc.heating_r1;
          hw[(size_t)q * ld + i] = in ? sc.heating_rate * g.cell_qw[i * nqc + q] : 0.0;
        }
      s->heat_w.upload(hw);
    }
    if (!s->mixed) s->srcb.alloc((size_t)nv * ld);
  }
  if (s->has_eq) s->eqth.alloc((size_t)4 * ld);
  if (s->has_eq && sc.steps_per_recompute > 1) {
    // zero counts: the first reconstruction of every cell refreshes
    s->sched_count.alloc(ld);
    s->sched_count.zero(s->stream);
    s->sched.alloc((size_t)4 * ld);
    s->sched.zero(s->stream);
  }
  s->u0.alloc((size_t)nv * ld);
  s->ux.alloc((size_t)nv * ld);
  if (!s->mixed) s->kbuf.alloc((size_t)std::max(1, sc.rk_stages - 1) * nv * ld);
  if (s->mixed) {
    s->pinv32.upload(h_pinv32);
    // FP32 copies: face frames, moments, scaled offsets of the quadrature points
    s->frame32.upload(std::vector<float>(h_frame.begin(), h_frame.end()));
    s->mom32.upload(std::vector<float>(h_mom.begin(), h_mom.end()));
    s->fqw32.upload(std::vector<float>(h_fqw.begin(), h_fqw.end()));
    std::vector<float> hxf((size_t)nf * nqf * nd * ld, 0.f), hxc((size_t)nqc * nd * ld, 0.f);
#pragma omp parallel for schedule(static)
    for (index_t i = 0; i < n; ++i) {
      const double il = 1.0 / g.char_length[i];
      for (int f = 0; f < nf; ++f) {
        index_t e = g.edge_indices[i * nf + f];
        for (int q = 0; q < nqf; ++q)
          for (int k = 0; k < nd; ++k)
            hxf[((size_t)(f * nqf + q) * nd + k) * ld + i] = (float)((g.face_qx[e * nqf + q][k] - g.cell_centers[i][k]) * il);
      }
      for (int q = 0; q < nqc; ++q)
        for (int k = 0; k < nd; ++k)
          hxc[((size_t)q * nd + k) * ld + i] = (float)((g.cell_qx[i * nqc + q][k] - g.cell_centers[i][k]) * il);
    }
    s->xfq32.upload(hxf);
    s->xcq32.upload(hxc);
    s->g32.alloc((size_t)nv * lde);
    s->mL32.alloc((size_t)nd * lde);
    s->mR32.alloc((size_t)nd * lde);
    s->kbuf32.alloc((size_t)std::max(1, sc.rk_stages - 1) * nv * ld);
    if (s->has_src) s->src32.alloc((size_t)nv * ld);
    for (auto *b : {&s->g32, &s->mL32, &s->mR32, &s->kbuf32, &s->src32}) b->zero(s->stream);
    if (s->has_src) {
      std::vector<double> hg((size_t)nd * ld, 0.0);
      std::vector<float> hwg((size_t)nqc * nd * ld, 0.f);
#pragma omp parallel for schedule(static)
      for (index_t i = 0; i < n; ++i)
        for (int k = 0; k < nd; ++k) {
          double acc = 0.0;
          for (int q = 0; q < nqc; ++q) {
            double wgq = h_cqw[(size_t)q * ld + i] * h_gphi_cq[((size_t)q * nd + k) * ld + i];
            acc += wgq;
            hwg[((size_t)q * nd + k) * ld + i] = (float)wgq;
          }
          hg[(size_t)k * ld + i] = acc;
        }
      s->gphi_w.upload(hg);
      s->wg32.upload(hwg);
    }
    s->fv32.alloc((size_t)nf * nqf * nv * ld);
    s->dev0.alloc((size_t)nv * ld);
    s->qsplit.alloc((size_t)2 * nv * ld);
    s->qsplit.zero(s->stream);
    if (s->has_eq) {
      auto pairs = [&](const std::vector<double> &x) {
        std::vector<float2> out(ld, make_float2(0.f, 0.f));
        for (index_t i = 0; i < n; ++i) {
          const float hi = (float)x[i];
          out[i] = make_float2(hi, (float)(x[i] - (double)hi));
        }
        return out;
      };
      s->m1s.upload(pairs(h_phi_m1));
      s->vars.upload(pairs(h_phi_var));
      // (h_r, f, K) pairs; K = -1 until a cell's equilibrium is found
      std::vector<float2> h_eq((size_t)3 * ld, make_float2(0.f, 0.f));
      for (size_t i = 2 * (size_t)ld; i < h_eq.size(); ++i) h_eq[i] = make_float2(-1.f, 0.f);
      s->eq32.upload(h_eq);
      std::vector<float2> hp((size_t)nqf * lde, make_float2(0.f, 0.f));
      for (size_t k = 0; k < hp.size(); ++k) {
        const float hi = (float)h_phi_fq[k];
        hp[k] = make_float2(hi, (float)(h_phi_fq[k] - (double)hi));
      }
      s->phi_fq2.upload(hp);
    }
    s->dev032.alloc((size_t)nv * ld);
    s->dev032.zero(s->stream);
  } else {
    s->fv.alloc((size_t)nf * nqf * nv * ld);
  }
  if (!s->mixed) s->nfb.alloc((size_t)nv * lde);
  s->tend.alloc((size_t)nv * ld);
  s->aos.alloc((size_t)5 * n);
  if (sc.step_rejection_drho > 0.0) {
    s->uprev.alloc((size_t)nv * ld);
    s->uprev.zero(s->stream);
  }
  if (s->na) {
    const size_t nq = (size_t)s->na * ld;
    s->tq0.alloc(nq);
    s->tqx.alloc(nq);
    s->tk.alloc((size_t)std::max(1, sc.rk_stages - 1) * nq);
    s->tfv.alloc((size_t)nf * s->nqf * nq);
    s->tnf.alloc((size_t)s->na * lde);
    s->ttend.alloc(nq);
    if (sc.step_rejection_drho > 0.0) s->tprev.alloc(nq);
    for (auto *b : {&s->tq0, &s->tqx, &s->tk, &s->tfv, &s->tnf, &s->ttend, &s->tprev}) b->zero(s->stream);
  }
  s->clock.alloc(1);
  for (auto *b : {&s->u0, &s->ux, &s->kbuf, &s->fv, &s->nfb, &s->tend, &s->dev0}) b->zero(s->stream);
  s->fv32.zero(s->stream);
  if (s->has_src) s->srcb.zero(s->stream);
  if (s->has_eq) s->eqth.zero(s->stream);
  Clock c = fresh_clock(s, 0.0);
  write_clock(s, c);
  CK(cudaStreamSynchronize(s->stream));

  DevData &D = s->D;
  D.n_cells = s->n_cells;
  D.ld = ld;
  D.n_edges = s->n_edges;
  D.lde = lde;
  D.flags = s->flags.p;
  D.l2g = s->l2g.p;
  D.pinv = s->pinv.p;
  D.pinv32 = s->pinv32.p;
  D.phi_m1 = s->phi_m1.p;
  D.frame32 = s->frame32.p;
  D.xfq32 = s->xfq32.p;
  D.xcq32 = s->xcq32.p;
  D.mom32 = s->mom32.p;
  D.fqw32 = s->fqw32.p;
  D.gphi_w = s->gphi_w.p;
  D.wg32 = s->wg32.p;
  D.m1s = s->m1s.p;
  D.vars = s->vars.p;
  D.phi_fq2 = s->phi_fq2.p;
  D.heat_w = s->heat_w.p;
  D.phi_var = s->phi_var.p;
  D.bloc = s->bloc.p;
  D.center = s->center.p;
  D.inv_len = s->inv_len.p;
  D.mom = s->mom.p;
  D.cface = s->cface.p;
  D.inv_vol = s->inv_vol.p;
  D.r_eff = s->r_eff.p;
  D.fL = s->fL.p;
  D.fR = s->fR.p;
  D.fkL = s->fkL.p;
  D.fkR = s->fkR.p;
  D.factive = s->factive.p;
  D.fqx = s->fqx.p;
  D.fqw = s->fqw.p;
  D.frame = s->frame.p;
  D.farea = s->farea.p;
  D.phi_cq = s->phi_cq.p;
  D.gphi_cq = s->gphi_cq.p;
  D.cqx = s->cqx.p;
  D.cqw = s->cqw.p;
  D.phi_fq = s->phi_fq.p;
  D.clock = s->clock.p;

  int64_t bytes = 0;
  auto add = [&](size_t nbytes) { bytes += (int64_t)nbytes; };
  add(s->flags.n + s->bloc.n + s->fkL.n + s->fkR.n + s->factive.n);
  add(4 * (s->l2g.n + s->cface.n + s->fL.n + s->fR.n + s->src_map.n));
  add(4 * (s->pinv32.n + s->fv32.n + s->frame32.n + s->xfq32.n + s->xcq32.n + s->mom32.n + s->wg32.n + s->g32.n +
           s->mL32.n + s->mR32.n + s->src32.n + s->kbuf32.n + s->fqw32.n));
  add(8 * (s->gphi_w.n + s->qsplit.n + s->m1s.n + s->vars.n + s->eq32.n + s->phi_fq2.n));
  add(4 * s->dev032.n);
  add(8 * s->uprev.n);
  add(4 * s->sched_count.n + 8 * s->sched.n);
  add(8 * s->heat_w.n);
  add(8 * (s->dev0.n + s->phi_m1.n + s->phi_var.n + s->pinv.n + s->center.n + s->inv_len.n + s->mom.n + s->inv_vol.n + s->r_eff.n + s->fqx.n + s->fqw.n +
           s->frame.n + s->farea.n + s->phi_cq.n + s->gphi_cq.n + s->cqx.n + s->cqw.n + s->phi_fq.n + s->u0.n +
           s->ux.n + s->kbuf.n + s->fv.n + s->nfb.n + s->srcb.n + s->eqth.n + s->tend.n + s->aos.n));
  add(8 * (s->tq0.n + s->tqx.n + s->tk.n + s->tfv.n + s->tnf.n + s->ttend.n + s->tprev.n));
  s->device_bytes = bytes;
  return ZFVM_OK;
}

}  // namespace

void reset_clock_for_run(zfvm_solver *s, int64_t n_steps, double t_end, double fixed_dt) {
  // step rejection belongs to the time loop (TimeLoop), not to a single step
  const double drho = fixed_dt > 0.0 ? 0.0 : s->scheme.step_rejection_drho;
  k_clock_reset<<<1, 1, 0, s->stream>>>(s->clock.p, (long long)n_steps, t_end, fixed_dt, drho);
  CK(cudaGetLastError());
}

namespace {

void capture_steps(zfvm_solver *s, int steps, cudaGraphExec_t *out) {
  cudaGraph_t g;
  CK(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
  try {
    for (int k = 0; k < steps; ++k) enqueue_step(s);
  } catch (...) {
    // end the capture, so the thread and the stream are usable again
    cudaGraph_t broken = nullptr;
    cudaStreamEndCapture(s->stream, &broken);
    if (broken) cudaGraphDestroy(broken);
    throw;
  }
  CK(cudaStreamEndCapture(s->stream, &g));
  CK(cudaGraphInstantiate(out, g, 0));
  cudaGraphDestroy(g);
}

void build_graph(zfvm_solver *s, int steps) {
  if (s->graph && s->graph_steps == steps) return;
  if (s->graph) cudaGraphExecDestroy(s->graph);
  s->graph = nullptr;
  capture_steps(s, steps, &s->graph);
  s->graph_steps = steps;
}

void build_tail_graph(zfvm_solver *s, int steps) {
  if (s->graph_tail && s->graph_tail_steps == steps) return;
  if (s->graph_tail) cudaGraphExecDestroy(s->graph_tail);
  s->graph_tail = nullptr;
  capture_steps(s, steps, &s->graph_tail);
  s->graph_tail_steps = steps;
}

}  // namespace

extern "C" int zfvm_solver_create(zfvm_mesh *m, const zfvm_scheme_desc *sc, zfvm_solver **out) {
  if (!m || !sc || !out) return fail(ZFVM_EINVAL, "null argument");
  if (sc->precision != ZFVM_FP64 && sc->precision != ZFVM_MIXED) return fail(ZFVM_EINVAL, "unknown precision");
  if (!(sc->gamma > 1.0) || !(sc->cfl_number > 0.0)) return fail(ZFVM_EINVAL, "bad gamma or cfl_number");
  auto s = std::make_unique<zfvm_solver>();
  s->mesh = m;
  s->scheme = *sc;
  SOLVER_GUARD_BEGIN
  int st = build_solver(s.get());
  if (st != ZFVM_OK) return st;
  *out = s.release();
  return ZFVM_OK;
  SOLVER_GUARD_END
}

extern "C" int zfvm_solver_destroy(zfvm_solver *s) {
  delete s;  // ~zfvm_solver waits for the solver's stream, then frees everything
  return ZFVM_OK;
}

namespace {

// Upload a host state and open a fresh clock at time t, all stream-ordered;
// ev_in is recorded once the host buffer has been read.
void upload_state(zfvm_solver *s, const double *cvars, double t) {
  const size_t n = s->n_cells;
  CK(cudaMemcpyAsync(s->aos.p, cvars, n * 5 * sizeof(double), cudaMemcpyHostToDevice, s->stream));
  CK(cudaEventRecord(s->ev_in, s->stream));
  // the stage state starts as a copy: the update writes interior cells only, so
  // frozen ghost cells carry their values into every stage from here
  k_state_in<<<(int)((n + 127) / 128), 128, 0, s->stream>>>(s->aos.p, s->u0.p, s->ux.p, s->qsplit.p, (int)n, s->ld,
                                                            s->nv);
  CK(cudaGetLastError());
  Clock c = fresh_clock(s, t);
  write_clock(s, c);
  launch_cfl(s);
}

// Download the step state into host rows (no synchronisation).
void download_state(zfvm_solver *s, double *cvars) {
  const size_t n = s->n_cells;
  k_soa_to_aos<<<(int)((n + 127) / 128), 128, 0, s->stream>>>(s->u0.p, s->aos.p, (int)n, s->ld, s->nv, s->src_map.p);
  CK(cudaGetLastError());
  if (cvars) CK(cudaMemcpyAsync(cvars, s->aos.p, n * 5 * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
}

// The time loop on the device: graph-replayed chunks of steps until the
// clock is done, then the close of the last step.  Polls the clock only when
// the end is a time or steps may be rejected.
void run_steps(zfvm_solver *s, int64_t n_steps, double t_end, double fixed_dt) {
  reset_clock_for_run(s, n_steps, t_end, fixed_dt);
  const int chunk = n_steps > 0 ? (int)std::min<int64_t>(n_steps, 16) : 16;
  build_graph(s, chunk);
  int64_t launched = 0;
  const bool rejecting = s->uprev.p != nullptr;  // rejected steps do not count
  while (true) {
    CK(cudaGraphLaunch(s->graph, s->stream));
    launched += chunk;
    if (n_steps > 0 && launched >= n_steps && !rejecting) break;
    if (launched % (chunk * 8) == 0 || n_steps <= 0 || rejecting) {
      Clock c = read_clock(s);
      if (c.done) break;
    }
  }
  close_step(s);
}

}  // namespace

extern "C" int zfvm_set_state(zfvm_solver *s, const double *cvars, double t) {
  if (!s || !cvars) return fail(ZFVM_EINVAL, "null argument");
  SOLVER_GUARD_BEGIN
  upload_state(s, cvars, t);
  // return once the caller's buffer has been read; the layout and CFL kernels
  // run on, ordered before the solver's next work on its stream
  CK(cudaEventSynchronize(s->ev_in));
  return ZFVM_OK;
  SOLVER_GUARD_END
}

extern "C" int zfvm_step_host(zfvm_solver *s, const double *cvars_in, double t, int64_t n_steps, double t_end,
                              double fixed_dt, double *cvars_out, double *t_out, int64_t *steps_out) {
  if (!s || !cvars_in || !cvars_out) return fail(ZFVM_EINVAL, "null argument");
  if (n_steps <= 0 && !(t_end > t)) return fail(ZFVM_EINVAL, "need n_steps > 0 or t_end > t");
  if (fixed_dt < 0.0) return fail(ZFVM_EINVAL, "negative fixed_dt");
  SOLVER_GUARD_BEGIN
  upload_state(s, cvars_in, t);
  run_steps(s, n_steps, t_end, fixed_dt);
  // cvars_out may be cvars_in: the upload has read it before the download lands
  download_state(s, cvars_out);
  const Clock c = read_clock(s);  // the one synchronisation of the call
  if (t_out) *t_out = c.t;
  if (steps_out) *steps_out = c.step;
  std::string msg;
  const int code = status_to_code(c.status, msg);
  if (code) return fail(code, msg);
  return ZFVM_OK;
  SOLVER_GUARD_END
}

extern "C" int zfvm_get_state(zfvm_solver *s, double *cvars, double *t) {
  if (!s) return fail(ZFVM_EINVAL, "null argument");
  SOLVER_GUARD_BEGIN
  download_state(s, cvars);
  Clock c = read_clock(s);
  if (t) *t = c.t;
  return ZFVM_OK;
  SOLVER_GUARD_END
}

extern "C" int zfvm_set_avars(zfvm_solver *s, const double *avars) {
  if (!s || (s->na && !avars)) return fail(ZFVM_EINVAL, "null argument");
  if (!s->na) return ZFVM_OK;
  SOLVER_GUARD_BEGIN
  const size_t n = s->n_cells, na = s->na, ld = s->ld;
  std::vector<double> soa((size_t)na * ld, 0.0);
  for (size_t i = 0; i < n; ++i)
    for (size_t t = 0; t < na; ++t) soa[t * ld + i] = avars[i * na + t];
  CK(cudaMemcpyAsync(s->tq0.p, soa.data(), soa.size() * sizeof(double), cudaMemcpyHostToDevice, s->stream));
  // frozen ghost cells keep these values in every stage, like the state
  CK(cudaMemcpyAsync(s->tqx.p, s->tq0.p, soa.size() * sizeof(double), cudaMemcpyDeviceToDevice, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  return ZFVM_OK;
  SOLVER_GUARD_END
}

extern "C" int zfvm_get_avars(zfvm_solver *s, double *avars) {
  if (!s || (s->na && !avars)) return fail(ZFVM_EINVAL, "null argument");
  if (!s->na) return ZFVM_OK;
  SOLVER_GUARD_BEGIN
  const size_t n = s->n_cells, na = s->na, ld = s->ld;
  std::vector<double> soa((size_t)na * ld);
  CK(cudaMemcpyAsync(soa.data(), s->tq0.p, soa.size() * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  // periodic ghost cells report their source's values, as zfvm_get_state does
  for (size_t i = 0; i < n; ++i)
    for (size_t t = 0; t < na; ++t) avars[i * na + t] = soa[t * ld + (size_t)s->src_host[i]];
  return ZFVM_OK;
  SOLVER_GUARD_END
}

extern "C" int zfvm_solver_write_snapshot(zfvm_solver *s, const char *path, int64_t n_steps) {
  if (!s || !path) return fail(ZFVM_EINVAL, "null argument");
  std::vector<double> u, q;
  try {
    u.resize((size_t)s->n_cells * 5);
    q.resize((size_t)s->n_cells * s->na);
  } catch (const std::bad_alloc &) {
    return fail(ZFVM_ENOMEM, "host allocation failed");
  }
  double t = 0.0;
  int st = zfvm_get_state(s, u.data(), &t);
  if (st == ZFVM_OK) st = zfvm_get_avars(s, q.data());
  if (st != ZFVM_OK) return st;
  return zfvm_snapshot_write(path, s->n_cells, u.data(), s->na, q.data(), 1, t, n_steps);
}

extern "C" int zfvm_solver_read_snapshot(zfvm_solver *s, const char *path, int64_t *n_steps) {
  if (!s || !path) return fail(ZFVM_EINVAL, "null argument");
  int64_t n = 0;
  int32_t na = 0, has_clock = 0;
  int st = zfvm_snapshot_info(path, &n, &na, &has_clock);
  if (st != ZFVM_OK) return st;
  if (n != s->n_cells)
    return fail(ZFVM_EINVAL, std::string(path) + " holds " + std::to_string(n) + " cells, the solver's mesh " +
                                 std::to_string(s->n_cells));
  if (!has_clock) return fail(ZFVM_EINVAL, std::string(path) + " has no \"time\" and \"n_steps\" (a steady state?)");
  if (na != s->na)
    return fail(ZFVM_EINVAL, std::string(path) + " holds " + std::to_string(na) + " advected variables, the solver " +
                                 std::to_string(s->na));
  std::vector<double> u, q;
  try {
    u.resize((size_t)n * 5);
    q.resize((size_t)n * na);
  } catch (const std::bad_alloc &) {
    return fail(ZFVM_ENOMEM, "host allocation failed");
  }
  double t = 0.0;
  int64_t steps = 0;
  st = zfvm_snapshot_read(path, n, u.data(), na, q.data(), &t, &steps);
  if (st != ZFVM_OK) return st;
  st = zfvm_set_state(s, u.data(), t);
  if (st == ZFVM_OK) st = zfvm_set_avars(s, q.data());
  if (st == ZFVM_OK && n_steps) *n_steps = steps;
  return st;
}

extern "C" int zfvm_rate_of_change_all(zfvm_solver *s, double *tendency, double *avars_tendency) {
  if (!s || !tendency || (s->na && !avars_tendency)) return fail(ZFVM_EINVAL, "null argument");
  SOLVER_GUARD_BEGIN
  Clock c = read_clock(s);
  c.done = 0;
  c.status = 0;
  write_clock(s, c);
  CK(cudaMemsetAsync(s->tend.p, 0, s->tend.n * sizeof(double), s->stream));
  StageArgs a = stage_args(s, 0, s->tend.p);
  dispatch_stage(s, a);
  if (s->na) {
    s->ttend.zero(s->stream);
    dispatch_tracers(s, a, s->ttend.p);
    std::vector<double> soa(s->ttend.n);
    CK(cudaMemcpyAsync(soa.data(), s->ttend.p, soa.size() * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    const size_t n = s->n_cells, na = s->na, ld = s->ld;
    for (size_t i = 0; i < n; ++i)
      for (size_t t = 0; t < na; ++t) avars_tendency[i * na + t] = soa[t * ld + i];
  }
  const size_t n = s->n_cells;
  std::vector<int> ident(n);
  for (size_t i = 0; i < n; ++i) ident[i] = (int)i;
  DBuf<int> idb;
  idb.upload(ident);
  k_soa_to_aos<<<(int)((n + 127) / 128), 128, 0, s->stream>>>(s->tend.p, s->aos.p, (int)n, s->ld, s->nv, idb.p);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(tendency, s->aos.p, n * 5 * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  Clock c2 = read_clock(s);
  std::string msg;
  int code = status_to_code(c2.status, msg);
  if (code) return fail(code, msg);
  return ZFVM_OK;
  SOLVER_GUARD_END
}

extern "C" int zfvm_rate_of_change(zfvm_solver *s, double *tendency) {
  if (!s || !tendency) return fail(ZFVM_EINVAL, "null argument");
  if (!s->na) return zfvm_rate_of_change_all(s, tendency, nullptr);
  std::vector<double> scratch;
  try {
    scratch.resize((size_t)s->n_cells * s->na);
  } catch (const std::bad_alloc &) {
    return fail(ZFVM_ENOMEM, "host allocation failed");
  }
  return zfvm_rate_of_change_all(s, tendency, scratch.data());
}

extern "C" int zfvm_cfl_dt(zfvm_solver *s, double *dt) {
  if (!s || !dt) return fail(ZFVM_EINVAL, "null argument");
  SOLVER_GUARD_BEGIN
  Clock c = read_clock(s);
  c.cfl_min = 0x7ff0000000000000ull;
  write_clock(s, c);
  launch_cfl(s);
  c = read_clock(s);
  *dt = s->P.cfl * __builtin_bit_cast(double, c.cfl_min);
  return ZFVM_OK;
  SOLVER_GUARD_END
}

extern "C" int zfvm_step(zfvm_solver *s, double dt) {
  if (!s || !(dt > 0.0)) return fail(ZFVM_EINVAL, "bad argument");
  SOLVER_GUARD_BEGIN
  reset_clock_for_run(s, 1, 0.0, dt);
  enqueue_step(s);
  close_step(s);
  Clock c = read_clock(s);
  std::string msg;
  int code = status_to_code(c.status, msg);
  if (code) return fail(code, msg);
  return ZFVM_OK;
  SOLVER_GUARD_END
}

extern "C" int zfvm_advance(zfvm_solver *s, int64_t n_steps, double t_end, double *t_out, int64_t *steps_out) {
  if (!s) return fail(ZFVM_EINVAL, "null solver");
  if (n_steps <= 0 && !(t_end > 0.0)) return fail(ZFVM_EINVAL, "need n_steps > 0 or t_end > 0");
  SOLVER_GUARD_BEGIN
  run_steps(s, n_steps, t_end, 0.0);
  Clock c = read_clock(s);
  if (t_out) *t_out = c.t;
  if (steps_out) *steps_out = c.step;
  std::string msg;
  int code = status_to_code(c.status, msg);
  if (code) return fail(code, msg);
  return ZFVM_OK;
  SOLVER_GUARD_END
}

extern "C" int zfvm_advance_timed(zfvm_solver *s, int64_t n_steps, float *ms) {
  if (!s || !ms || n_steps <= 0) return fail(ZFVM_EINVAL, "bad argument");
  SOLVER_GUARD_BEGIN
  reset_clock_for_run(s, n_steps, 0.0, 0.0);
  // exactly n_steps steps: whole 16-step graphs and one graph of the rest
  const int chunk = (int)std::min<int64_t>(n_steps, 16), tail = (int)(n_steps % chunk);
  build_graph(s, chunk);
  if (tail) build_tail_graph(s, tail);
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  CK(cudaStreamSynchronize(s->stream));
  CK(cudaEventRecord(e0, s->stream));
  for (int64_t k = 0; k + chunk <= n_steps; k += chunk) CK(cudaGraphLaunch(s->graph, s->stream));
  if (tail) CK(cudaGraphLaunch(s->graph_tail, s->stream));
  CK(cudaEventRecord(e1, s->stream));
  CK(cudaEventSynchronize(e1));
  CK(cudaEventElapsedTime(ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  close_step(s);
  Clock c = read_clock(s);
  std::string msg;
  int code = status_to_code(c.status, msg);
  if (code) return fail(code, msg);
  if (c.step != n_steps) return fail(ZFVM_EINVAL, "step count mismatch in the timed loop");
  return ZFVM_OK;
  SOLVER_GUARD_END
}

extern "C" int zfvm_launches_per_step(const zfvm_solver *s, int32_t *launches) {
  if (!s || !launches) return fail(ZFVM_EINVAL, "null argument");
  // clock, restore (step rejection), three kernels per stage, three more with advected variables
  *launches = 1 + (s->uprev.p ? 1 : 0) + 3 * s->P.n_stages * (s->na ? 2 : 1);
  return ZFVM_OK;
}

extern "C" int zfvm_device_bytes(const zfvm_solver *s, int64_t *bytes) {
  if (!s || !bytes) return fail(ZFVM_EINVAL, "null argument");
  *bytes = s->device_bytes;
  return ZFVM_OK;
}

extern "C" int zfvm_kernel_times(zfvm_solver *s, int64_t n_steps, float *ms) {
  if (!s || !ms || n_steps <= 0) return fail(ZFVM_EINVAL, "bad argument");
  SOLVER_GUARD_BEGIN
  reset_clock_for_run(s, n_steps, 0.0, 0.0);
  const int S = s->P.n_stages;
  std::vector<cudaEvent_t> ev((size_t)n_steps * S * 4);
  for (auto &e : ev) CK(cudaEventCreate(&e));
  for (int64_t k = 0; k < n_steps; ++k) {
    k_clock<<<1, 1, 0, s->stream>>>(s->clock.p, s->P.cfl, 0);
    enqueue_restore(s);
    for (int st = 0; st < S; ++st) {
      StageArgs a = stage_args(s, st, nullptr);
      dispatch_stage(s, a, &ev[((size_t)k * S + st) * 4]);
    }
  }
  close_step(s);
  CK(cudaStreamSynchronize(s->stream));
  double acc[3] = {0, 0, 0};
  for (size_t b = 0; b < ev.size(); b += 4)
    for (int j = 0; j < 3; ++j) {
      float t;
      CK(cudaEventElapsedTime(&t, ev[b + j], ev[b + j + 1]));
      acc[j] += t;
    }
  const double launches = (double)n_steps * S;
  for (int j = 0; j < 3; ++j) ms[j] = (float)(acc[j] / launches);
  for (auto &e : ev) cudaEventDestroy(e);
  Clock c = read_clock(s);
  std::string msg;
  int code = status_to_code(c.status, msg);
  if (code) return fail(code, msg);
  return ZFVM_OK;
  SOLVER_GUARD_END
}

// Device bytes zfvm_solver_create would allocate for this mesh and scheme: the
// same buffers and sizes as build_solver, so a caller (or the server's
// admission control) can decide before allocating.
int64_t solver_footprint(const zfvm_mesh *m, const zfvm_scheme_desc &sc) {
  const Grid &g = m->grid;
  const auto &sp = m->sparams;
  const int64_t nd = g.n_dims, nv = nd + 2, nf = nd + 1, nqf = g.n_face_qp, nqc = g.n_cell_qp;
  const int64_t ld = (g.n_cells + 31) / 32 * 32, lde = (g.n_edges + 31) / 32 * 32, n = g.n_cells;
  const int ns = (int)sp.orders.size();
  if (ns < 2) return -1;
  const int64_t R0 = (int64_t)required_stencil_size(sp.orders[0] - 1, sp.overfit[0], (int)nd) - 1;
  const int64_t C0 = poly_dof(sp.orders[0] - 1, (int)nd) - 1;
  const int64_t NB = ns - 1;
  const int64_t RB = (int64_t)required_stencil_size(sp.orders[1] - 1, sp.overfit[1], (int)nd) - 1;
  const int64_t CB = poly_dof(sp.orders[1] - 1, (int)nd) - 1;
  const int64_t NC = std::max(C0, CB), NP = R0 * C0 + NB * RB * CB, MAXL = R0 + 1 + NB * RB;
  const bool mixed = sc.precision == ZFVM_MIXED, has_eq = sc.equilibrium == ZFVM_EQ_ISENTROPIC,
             has_src = sc.gravity != ZFVM_GRAVITY_NONE;
  const int64_t kst = std::max(1, sc.rk_stages - 1);
  int64_t b = 0;
  // flags, bloc, fkL, fkR, factive
  b += ld + NB * RB * ld + 3 * lde;
  // l2g, cface, fL, fR, src_map
  b += 4 * (MAXL * ld + nf * ld + 2 * lde + ld);
  // geometry, faces, state and tendency
  b += 8 * (nd * ld + ld + NC * ld + ld + ld);                       // center, inv_len, mom, inv_vol, r_eff
  b += 8 * (nqf * nd * lde + nqf * lde + nd * nd * lde + lde);       // fqx, fqw, frame, farea
  b += 8 * (2 * nv * ld + nv * ld + 5 * n);                          // u0, ux, tend, aos
  if (has_src) {
    b += 8 * (nqc * ld + 2 * ld + 2 * nqc * nd * ld + nqc * ld + nqf * lde);  // phi_cq, m1, var, gphi, cqx, cqw, phi_fq
    if (!mixed) b += 8 * nv * ld;                                               // srcb
  }
  if (has_eq) b += 8 * 4 * ld;                                                  // eqth
  if (has_eq && sc.steps_per_recompute > 1) b += 4 * ld + 8 * 4 * ld;           // sched_count, sched
  if (sc.step_rejection_drho > 0.0) b += 8 * nv * ld;                            // uprev
  if (sc.heating_rate != 0.0 && has_src) b += 8 * nqc * ld;                       // heat_w
  if (mixed) {
    b += 4 * (NP * ld + nd * nd * lde + NC * ld + nf * nqf * nd * ld + nqc * nd * ld + nqf * lde);  // pinv32 frame32 mom32 xfq32 xcq32 fqw32
    b += 4 * (nv * lde + 2 * nd * lde + kst * nv * ld + nf * nqf * nv * ld);          // g32 mL32 mR32 kbuf32 fv32
    b += 8 * nv * ld;                                                                   // dev0
    b += 8 * 2 * nv * ld + 4 * nv * ld;                                                 // qsplit dev032
    if (has_eq) b += 8 * 2 * ld + 8 * 3 * ld + 8 * nqf * lde;                           // m1s vars eq32 phi_fq2
    if (has_src) b += 4 * nv * ld + 8 * nd * ld + 4 * nqc * nd * ld;                   // src32 gphi_w wg32
  } else {
    b += 8 * (NP * ld + kst * nv * ld + nf * nqf * nv * ld + nv * lde);  // pinv kbuf fv nfb
  }
  const int64_t na = sc.n_avars;
  if (na > 0) {
    if (mixed) b += 8 * NP * ld;                                               // FP64 pinv
    b += 8 * (na * ld * (3 + kst) + nf * nqf * na * ld + na * lde);             // tq0 tqx ttend tk tfv tnf
    if (sc.step_rejection_drho > 0.0) b += 8 * na * ld;                         // tprev
  }
  return b;
}

extern "C" int zfvm_solver_footprint(const zfvm_mesh *m, const zfvm_scheme_desc *sc, int64_t *bytes) {
  if (!m || !sc || !bytes) return fail(ZFVM_EINVAL, "null argument");
  const int64_t b = solver_footprint(m, *sc);
  if (b < 0) return fail(ZFVM_EINVAL, "the mesh has fewer than two stencils");
  *bytes = b;
  return ZFVM_OK;
}

namespace {

// GlobalReconstruction::operator()(i, x) on the host from the exported records
template <class S>
int eval_records(const zfvm_solver *s, int64_t n, const int64_t *cells, const double *x, double *u) {
  using PR = PolyRecord<S>;
  constexpr int NV = S::NV, ND = S::ND, NC = S::NC;
  const int ld = s->ld;
  const double *rec = s->poly_host.data();
  const auto &sc = s->scheme;
  EqEval ev{sc.gamma, sc.gamma - 1.0, 1.0 / (sc.gamma - 1.0)};
  for (int64_t k = 0; k < n; ++k) {
    const int64_t i = cells[k];
    if (i < 0 || i >= s->n_cells) return fail(ZFVM_EINVAL, "cell index out of range");
    auto at = [&](int row) { return rec[(size_t)row * ld + i]; };
    if (at(PR::VALID) != 1.0) return fail(ZFVM_EINVAL, "cell " + std::to_string(i) + " has no reconstruction");
    double X[ND], C[NC], phi_c[NC];
    for (int d = 0; d < ND; ++d) X[d] = (x[3 * k + d] - at(PR::XC + d)) * at(PR::IL);
    for (int c = 0; c < NC; ++c) C[c] = at(PR::MOM + c);
    basis<ND, NC>(X, C, phi_c);
    double w[NV];
    for (int v = 0; v < NV; ++v) {
      double acc = at(PR::DEV + v);
      for (int c = 0; c < NC; ++c) acc += at(PR::COEF + c * NV + v) * phi_c[c];
      w[v] = acc;
    }
    if (at(PR::EQ + 3) != 0.0) {
      const double phi = s->pot.phi(Vec3{x[3 * k], x[3 * k + 1], x[3 * k + 2]});
      EqEval::Bound b{at(PR::EQ), at(PR::EQ + 1), at(PR::EQ + 2)};
      double rho, E;
      b.at(ev, phi, rho, E);
      w[0] += rho;
      w[NV - 1] += E;
    }
    double *o = u + 5 * k;
    for (int v = 0; v < 5; ++v) o[v] = 0.0;
    for (int v = 0; v < NV - 1; ++v) o[v] = w[v];
    o[4] = w[NV - 1];
  }
  return ZFVM_OK;
}

int poly_record_size(int shape_id) {
  switch (shape_id) {
    case 0: return PolyRecord<S2o3>::SIZE;
    case 1: return PolyRecord<S2o2>::SIZE;
    case 2: return PolyRecord<S3o3>::SIZE;
    default: return PolyRecord<S3o2>::SIZE;
  }
}

}  // namespace

// EulerGlobalReconstruction::compute (reconstruction/global_reconstruction_impl.hpp:100-163)
extern "C" int zfvm_reconstruct(zfvm_solver *s) {
  if (!s) return fail(ZFVM_EINVAL, "null argument");
  SOLVER_GUARD_BEGIN
  const size_t size = (size_t)poly_record_size(s->shape_id) * s->ld;
  if (s->poly.n != size) s->poly.alloc(size);
  CK(cudaMemsetAsync(s->poly.p, 0, size * sizeof(double), s->stream));
  Clock c = read_clock(s);
  c.done = 0;
  c.status = 0;
  write_clock(s, c);
  StageArgs a = stage_args(s, 0, s->tend.p);
  a.poly_out = s->poly.p;
  LaunchCfg lc = launch_cfg(s);
  switch (s->shape_id) {
    case 0: launch_export_s2o3(s->D, s->P, a, lc); break;
    case 1: launch_export_s2o2(s->D, s->P, a, lc); break;
    case 2: launch_export_s3o3(s->D, s->P, a, lc); break;
    case 3: launch_export_s3o2(s->D, s->P, a, lc); break;
  }
  CK(cudaGetLastError());
  s->poly_host.resize(size);
  CK(cudaMemcpyAsync(s->poly_host.data(), s->poly.p, size * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  Clock c2 = read_clock(s);
  std::string msg;
  int code = status_to_code(c2.status, msg);
  if (code) return fail(code, msg);
  return ZFVM_OK;
  SOLVER_GUARD_END
}

// GlobalReconstruction::operator()(i, x) (global_reconstruction_decl.hpp:29)
extern "C" int zfvm_reconstruction_eval(const zfvm_solver *s, int64_t n, const int64_t *cells, const double *x,
                                        double *u) {
  if (!s || (n > 0 && (!cells || !x || !u))) return fail(ZFVM_EINVAL, "null argument");
  if (s->poly_host.empty()) return fail(ZFVM_EINVAL, "call zfvm_reconstruct first");
  switch (s->shape_id) {
    case 0: return eval_records<S2o3>(s, n, cells, x, u);
    case 1: return eval_records<S2o2>(s, n, cells, x, u);
    case 2: return eval_records<S3o3>(s, n, cells, x, u);
    default: return eval_records<S3o2>(s, n, cells, x, u);
  }
}

// number of steps rejected (RejectLargeDensityChange) since the state was set
extern "C" int zfvm_step_rejections(zfvm_solver *s, int64_t *n) {
  if (!s || !n) return fail(ZFVM_EINVAL, "null argument");
  SOLVER_GUARD_BEGIN
  *n = read_clock(s).n_rejected;
  return ZFVM_OK;
  SOLVER_GUARD_END
}
