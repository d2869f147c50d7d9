// Advected variables (AllVariables::avars): mass-weighted tracers mq carried
// along with the flow, three kernels per Runge-Kutta stage after the stage's
// own three.  They follow the reference's FluxLoop with tracers:
//   - EulerGlobalReconstruction::compute reconstructs every tracer of a cell
//     on its own from its raw cell averages over the cell's stencils, with
//     the same CWENO-AO / WENO-AO combination but its own smoothness
//     indicators and no equilibrium or scaling
//     (global_reconstruction_impl.hpp:101-129, local_reconstruction.hpp:127-147);
//   - FluxLoop::compute_patch evaluates the tracer polynomials at every face
//     point and integrates HLLCBatten::tracer_flux with the wave speeds of the
//     Euler flux at that point (flux_loop.hpp:140-192, hllc.hpp:178-197);
//   - the tendency enters the same RK combination as the conserved variables
//     (runge_kutta.cpp:181-202).
// Boundary fluxes (FluxBC, EquilibriumFluxBC) carry no tracer: the reference's
// boundary terms only write cvars.
//
// Everything here is FP64 in both forms.  The face kernel rebuilds the Euler
// face states from what the stage's reconstruction left (the FP64 face values,
// or in the mixed form the FP64 base plus the FP32 polynomial part) and
// computes the wave speeds from them; the Euler kernels are unchanged and cost
// nothing extra when there are no tracers.
#pragma once

namespace zfvm {
namespace dev {

// The advected variables of one stage.  Layouts: state [NA][ld], face values
// [NF * NQF][NA][ld] (cell-local face f, point q), face fluxes [NA][lde].
struct TracerArgs {
  int na;
  const double *q;   // stage values
  double *fv;        // values of the limited polynomials at the cell's face points
  double *nf;        // integrated tracer flux of every face, left to right
  double *u0, *ux;   // step start (overwritten at the last stage) / next stage
  double *k[4];      // stage tendencies
  double *tend_out;  // when non-null: write the tendency and do no RK update
  double *uprev;     // step rejection: the step's start values, saved at the last stage
};

template <class S>
__global__ void __launch_bounds__(128) k_tracer_reconstruct(const DevData d, const Params P, TracerArgs ta) {
  constexpr int ND = S::ND, NF = S::NF, NC = S::NC, C0 = S::C0, CB = S::CB, NB = S::NB;
  constexpr int R0 = S::R0, RB = S::RB, NQF = S::NQF;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.n_cells || d.clock->done) return;
  if (!(d.flags[i] & (kInterior | kGhostL1))) return;
  const int ld = d.ld, lde = d.lde, na = ta.na;
  const int j0 = d.l2g[i];
  double xc[ND], C[NC];
#pragma unroll
  for (int k = 0; k < ND; ++k) xc[k] = d.center[k * ld + i];
  const double il = d.inv_len[i];
#pragma unroll
  for (int c = 0; c < NC; ++c) C[c] = d.mom[c * ld + i];
  for (int t = 0; t < na; ++t) {
    const double *__restrict__ q = ta.q + (size_t)t * ld;
    const double q0 = q[j0];
    // LSQ fits of every stencil (HybridWENO::compute_polys, hybrid_weno.cpp:66-91)
    double b0[C0], bb[NB][CB];
#pragma unroll
    for (int c = 0; c < C0; ++c) b0[c] = 0.0;
#pragma unroll
    for (int k = 0; k < NB; ++k)
#pragma unroll
      for (int c = 0; c < CB; ++c) bb[k][c] = 0.0;
#pragma unroll 2
    for (int r = 0; r < R0; ++r) {
      const double dq = q[d.l2g[(r + 1) * ld + i]] - q0;
#pragma unroll
      for (int c = 0; c < C0; ++c) b0[c] += d.pinv[(c * R0 + r) * ld + i] * dq;
    }
#pragma unroll
    for (int k = 0; k < NB; ++k)
#pragma unroll
      for (int r = 0; r < RB; ++r) {
        const int l = d.bloc[(k * RB + r) * ld + i];
        const double dq = q[d.l2g[l * ld + i]] - q0;
#pragma unroll
        for (int c = 0; c < CB; ++c) bb[k][c] += d.pinv[(R0 * C0 + (k * CB + c) * RB + r) * ld + i] * dq;
      }
    // CWENO-AO central polynomial (cweno_ao.cpp:35-53), or WENO-AO's p_opt
    double pf[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      double x = c < C0 ? b0[c] : 0.0;
      if (!P.weno_ao) {
#pragma unroll
        for (int k = 0; k < NB; ++k)
          if (c < CB) x -= P.lw[k + 1] * bb[k][c];
        x *= P.inv_lw0;
      }
      pf[c] = x;
    }
    // eno_hybridize with the tracer's own smoothness indicators
    auto weight = [&](double IS, double g) {
      const double pw = P.exponent == 4.0 ? (IS * IS) * (IS * IS) : pow(IS, P.exponent);
      return g / (P.epsilon + pw);
    };
    double alpha[NB + 1];
    {
      double is = 0.0;
#pragma unroll
      for (int c = 0; c < C0; ++c) is += pf[c] * pf[c];
      alpha[0] = weight(is, P.lw[0]);
    }
#pragma unroll
    for (int k = 0; k < NB; ++k) {
      double is = 0.0;
#pragma unroll
      for (int c = 0; c < CB; ++c) is += bb[k][c] * bb[k][c];
      alpha[k + 1] = weight(is, P.lw[k + 1]);
    }
    double al_tot = 0.0;
#pragma unroll
    for (int k = 0; k <= NB; ++k) al_tot += alpha[k];
    const double w0 = alpha[0] / al_tot;
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      double x = w0 * pf[c];
#pragma unroll
      for (int k = 0; k < NB; ++k)
        if (c < CB) x += (alpha[k + 1] / al_tot) * bb[k][c];
      pf[c] = x;
    }
    // values at the cell's face points
#pragma unroll
    for (int f = 0; f < NF; ++f) {
      const int cf = d.cface[f * ld + i];
      if (cf < 0) continue;
      const int e = cf >> 1;
#pragma unroll
      for (int qq = 0; qq < NQF; ++qq) {
        double X[ND], phi[NC];
#pragma unroll
        for (int k = 0; k < ND; ++k) X[k] = (d.fqx[(qq * ND + k) * lde + e] - xc[k]) * il;
        basis<ND, NC>(X, C, phi);
        double v = 0.0;
#pragma unroll
        for (int c = 0; c < NC; ++c) v += pf[c] * phi[c];
        ta.fv[((size_t)(f * NQF + qq) * na + t) * ld + i] = q0 + v;
      }
    }
  }
}

template <class S, int FLUX, int EQ, bool MIXED>
__global__ void __launch_bounds__(128) k_tracer_face(const DevData d, const Params P, StageArgs a, TracerArgs ta) {
  constexpr int NV = S::NV, ND = S::ND, NQF = S::NQF;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= d.n_edges || d.clock->done) return;
  const int lde = d.lde, ld = d.ld, na = ta.na;
  const int L = d.fL[e], R = d.fR[e];
  if (!d.factive[e] || R < 0) {
    for (int t = 0; t < na; ++t) ta.nf[(size_t)t * lde + e] = 0.0;
    return;
  }
  const int kL = d.fkL[e], kR = d.fkR[e];
  EqEval ev{P.gamma, P.gm1, P.inv_gm1};
  // the wave fan at every face point, from the stage's Euler face states
  HllcWaves<double> w[NQF];
  double wq[NQF];
#pragma unroll
  for (int qq = 0; qq < NQF; ++qq) {
    const size_t sL = (size_t)((kL * NQF + qq) * NV) * ld + L;
    const size_t sR = (size_t)((kR * NQF + qq) * NV) * ld + R;
    double uL[NV], uR[NV], wL[NV], wR[NV];
    if (!MIXED) {
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        uL[v] = a.fv[sL + (size_t)v * ld];
        uR[v] = a.fv[sR + (size_t)v * ld];
      }
    } else {
      const double phi = EQ ? d.phi_fq[qq * lde + e] : 0.0;
      mixed_base<S, EQ>(d, a, ev, L, phi, uL);
      mixed_base<S, EQ>(d, a, ev, R, phi, uR);
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        uL[v] += double(a.fv32[sL + (size_t)v * ld]);
        uR[v] += double(a.fv32[sR + (size_t)v * ld]);
      }
    }
    to_face<NV, ND>(uL, d.frame, lde, e, wL);
    to_face<NV, ND>(uR, d.frame, lde, e, wR);
    if (FLUX == 0) {
      w[qq] = hllc_waves<NV>(wL, wR, P.gamma);
    } else {
      w[qq].vL = wL[1] / wL[0];
      w[qq].vR = wR[1] / wR[0];
      w[qq].sR = rusanov_speed<NV>(wL, wR, P.gamma);
    }
    wq[qq] = d.fqw[qq * lde + e];
  }
  for (int t = 0; t < na; ++t) {
    double F = 0.0;
#pragma unroll
    for (int qq = 0; qq < NQF; ++qq) {
      const double qL = ta.fv[((size_t)(kL * NQF + qq) * na + t) * ld + L];
      const double qR = ta.fv[((size_t)(kR * NQF + qq) * na + t) * ld + R];
      F += wq[qq] * (FLUX == 0 ? hllc_tracer_flux(w[qq], qL, qR)
                               : rusanov_tracer_flux(w[qq].sR, w[qq].vL, w[qq].vR, qL, qR));
    }
    ta.nf[(size_t)t * lde + e] = F;
  }
}

template <class S>
__global__ void __launch_bounds__(128) k_tracer_update(const DevData d, const Params P, StageArgs a, TracerArgs ta) {
  constexpr int NF = S::NF;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.n_cells || d.clock->done || !(d.flags[i] & kInterior)) return;
  const int ld = d.ld, lde = d.lde, na = ta.na, s = a.stage;
  const bool last = s == P.n_stages - 1;
  int ef[NF];
  bool right[NF];
#pragma unroll
  for (int f = 0; f < NF; ++f) {
    const int cf = d.cface[f * ld + i];
    ef[f] = cf < 0 ? -1 : cf >> 1;
    right[f] = cf & 1;
  }
  const double iv = d.inv_vol[i];
  const double dt = d.clock->dt;
  bool finite = true;
  for (int t = 0; t < na; ++t) {
    double tend = 0.0;
#pragma unroll
    for (int f = 0; f < NF; ++f) {
      if (ef[f] < 0) continue;
      const double x = ta.nf[(size_t)t * lde + ef[f]];
      tend += right[f] ? x : -x;
    }
    tend *= iv;
    const size_t o = (size_t)t * ld + i;
    if (ta.tend_out) {
      ta.tend_out[o] = tend;
      continue;
    }
    double dudt = 0.0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      if (j > s) break;
      const double c = a.coef[j];
      if (c != 0.0) dudt += c * (j == s ? tend : ta.k[j][o]);
    }
    const double un = ta.u0[o] + dt * dudt;
    if (!last) {
      ta.k[s][o] = tend;
      ta.ux[o] = un;
    } else {
      if (ta.uprev) ta.uprev[o] = ta.u0[o];
      ta.u0[o] = un;
      finite = finite && isfinite(un);
    }
  }
  if (!finite) set_status(d.clock, kStNonFinite);
}

template <class S, bool MIXED>
void launch_tracer_p(const DevData &D, const Params &P, StageArgs &a, TracerArgs &ta, int n_cells, int n_edges,
                     bool eq, int flux, cudaStream_t stream) {
  const int nb = (n_cells + 127) / 128, nbe = (n_edges + 127) / 128;
  k_tracer_reconstruct<S><<<nb, 128, 0, stream>>>(D, P, ta);
  if (flux == 0) {
    if (eq)
      k_tracer_face<S, 0, 1, MIXED><<<nbe, 128, 0, stream>>>(D, P, a, ta);
    else
      k_tracer_face<S, 0, 0, MIXED><<<nbe, 128, 0, stream>>>(D, P, a, ta);
  } else {
    if (eq)
      k_tracer_face<S, 1, 1, MIXED><<<nbe, 128, 0, stream>>>(D, P, a, ta);
    else
      k_tracer_face<S, 1, 0, MIXED><<<nbe, 128, 0, stream>>>(D, P, a, ta);
  }
  k_tracer_update<S><<<nb, 128, 0, stream>>>(D, P, a, ta);
}

}  // namespace dev
}  // namespace zfvm
