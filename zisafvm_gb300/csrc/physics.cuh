// Device-side Euler physics: ideal-gas EOS, physical flux, HLLC with Batten
// wave speeds and the Rusanov flux, in the face frame (normal momentum first).
//
// HLLC follows flux/hllc.hpp:17-176 of ZisaFVM; Euler::flux follows
// model/euler_impl.hpp:23-36; the EOS follows model/ideal_gas_eos.hpp.  The
// Rusanov flux has no counterpart in the reference; it uses the same call
// signature so it can replace HLLCBatten as the FluxLoop template argument.
#pragma once

#include <cuda_runtime.h>

namespace zfvm {
namespace dev {

// NV = n_dims + 2 variables: rho, m_1 .. m_ndim, E.  In two dimensions the third
// momentum of the reference is identically zero and is not stored.
template <int NV, class R>
struct State {
  R v[NV];
};

template <int NV, class R>
__device__ __forceinline__ R kinetic_energy(const R *u) {
  R m2 = u[1] * u[1];
#pragma unroll
  for (int d = 2; d < NV - 1; ++d) m2 += u[d] * u[d];
  return R(0.5) * m2 / u[0];
}

// IdealGasEOS::pressure(u) = (E - E_kin) (gamma - 1)
template <int NV, class R>
__device__ __forceinline__ R pressure(const R *u, R gamma) {
  return (u[NV - 1] - kinetic_energy<NV>(u)) * (gamma - R(1));
}

template <class R>
__device__ __forceinline__ R sound_speed(R rho, R p, R gamma) {
  return sqrt(gamma * p / rho);
}

// Euler::flux(u, p) in the face frame.
template <int NV, class R>
__device__ __forceinline__ void euler_flux(const R *u, R p, R *f) {
  R v = u[1] / u[0];
  f[0] = u[1];
  f[1] = v * u[1] + p;
#pragma unroll
  for (int d = 2; d < NV - 1; ++d) f[d] = v * u[d];
  f[NV - 1] = v * (u[NV - 1] + p);
}

template <class R>
struct RoeAverage {
  R ratio;
  __device__ __forceinline__ RoeAverage(R rhoL, R rhoR) : ratio(sqrt(rhoR / rhoL)) {}
  __device__ __forceinline__ R operator()(R qL, R qR) const { return (qL + qR * ratio) / (R(1) + ratio); }
};

// hllc_speeds<IdealGasEOS> (flux/hllc.hpp:35-81) and the contact speed s*:
// the wave fan of the face, with the pressures and normal velocities it used.
template <class R>
struct HllcWaves {
  R pL, pR, vL, vR, sL, s_star, sR;
};

template <int NV, class R>
__device__ __forceinline__ HllcWaves<R> hllc_waves(const R *uL, const R *uR, R gamma) {
  HllcWaves<R> w;
  w.pL = pressure<NV>(uL, gamma), w.pR = pressure<NV>(uR, gamma);
  R aL = sound_speed(uL[0], w.pL, gamma), aR = sound_speed(uR[0], w.pR, gamma);
  RoeAverage<R> roe(uL[0], uR[0]);
  w.vL = uL[1] / uL[0], w.vR = uR[1] / uR[0];
  R v_t = roe(w.vL, w.vR);
  R HL = (uL[NV - 1] + w.pL) / uL[0], HR = (uR[NV - 1] + w.pR) / uR[0];
  R H_t = roe(HL, HR);
  R vroe2 = R(0);
#pragma unroll
  for (int d = 1; d < NV - 1; ++d) {
    R a = roe(uL[d] / uL[0], uR[d] / uR[0]);
    vroe2 += a * a;
  }
  R a_t = sqrt((gamma - R(1)) * (H_t - R(0.5) * vroe2));
  w.sL = fmin(w.vL - aL, v_t - a_t);
  w.sR = fmax(w.vR + aR, v_t + a_t);
  w.s_star = (uR[1] * (w.sR - w.vR) - uL[1] * (w.sL - w.vL) + w.pL - w.pR) /
             (uR[0] * (w.sR - w.vR) - uL[0] * (w.sL - w.vL));
  return w;
}

// HLLCBatten<IdealGasEOS>::flux
template <int NV, class R>
__device__ __forceinline__ void hllc_flux(const R *uL, const R *uR, R gamma, R *nf) {
  const HllcWaves<R> w = hllc_waves<NV>(uL, uR, gamma);
  const R pL = w.pL, pR = w.pR, vL = w.vL, vR = w.vR, sL = w.sL, sR = w.sR, s_star = w.s_star;
  const bool left = R(0) <= s_star;
  const R *uK = left ? uL : uR;
  R pK = left ? pL : pR;
  euler_flux<NV>(uK, pK, nf);
  if (sL < R(0) && R(0) <= sR) {
    R sK = left ? sL : sR;
    R vK = left ? vL : vR;
    R cK = (sK - vK) / (sK - s_star);
    nf[0] += sK * (cK * uK[0] - uK[0]);
    nf[1] += sK * (cK * uK[0] * s_star - uK[1]);
#pragma unroll
    for (int d = 2; d < NV - 1; ++d) nf[d] += sK * (cK * uK[d] - uK[d]);
    nf[NV - 1] += sK * (cK * (uK[NV - 1] + (s_star - vK) * (uK[0] * s_star + pK / (sK - vK))) - uK[NV - 1]);
  }
}

// HLLCBatten::tracer_flux (flux/hllc.hpp:178-197): an advected variable mq
// upwinded on s*, with the star-state correction inside the fan.
__device__ __forceinline__ double hllc_tracer_flux(const HllcWaves<double> &w, double mqL, double mqR) {
  const bool left = 0.0 <= w.s_star;
  const double mqK = left ? mqL : mqR;
  const double vK = left ? w.vL : w.vR;
  const double fK = mqK * vK;
  if (w.sL < 0.0 && 0.0 < w.sR) {
    const double sK = left ? w.sL : w.sR;
    const double cK = (sK - vK) / (sK - w.s_star);
    return fK + sK * (cK * mqK - mqK);
  }
  return fK;
}

// Rusanov / local Lax-Friedrichs:
//   F = (F(uL) + F(uR)) / 2 - s_max (uR - uL) / 2,  s_max = max(|vL| + aL, |vR| + aR).
template <int NV, class R>
__device__ __forceinline__ void rusanov_flux(const R *uL, const R *uR, R gamma, R *nf) {
  R pL = pressure<NV>(uL, gamma), pR = pressure<NV>(uR, gamma);
  R aL = sound_speed(uL[0], pL, gamma), aR = sound_speed(uR[0], pR, gamma);
  R vL = uL[1] / uL[0], vR = uR[1] / uR[0];
  R smax = fmax(fabs(vL) + aL, fabs(vR) + aR);
  R fL[NV], fR[NV];
  euler_flux<NV>(uL, pL, fL);
  euler_flux<NV>(uR, pR, fR);
#pragma unroll
  for (int k = 0; k < NV; ++k) nf[k] = R(0.5) * (fL[k] + fR[k]) - R(0.5) * smax * (uR[k] - uL[k]);
}

// The Rusanov flux's speed s_max, and its flux of an advected variable:
// (mqL vL + mqR vR) / 2 - s_max (mqR - mqL) / 2.
template <int NV>
__device__ __forceinline__ double rusanov_speed(const double *uL, const double *uR, double gamma) {
  const double pL = pressure<NV>(uL, gamma), pR = pressure<NV>(uR, gamma);
  const double aL = sound_speed(uL[0], pL, gamma), aR = sound_speed(uR[0], pR, gamma);
  return fmax(fabs(uL[1] / uL[0]) + aL, fabs(uR[1] / uR[0]) + aR);
}
__device__ __forceinline__ double rusanov_tracer_flux(double smax, double vL, double vR, double mqL, double mqR) {
  return 0.5 * (mqL * vL + mqR * vR) - 0.5 * smax * (mqR - mqL);
}

}  // namespace dev
}  // namespace zfvm

namespace zfvm {
namespace dev {

// Perturbation form of the fluxes around a resting base state w = (rho_w, 0, E_w)
// (an equilibrium at the face point).  Inputs are the deviations dL, dR of the
// two face states from w; the output is F(w + dL, w + dR) - F(w), where
// F(w) = (0, p_w, 0, 0) in the face frame.  The pressure is carried as
// p_w + dp with dp = (gamma - 1)(dE - E_kin) and HLLC's c_K - 1 is formed
// directly, so every small quantity keeps its own relative precision in FP32
// and a vanishing perturbation gives an exactly vanishing result.
template <int NV, class R>
struct DevSide {
  R rho, m[NV - 2], dE, E, dp, p, v, a, H;
  __device__ __forceinline__ void set(const R *d, R rho_w, R E_w, R p_w, R gamma) {
    rho = rho_w + d[0];
    R m2 = R(0);
#pragma unroll
    for (int k = 0; k < NV - 2; ++k) {
      m[k] = d[1 + k];
      m2 += m[k] * m[k];
    }
    dE = d[NV - 1];
    E = E_w + dE;
    dp = (dE - R(0.5) * m2 / rho) * (gamma - R(1));
    p = p_w + dp;
    v = m[0] / rho;
    a = sqrt(gamma * p / rho);
    H = (E + p) / rho;
  }
  // F(u) - F(w) for this side
  __device__ __forceinline__ void dflux(R *f) const {
    f[0] = m[0];
    f[1] = v * m[0] + dp;
#pragma unroll
    for (int k = 1; k < NV - 2; ++k) f[1 + k] = v * m[k];
    f[NV - 1] = v * (E + p);
  }
};

template <int NV, class R>
__device__ __forceinline__ void hllc_flux_dev(const R *dL, const R *dR, R rho_w, R E_w, R gamma, R *df) {
  const R p_w = E_w * (gamma - R(1));
  DevSide<NV, R> L, Rr;
  L.set(dL, rho_w, E_w, p_w, gamma);
  Rr.set(dR, rho_w, E_w, p_w, gamma);
  const R ratio = sqrt(Rr.rho / L.rho);
  auto roe = [&](R a, R b) { return (a + b * ratio) / (R(1) + ratio); };
  const R v_t = roe(L.v, Rr.v);
  const R H_t = roe(L.H, Rr.H);
  R vroe2 = R(0);
#pragma unroll
  for (int k = 0; k < NV - 2; ++k) {
    R a = roe(L.m[k] / L.rho, Rr.m[k] / Rr.rho);
    vroe2 += a * a;
  }
  const R a_t = sqrt((gamma - R(1)) * (H_t - R(0.5) * vroe2));
  const R sL = fmin(L.v - L.a, v_t - a_t);
  const R sR = fmax(Rr.v + Rr.a, v_t + a_t);
  const R s_star = (Rr.m[0] * (sR - Rr.v) - L.m[0] * (sL - L.v) + (L.dp - Rr.dp)) /
                   (Rr.rho * (sR - Rr.v) - L.rho * (sL - L.v));
  const bool left = R(0) <= s_star;
  const DevSide<NV, R> &K = left ? L : Rr;
  K.dflux(df);
  if (sL < R(0) && R(0) <= sR) {
    const R sK = left ? sL : sR;
    const R vK = K.v;
    const R cm1 = (s_star - vK) / (sK - s_star);  // c_K - 1
    const R cK = R(1) + cm1;
    df[0] += sK * (cm1 * K.rho);
    df[1] += sK * (cK * K.rho * s_star - K.m[0]);
#pragma unroll
    for (int k = 1; k < NV - 2; ++k) df[1 + k] += sK * (cm1 * K.m[k]);
    df[NV - 1] += sK * (cm1 * K.E + cK * (s_star - vK) * (K.rho * s_star + K.p / (sK - vK)));
  }
}

template <int NV, class R>
__device__ __forceinline__ void rusanov_flux_dev(const R *dL, const R *dR, R rho_w, R E_w, R gamma, R *df) {
  const R p_w = E_w * (gamma - R(1));
  DevSide<NV, R> L, Rr;
  L.set(dL, rho_w, E_w, p_w, gamma);
  Rr.set(dR, rho_w, E_w, p_w, gamma);
  const R smax = fmax(fabs(L.v) + L.a, fabs(Rr.v) + Rr.a);
  R fL[NV], fR[NV];
  L.dflux(fL);
  Rr.dflux(fR);
#pragma unroll
  for (int k = 0; k < NV; ++k) df[k] = R(0.5) * (fL[k] + fR[k]) - R(0.5) * smax * (dR[k] - dL[k]);
}

}  // namespace dev
}  // namespace zfvm
