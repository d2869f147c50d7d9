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

// HLLCBatten<IdealGasEOS>::flux
template <int NV, class R>
__device__ __forceinline__ void hllc_flux(const R *uL, const R *uR, R gamma, R *nf) {
  R pL = pressure<NV>(uL, gamma), pR = pressure<NV>(uR, gamma);
  R aL = sound_speed(uL[0], pL, gamma), aR = sound_speed(uR[0], pR, gamma);
  RoeAverage<R> roe(uL[0], uR[0]);
  R vL = uL[1] / uL[0], vR = uR[1] / uR[0];
  R v_t = roe(vL, vR);
  R HL = (uL[NV - 1] + pL) / uL[0], HR = (uR[NV - 1] + pR) / uR[0];
  R H_t = roe(HL, HR);
  R vroe2 = R(0);
#pragma unroll
  for (int d = 1; d < NV - 1; ++d) {
    R a = roe(uL[d] / uL[0], uR[d] / uR[0]);
    vroe2 += a * a;
  }
  R a_t = sqrt((gamma - R(1)) * (H_t - R(0.5) * vroe2));
  R sL = fmin(vL - aL, v_t - a_t);
  R sR = fmax(vR + aR, v_t + a_t);
  R s_star = (uR[1] * (sR - vR) - uL[1] * (sL - vL) + pL - pR) / (uR[0] * (sR - vR) - uL[0] * (sL - vL));
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

}  // namespace dev
}  // namespace zfvm
