// Radial gravity potentials phi(r) and phi'(r), evaluated on the host.
//
// The kernels never evaluate a potential: the solver set-up tabulates phi and
// grad phi at every quadrature point (and the mixed form's <phi>, var(phi))
// once, so any radial potential costs the same per stage.  The potentials are
// the ones ZisaFVM's Euler factory builds (model/euler_factory.cpp:60-121,
// model/gravity_decl.hpp, model/gravity_impl.hpp), all with RadialAlignment
// (chi = |x|, d chi / dx_k = x_k / (|x| + 1e-50)):
//   CONSTANT_RADIAL          phi = g r                          (ConstantGravity)
//   HARMONIC_RADIAL          phi = k r^2 / 2                    (new: the C2 benchmark's potential)
//   POLYTROPE_RADIAL         phi = -2 K rhoC sin(a c) / (a c),   (PolytropeGravity, gamma = 2 Lane-Emden)
//                            c = r + eps, a = sqrt(2 pi G / K), eps = DBL_MIN
//   POLYTROPE_JUMP_RADIAL    inner polytrope (rhoC, K_inner) below r_crit, outer
//                            (rhoC_outer, K_outer) above, rhoC_outer making phi
//                            continuous at r_crit (PolytropeGravityWithJump)
//   POINT_MASS_RADIAL        phi = G M / (X + r)                (PointMassGravity)
//   RADIAL_TABLE             linear interpolation of phi between tabulated
//                            radii (RadialGravity over NonUniformLinearInterpolation,
//                            math/linear_interpolation.hpp:14-45)
#pragma once

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <string>
#include <vector>

#include "host_common.hpp"
#include "zfvm.h"

namespace zfvm {

// PolytropeGravity (gravity_impl.hpp:29-58): the gamma = 2 Lane-Emden potential.
struct LaneEmden {
  double rhoC = 1.0, K = 1.0, G = 1.0;
  double alpha() const { return std::sqrt(2.0 * M_PI * G / K); }
  double phi(double r) const {
    const double a = alpha(), c = a * (r + DBL_MIN);
    return -2.0 * K * rhoC * std::sin(c) / c;
  }
  double dphi(double r) const {
    const double a = alpha(), c = a * (r + DBL_MIN);
    const double d = (std::cos(c) - std::sin(c) / c) / c;
    return -2.0 * K * rhoC * d * a;
  }
};

struct RadialPotential {
  int kind = ZFVM_GRAVITY_NONE;
  double g = 0.0;              // gravity_strength
  LaneEmden inner, outer;      // polytrope potentials
  double r_crit = 0.0;         // polytrope with a jump
  double GM = 0.0, X = 0.0;    // point mass
  std::vector<double> tr, tphi;  // table

  // Throws SetupError(ZFVM_EINVAL) on an unusable configuration.
  static RadialPotential from_scheme(const zfvm_scheme_desc &sc) {
    RadialPotential p;
    p.kind = sc.gravity;
    p.g = sc.gravity_strength;
    const double *a = sc.gravity_params;
    switch (p.kind) {
      case ZFVM_GRAVITY_NONE:
      case ZFVM_GRAVITY_CONSTANT_RADIAL:
      case ZFVM_GRAVITY_HARMONIC_RADIAL:
        break;
      case ZFVM_GRAVITY_POLYTROPE_RADIAL:
        p.inner = LaneEmden{a[0], a[1], a[2]};
        if (!(a[1] > 0.0) || !(a[2] > 0.0)) throw SetupError(ZFVM_EINVAL, "polytrope gravity needs K > 0 and G > 0");
        break;
      case ZFVM_GRAVITY_POLYTROPE_JUMP_RADIAL: {
        // PolytropeGravityWithJump's constructor (gravity_impl.hpp:70-76)
        p.r_crit = a[0];
        p.inner = LaneEmden{a[1], a[2], a[4]};
        p.outer = LaneEmden{1.0, a[3], a[4]};
        if (!(a[2] > 0.0) || !(a[3] > 0.0) || !(a[4] > 0.0))
          throw SetupError(ZFVM_EINVAL, "polytrope gravity with a jump needs K_inner, K_outer, G > 0");
        const double rhoC_outer = p.inner.phi(p.r_crit) / p.outer.phi(p.r_crit);
        p.outer = LaneEmden{rhoC_outer, a[3], a[4]};
        break;
      }
      case ZFVM_GRAVITY_POINT_MASS_RADIAL:
        p.GM = a[0] * a[1];
        p.X = a[2];
        break;
      case ZFVM_GRAVITY_RADIAL_TABLE: {
        if (sc.gravity_table_n < 2 || !sc.gravity_table_r || !sc.gravity_table_phi)
          throw SetupError(ZFVM_EINVAL, "tabulated gravity needs at least two radii and potentials");
        p.tr.assign(sc.gravity_table_r, sc.gravity_table_r + sc.gravity_table_n);
        p.tphi.assign(sc.gravity_table_phi, sc.gravity_table_phi + sc.gravity_table_n);
        for (size_t k = 1; k < p.tr.size(); ++k)
          if (!(p.tr[k] > p.tr[k - 1])) throw SetupError(ZFVM_EINVAL, "tabulated gravity radii must increase");
        break;
      }
      default:
        throw SetupError(ZFVM_EINVAL, "unknown gravity kind");
    }
    return p;
  }

  // NonUniformLinearInterpolation::index: the interval below the first
  // tabulated radius >= r (the first interval for r at or below the start).
  // The reference reads past the table beyond its last radius; here the
  // set-up checks every radius it evaluates (covers()).
  size_t interval(double r) const {
    const size_t i = (size_t)(std::lower_bound(tr.begin(), tr.end(), r) - tr.begin());
    return i == 0 ? 0 : i - 1;
  }
  bool covers(double r) const { return kind != ZFVM_GRAVITY_RADIAL_TABLE || r <= tr.back(); }

  double phi_r(double r) const {
    switch (kind) {
      case ZFVM_GRAVITY_CONSTANT_RADIAL: return g * r;
      case ZFVM_GRAVITY_HARMONIC_RADIAL: return 0.5 * g * r * r;
      case ZFVM_GRAVITY_POLYTROPE_RADIAL: return inner.phi(r);
      case ZFVM_GRAVITY_POLYTROPE_JUMP_RADIAL: return r < r_crit ? inner.phi(r) : outer.phi(r);
      case ZFVM_GRAVITY_POINT_MASS_RADIAL: return GM / (X + r);
      case ZFVM_GRAVITY_RADIAL_TABLE: {
        const size_t i = interval(r);
        const double w = (r - tr[i]) / (tr[i + 1] - tr[i]);
        return (1 - w) * tphi[i] + w * tphi[i + 1];
      }
      default: return 0.0;
    }
  }
  double dphi_r(double r) const {
    switch (kind) {
      case ZFVM_GRAVITY_CONSTANT_RADIAL: return g;
      case ZFVM_GRAVITY_HARMONIC_RADIAL: return g * r;
      case ZFVM_GRAVITY_POLYTROPE_RADIAL: return inner.dphi(r);
      case ZFVM_GRAVITY_POLYTROPE_JUMP_RADIAL: return r < r_crit ? inner.dphi(r) : outer.dphi(r);
      case ZFVM_GRAVITY_POINT_MASS_RADIAL: return -GM / ((X + r) * (X + r));
      case ZFVM_GRAVITY_RADIAL_TABLE: {
        const size_t i = interval(r);
        return (tphi[i + 1] - tphi[i]) / (tr[i + 1] - tr[i]);
      }
      default: return 0.0;
    }
  }
  double phi(const Vec3 &x) const { return phi_r(norm(x)); }
  // Gravity::dphi_dx (gravity_decl.hpp:29-32) with RadialAlignment::dx (:85-88)
  double dphi_dx(const Vec3 &x, int dir) const {
    const double r = norm(x);
    return dphi_r(r) * (x[dir] / (r + 1e-50));
  }
};

}  // namespace zfvm
