// CPU ORACLE -- test infrastructure only.
//
// A restatement, in plain C++, of ZisaFVM's per-step rate-of-change and SSP-RK
// path.  It is the checker the GPU solver is compared against and the CPU
// baseline the benchmark times; nothing in the product (zisafvm_gb300) links or
// calls it.  Each function cites the reference file it follows (paths inside the
// ZisaFVM repository).  The reference itself cannot be compiled here (Eigen,
// Boost, HDF5 and the Zisa* sibling libraries are absent), so parity with the
// reference binary is unpinned; the pieces are pinned by the reference's own
// known-answer tests (tests/test_oracle_kat.py).
//
// Inputs are the reference's own: mesh vertices / vertex indices, ghost-cell
// mask, the stencil families (made once on the host, because the reference's
// last-resort stencil search is randomised), scheme parameters and the initial
// cell averages.  Geometry, quadrature, normalized moments and the LSQ matrices
// are recomputed here independently of the product code.
//
// Loop structure follows the reference's OpenMP structure:
// `omp parallel for schedule(static, 8)` over cells and faces, `omp atomic` for
// the face scatter, `reduction(min)` for the CFL time step.  With one thread
// every loop is serial and the result is deterministic.
#include <omp.h>

#include <algorithm>
#include <array>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <string>
#include <unordered_map>
#include <vector>

namespace oracle {

using idx = int64_t;

struct XYZ {
  double v[3] = {0, 0, 0};
  double &operator[](int i) { return v[i]; }
  double operator[](int i) const { return v[i]; }
};
static XYZ operator+(const XYZ &a, const XYZ &b) { return {{a[0] + b[0], a[1] + b[1], a[2] + b[2]}}; }
static XYZ operator-(const XYZ &a, const XYZ &b) { return {{a[0] - b[0], a[1] - b[1], a[2] - b[2]}}; }
static XYZ operator*(double s, const XYZ &a) { return {{s * a[0], s * a[1], s * a[2]}}; }
static XYZ operator/(const XYZ &a, double s) { return {{a[0] / s, a[1] / s, a[2] / s}}; }
static double dot(const XYZ &a, const XYZ &b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static double norm(const XYZ &a) { return std::sqrt(dot(a, a)); }
static XYZ cross(const XYZ &a, const XYZ &b) {
  return {{a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]}};
}
static XYZ normalize(const XYZ &a) { return a / norm(a); }

// 5 conserved variables: rho, mv1, mv2, mv3, E (model/euler_variables.hpp:36-48)
using Cv = std::array<double, 5>;

struct Error {
  int code;
  std::string msg;
};

// ------------------------------------------------------------ quadrature
// Reference-element rules (math/edge_rule.cpp, triangular_rule.cpp,
// tetrahedral_rule.cpp).  bary holds barycentric coordinates, or the [-1, 1]
// coordinate for edges.
struct Rule {
  std::vector<double> w;
  std::vector<std::array<double, 4>> x;
};

static void perm3(Rule &r, double w, double a, double b) {
  for (int k = 0; k < 3; ++k) r.w.push_back(w);
  r.x.push_back({a, b, b, 0});
  r.x.push_back({b, a, b, 0});
  r.x.push_back({b, b, a, 0});
}

static Rule edge_rule(int deg) {
  if (deg == -1) deg = 7;
  int n = deg / 2 + 1;
  Rule r;
  if (n == 1) {
    r.w = {1.0};
    r.x = {{0.0, 0, 0, 0}};
  } else if (n == 2) {
    double a = 1.0 / std::sqrt(3.0);
    r.w = {0.5, 0.5};
    r.x = {{-a, 0, 0, 0}, {a, 0, 0, 0}};
  } else if (n == 3) {
    double a = std::sqrt(3.0 / 5.0);
    r.w = {0.5 * 5.0 / 9.0, 0.5 * 8.0 / 9.0, 0.5 * 5.0 / 9.0};
    r.x = {{-a, 0, 0, 0}, {std::cos(M_PI / 2), 0, 0, 0}, {a, 0, 0, 0}};
  } else if (n == 4) {
    double s = 2.0 / 7.0 * std::sqrt(6.0 / 5.0);
    double a = std::sqrt(3.0 / 7.0 - s), b = std::sqrt(3.0 / 7.0 + s);
    double wa = (18.0 + std::sqrt(30.0)) / 36.0, wb = (18.0 - std::sqrt(30.0)) / 36.0;
    r.w = {0.5 * wb, 0.5 * wa, 0.5 * wa, 0.5 * wb};
    r.x = {{-b, 0, 0, 0}, {-a, 0, 0, 0}, {a, 0, 0, 0}, {b, 0, 0, 0}};
  } else {
    throw Error{1, "edge rule"};
  }
  return r;
}

static Rule tri_rule(int deg) {
  if (deg == -1) deg = 5;
  Rule r;
  switch (deg) {
    case 1:
      r.w = {1.0};
      r.x = {{1.0 / 3.0, 1.0 / 3.0, 1.0 / 3.0, 0}};
      break;
    case 2:
      perm3(r, 1.0 / 3.0, 2.0 / 3.0, 1.0 / 6.0);
      break;
    case 3:
      r.w = {-0.5625};
      r.x = {{1.0 / 3.0, 1.0 / 3.0, 1.0 / 3.0, 0}};
      perm3(r, 1.5625 / 3.0, 0.6, 0.2);
      break;
    case 4:
      perm3(r, 0.109951743655322, 0.816847572980459, 0.091576213509771);
      perm3(r, 0.223381589678011, 0.108103018168070, 0.445948490915965);
      break;
    case 5:
      r.w = {0.225};
      r.x = {{1.0 / 3.0, 1.0 / 3.0, 1.0 / 3.0, 0}};
      perm3(r, 0.132394152788506, 0.059715871789770, 0.470142064105115);
      perm3(r, 0.125939180544827, 0.797426985353087, 0.101286507323456);
      break;
    default:
      throw Error{1, "triangle rule"};
  }
  return r;
}

static Rule tet_rule(int deg) {
  if (deg == -1) deg = 3;
  Rule r;
  if (deg <= 1) {
    r.w = {1.0};
    r.x = {{0.25, 0.25, 0.25, 0.25}};
  } else if (deg == 2) {
    double a = 0.5854101966249680, b = 0.1381966011250110;
    r.w = {0.25, 0.25, 0.25, 0.25};
    r.x = {{a, b, b, b}, {b, a, b, b}, {b, b, a, b}, {b, b, b, a}};
  } else if (deg == 3) {
    double a = 0.7784952948213300, b = 0.0738349017262234, c = 0.4062443438840510, d = 0.0937556561159491;
    double wa = 0.0476331348432089, wc = 0.1349112434378610;
    r.w = {wa, wa, wa, wa, wc, wc, wc, wc, wc, wc};
    r.x = {{a, b, b, b}, {b, a, b, b}, {b, b, a, b}, {b, b, b, a}, {c, c, d, d},
           {c, d, c, d}, {c, d, d, c}, {d, c, c, d}, {d, c, d, c}, {d, d, c, c}};
  } else {
    throw Error{1, "tetrahedron rule"};
  }
  return r;
}

// DenormalizedRule (math/denormalized_rule.hpp:36-51)
struct QR {
  std::vector<double> w;
  std::vector<XYZ> x;
  double volume = 0;
};

static QR denormalize(const Rule &r, const XYZ *v, int nv, double vol) {
  QR q;
  q.volume = vol;
  for (size_t i = 0; i < r.w.size(); ++i) {
    q.w.push_back(vol * r.w[i]);
    if (nv == 2) {
      double xr = r.x[i][0];
      q.x.push_back((0.5 - 0.5 * xr) * v[0] + (0.5 + 0.5 * xr) * v[1]);  // math/edge.hpp coord
    } else {
      XYZ p;
      for (int d = 0; d < 3; ++d) {
        double s = v[0][d] * r.x[i][0];
        for (int k = 1; k < nv; ++k) s = s + v[k][d] * r.x[i][k];
        p[d] = s;
      }
      q.x.push_back(p);
    }
  }
  return q;
}

static double mul(double a, double b) { return a * b; }
static double add(double a, double b) { return a + b; }
static XYZ mul(double a, const XYZ &b) { return a * b; }
static XYZ add(const XYZ &a, const XYZ &b) { return a + b; }
static Cv mul(double a, const Cv &b) {
  Cv r;
  for (int k = 0; k < 5; ++k) r[k] = a * b[k];
  return r;
}
static Cv add(const Cv &a, const Cv &b) {
  Cv r;
  for (int k = 0; k < 5; ++k) r[k] = a[k] + b[k];
  return r;
}
using RhoE = std::array<double, 2>;
static RhoE mul(double a, const RhoE &b) { return {a * b[0], a * b[1]}; }
static RhoE add(const RhoE &a, const RhoE &b) { return {a[0] + b[0], a[1] + b[1]}; }


// quadrature(qr, f) and average (math/quadrature.hpp:33-62)
template <class T, class F>
static T quadrature(const QR &qr, const F &f) {
  T ret = mul(qr.w[0], f(qr.x[0]));
  for (size_t i = 1; i < qr.w.size(); ++i) ret = add(ret, mul(qr.w[i], f(qr.x[i])));
  return ret;
}
template <class T, class F>
static T average(const QR &qr, const F &f) {
  T q = quadrature<T>(qr, f);
  if constexpr (std::is_same_v<T, double>) {
    return q / qr.volume;
  } else if constexpr (std::is_same_v<T, XYZ>) {
    return q / qr.volume;
  } else {
    T r;
    for (size_t k = 0; k < r.size(); ++k) r[k] = q[k] / qr.volume;
    return r;
  }
}

// --------------------------------------------------------------- poly
static int poly_dof(int deg, int nd) {
  return nd == 2 ? ((deg + 1) * (deg + 2)) / 2 : ((deg + 1) * (deg + 2) * (deg + 3)) / 6;
}
static int pidx2(int a, int b) {
  int n = a + b;
  return ((n + 1) * n) / 2 + b;
}
static int pidx3(int a, int b, int c) { return poly_dof(a + b + c - 1, 3) + pidx2(b, c); }

// PolyND<35, 5> (math/poly2d_decl.hpp, poly2d_impl.hpp)
struct Poly {
  double a[35 * 5];
  double c[35];
  int degree = 0, n_dims = 0;
  XYZ xc;
  double len = 1.0;
  Poly() {
    std::fill(a, a + 175, 0.0);
    std::fill(c, c + 35, 0.0);
  }
  Poly(int deg, const std::vector<double> &moments, const XYZ &x_center, double length, int nd)
      : degree(deg), n_dims(nd), xc(x_center), len(length) {
    std::fill(a, a + 175, 0.0);
    std::fill(c, c + 35, 0.0);
    for (size_t i = 3; i < moments.size() && i < 35; ++i) c[i] = moments[i];
  }
  int dof() const { return poly_dof(degree, n_dims); }
  Cv eval(const XYZ &xyz) const {
    XYZ X = (xyz - xc) / len;
    Cv px{0, 0, 0, 0, 0};
    if (n_dims == 2) {
      double pxk = 1.0;
      for (int kx = 0; kx <= degree; ++kx) {
        double pyk = 1.0;
        for (int ky = 0; ky <= degree - kx; ++ky) {
          int i = pidx2(kx, ky);
          for (int k = 0; k < 5; ++k) px[k] += a[i * 5 + k] * (pxk * pyk - c[i]);
          pyk *= X[1];
        }
        pxk *= X[0];
      }
    } else {
      double pxk = 1.0;
      for (int kx = 0; kx <= degree; ++kx) {
        double pyk = 1.0;
        for (int ky = 0; ky <= degree - kx; ++ky) {
          double pzk = 1.0;
          for (int kz = 0; kz <= degree - kx - ky; ++kz) {
            int i = pidx3(kx, ky, kz);
            for (int k = 0; k < 5; ++k) px[k] += a[i * 5 + k] * (pxk * pyk * pzk - c[i]);
            pzk *= X[2];
          }
          pyk *= X[1];
        }
        pxk *= X[0];
      }
    }
    return px;
  }
};

// PointwiseSum / PointwiseSubtract / PointwiseScale assignment semantics
// (math/polynomial_expr.hpp): coefficients combine entry-wise, the moments,
// centre and length come from the higher-degree operand (the second on ties).
static void poly_axpy(Poly &lhs, double alpha, const Poly &rhs, double sign) {
  Poly out;
  const bool first = lhs.degree > rhs.degree;
  out.degree = std::max(lhs.degree, rhs.degree);
  out.n_dims = std::max(lhs.n_dims, rhs.n_dims);
  for (int i = 0; i < 175; ++i) out.a[i] = sign > 0 ? lhs.a[i] + alpha * rhs.a[i] : lhs.a[i] - alpha * rhs.a[i];
  for (int i = 0; i < 35; ++i) out.c[i] = first ? lhs.c[i] : rhs.c[i];
  out.xc = first ? lhs.xc : rhs.xc;
  out.len = first ? lhs.len : rhs.len;
  lhs = out;
}

static std::array<double, 5> smoothness_indicator(const Poly &p) {
  std::array<double, 5> b{0, 0, 0, 0, 0};
  int n = p.dof();
  for (int i = poly_dof(0, p.n_dims); i < n; ++i)
    for (int k = 0; k < 5; ++k) b[k] += p.a[i * 5 + k] * p.a[i * 5 + k];
  return b;
}

// ---------------------------------------------------------- physics
struct EOS {
  double gamma = 1.4, R = 1.0;
  double kinetic(const Cv &u) const { return 0.5 * (u[1] * u[1] + u[2] * u[2] + u[3] * u[3]) / u[0]; }
  double internal_energy(const Cv &u) const { return u[4] - kinetic(u); }
  double pressure_rhoE(double E) const { return E * (gamma - 1.0); }
  double pressure(const Cv &u) const { return pressure_rhoE(u[4] - kinetic(u)); }
  double sound_speed(double rho, double p) const { return std::sqrt(gamma * p / rho); }
  // xvars(u) -> (p, a)  (model/ideal_gas_eos.hpp:26-33)
  std::array<double, 2> xvars(const Cv &u) const {
    double p = pressure(u);
    return {p, sound_speed(u[0], pressure(u))};
  }
  std::array<double, 2> xvars_rhoE(const RhoE &r) const { return xvars(Cv{r[0], 0, 0, 0, r[1]}); }
  double rho_hK(double h, double K) const {
    double base = 1.0 / K * (gamma - 1.0) / gamma * h;
    return std::pow(base, 1.0 / (gamma - 1.0));
  }
  // enthalpy_entropy(RhoE) via rhoP(RhoE) (ideal_gas_eos.hpp:74-76,131-133,146-160):
  // h = gamma / (gamma - 1) p / rho, K = p / rho^gamma
  std::array<double, 2> hK_rhoE(const RhoE &r) const {
    double p = pressure_rhoE(r[1]);
    return {gamma / (gamma - 1.0) * p / r[0], p / std::pow(r[0], gamma)};
  }
  // rhoE(RhoP) (ideal_gas_eos.hpp:104-106): E = p / (gamma - 1)
  RhoE rhoE_rhoP(double rho, double p) const { return {rho, p / (gamma - 1.0)}; }
  // rhoE(EnthalpyEntropy)  (ideal_gas_eos.hpp:86-91,162-168,184-187)
  RhoE rhoE_hK(double h, double K) const {
    double rho = rho_hK(h, K);
    double p = K * std::pow(rho_hK(h, K), gamma);
    return {rho, p / (gamma - 1.0)};
  }
};

// Euler::flux (model/euler_impl.hpp:23-36)
static Cv euler_flux(const Cv &u, double p) {
  double v = u[1] / u[0];
  return {u[1], v * u[1] + p, v * u[2], v * u[3], v * (u[4] + p)};
}

// HLLCBatten<IdealGasEOS>::flux (flux/hllc.hpp:35-176); the wave speeds
// (s_L, s*, s_R) it returns beside the flux go to speeds when given.
static Cv hllc(const EOS &eos, const Cv &uL, const Cv &uR, double *speeds = nullptr) {
  auto xL = eos.xvars(uL), xR = eos.xvars(uR);
  double ratio = std::sqrt(uR[0] / uL[0]);
  auto roe = [&](double a, double b) { return (a + b * ratio) / (1.0 + ratio); };
  double pL = xL[0], aL = xL[1], pR = xR[0], aR = xR[1];
  double vL = uL[1] / uL[0], vR = uR[1] / uR[0];
  double v_t = roe(vL, vR);
  double HL = (uL[4] + pL) / uL[0], HR = (uR[4] + pR) / uR[0];
  double H_t = roe(HL, HR);
  double r1 = roe(uL[1] / uL[0], uR[1] / uR[0]), r2 = roe(uL[2] / uL[0], uR[2] / uR[0]),
         r3 = roe(uL[3] / uL[0], uR[3] / uR[0]);
  double vroe2 = r1 * r1 + r2 * r2 + r3 * r3;
  double a_t = std::sqrt((eos.gamma - 1.0) * (H_t - 0.5 * vroe2));
  double sL = std::min(vL - aL, v_t - a_t);
  double sR = std::max(vR + aR, v_t + a_t);
  double s_star = (uR[1] * (sR - vR) - uL[1] * (sL - vL) + pL - pR) / (uR[0] * (sR - vR) - uL[0] * (sL - vL));
  if (speeds) speeds[0] = sL, speeds[1] = s_star, speeds[2] = sR;
  const Cv &uK = 0.0 <= s_star ? uL : uR;
  double pK = 0.0 <= s_star ? pL : pR;
  Cv nf = euler_flux(uK, pK);
  if (sL < 0.0 && 0.0 <= sR) {
    double sK = 0.0 <= s_star ? sL : sR;
    double vK = 0.0 <= s_star ? uL[1] / uL[0] : uR[1] / uR[0];
    double cK = (sK - vK) / (sK - s_star);
    nf[0] += sK * (cK * uK[0] - uK[0]);
    nf[1] += sK * (cK * uK[0] * s_star - uK[1]);
    nf[2] += sK * (cK * uK[2] - uK[2]);
    nf[3] += sK * (cK * uK[3] - uK[3]);
    nf[4] += sK * (cK * (uK[4] + (s_star - vK) * (uK[0] * s_star + pK / (sK - vK))) - uK[4]);
  }
  return nf;
}

// Rusanov flux: a new flux with HLLCBatten's call signature; its one speed
// s_max goes to speeds[0] when given.
static Cv rusanov(const EOS &eos, const Cv &uL, const Cv &uR, double *speeds = nullptr) {
  auto xL = eos.xvars(uL), xR = eos.xvars(uR);
  double vL = uL[1] / uL[0], vR = uR[1] / uR[0];
  double smax = std::max(std::fabs(vL) + xL[1], std::fabs(vR) + xR[1]);
  if (speeds) speeds[0] = smax;
  Cv fL = euler_flux(uL, xL[0]), fR = euler_flux(uR, xR[0]);
  Cv nf;
  for (int k = 0; k < 5; ++k) nf[k] = 0.5 * (fL[k] + fR[k]) - 0.5 * smax * (uR[k] - uL[k]);
  return nf;
}

// HLLCBatten::tracer_flux (flux/hllc.hpp:178-197): the flux of an advected
// variable mq (a mass-weighted tracer) through the face, upwinded on s*, with
// the HLLC star-state correction when the fan straddles the face.  uL, uR are
// in the face frame.
static double tracer_flux_hllc(const Cv &uL, const Cv &uR, double mqL, double mqR, const double *speeds) {
  const double sL = speeds[0], s_star = speeds[1], sR = speeds[2];
  const double mqK = 0.0 <= s_star ? mqL : mqR;
  const double vK = 0.0 <= s_star ? uL[1] / uL[0] : uR[1] / uR[0];
  const double fK = mqK * vK;
  if (sL < 0.0 && 0.0 < sR) {
    const double sK = 0.0 <= s_star ? sL : sR;
    const double cK = (sK - vK) / (sK - s_star);
    return fK + sK * (cK * mqK - mqK);
  }
  return fK;
}

// The Rusanov flux of an advected variable (no counterpart in the reference,
// which has no Rusanov flux): (mqL vL + mqR vR) / 2 - s_max (mqR - mqL) / 2.
static double tracer_flux_rusanov(const Cv &uL, const Cv &uR, double mqL, double mqR, const double *speeds) {
  return 0.5 * (mqL * (uL[1] / uL[0]) + mqR * (uR[1] / uR[0])) - 0.5 * speeds[0] * (mqR - mqL);
}

// coord_transform / inv_coord_transform (model/euler_variables.cpp:29-67)
static void coord_transform(Cv &u, const XYZ &n, const XYZ &t1, const XYZ &t2) {
  double un = u[1] * n[0] + u[2] * n[1] + u[3] * n[2];
  double u1 = u[1] * t1[0] + u[2] * t1[1] + u[3] * t1[2];
  double u2 = u[1] * t2[0] + u[2] * t2[1] + u[3] * t2[2];
  u[1] = un, u[2] = u1, u[3] = u2;
}
static void inv_coord_transform(Cv &u, const XYZ &n, const XYZ &t1, const XYZ &t2) {
  double ux = u[1] * n[0] + u[2] * t1[0] + u[3] * t2[0];
  double uy = u[1] * n[1] + u[2] * t1[1] + u[3] * t2[1];
  double uz = u[1] * n[2] + u[2] * t1[2] + u[3] * t2[2];
  u[1] = ux, u[2] = uy, u[3] = uz;
}

// Gravity<Base, RadialAlignment> (model/gravity_decl.hpp:17-88, gravity_impl.hpp):
// chi = |x|, phi(x) = base.phi(chi), dphi/dx_k = base.dphi_dx(chi) x_k / (|x| + 1e-50).
// Bases: ConstantGravity (gravity_impl.hpp:12-19), the harmonic k chi^2 / 2 (new),
// PolytropeGravity (:29-58), PolytropeGravityWithJump (:70-92), PointMassGravity
// (:21-27) and SphericalGravity over NonUniformLinearInterpolation
// (:94-101, math/linear_interpolation.hpp:14-45).
struct PolytropeBase {
  double rhoC = 1.0, K = 1.0, G = 1.0, eps = std::numeric_limits<double>::min();
  double alpha() const { return std::sqrt(2.0 * M_PI * G / K); }  // gamma == 2
  double phi(double chi) const {
    double a = alpha();
    double chi_eff = a * (chi + eps);
    return -2.0 * K * rhoC * std::sin(chi_eff) / chi_eff;
  }
  double dphi_dx(double chi) const {
    double a = alpha();
    double chi_eff = a * (chi + eps);
    double dphi = (std::cos(chi_eff) - std::sin(chi_eff) / chi_eff) / chi_eff;
    return -2.0 * K * rhoC * dphi * a;
  }
};

struct Gravity {
  // 0 none, 1 constant radial (phi = g r), 2 harmonic radial (phi = k r^2 / 2),
  // 3 polytrope, 4 polytrope with a jump, 5 point mass, 6 tabulated
  int kind = 0;
  double g = 0.0;
  PolytropeBase inner, outer;
  double r_crit = 0.0;
  double GM = 0.0, X = 0.0;
  std::vector<double> tr, tphi;

  void set_params(const double *a) {
    if (kind == 3) inner = PolytropeBase{a[0], a[1], a[2]};
    if (kind == 4) {
      // PolytropeGravityWithJump::PolytropeGravityWithJump (gravity_impl.hpp:70-76)
      r_crit = a[0];
      inner = PolytropeBase{a[1], a[2], a[4]};
      outer = PolytropeBase{1.0, a[3], a[4]};
      double rhoC_outer = inner.phi(r_crit) / outer.phi(r_crit);
      outer = PolytropeBase{rhoC_outer, a[3], a[4]};
    }
    if (kind == 5) GM = a[0] * a[1], X = a[2];
  }
  // NonUniformLinearInterpolation::index
  size_t index(double r) const {
    auto first_past = std::lower_bound(tr.begin(), tr.end(), r);
    size_t i = (size_t)(first_past - tr.begin());
    return i == 0 ? 0 : i - 1;
  }
  double base_phi(double chi) const {
    switch (kind) {
      case 1: return g * chi;
      case 2: return 0.5 * g * chi * chi;
      case 3: return inner.phi(chi);
      case 4: return chi < r_crit ? inner.phi(chi) : outer.phi(chi);
      case 5: return GM / (X + chi);
      case 6: {
        size_t i = index(chi);
        double alpha = (chi - tr[i]) / (tr[i + 1] - tr[i]);
        return (1 - alpha) * tphi[i] + alpha * tphi[i + 1];
      }
      default: return 0.0;
    }
  }
  double base_dphi(double chi) const {
    switch (kind) {
      case 1: return g;
      case 2: return g * chi;
      case 3: return inner.dphi_dx(chi);
      case 4: return chi < r_crit ? inner.dphi_dx(chi) : outer.dphi_dx(chi);
      case 5: return -GM / ((X + chi) * (X + chi));
      case 6: {
        size_t i = index(chi);
        return (tphi[i + 1] - tphi[i]) / (tr[i + 1] - tr[i]);
      }
      default: return 0.0;
    }
  }
  double phi(const XYZ &x) const { return base_phi(norm(x)); }
  XYZ grad_phi(const XYZ &x) const {
    double d = base_dphi(norm(x));
    XYZ r;
    for (int k = 0; k < 3; ++k) r[k] = d * (x[k] / (norm(x) + 1e-50));
    return r;
  }
};

// quasi_newton (math/quasi_newton.hpp:12-50): x -= inv_df(x)(f(x)) until every
// |dx_k| <= atol_k, at most max_iter steps.  From the fifth step on, the step
// must be converging in the sense of RollingConvergenceRate::is_converging(0)
// (math/rolling_convergence_rate.hpp): the last step within atol (compared
// signed, as there), or every component's rate log(|c| / |b|) / log(|b| / |a|)
// over the last three steps at least 0.  Returns 0 when converged; 2 when not
// converging (the reference logs an error); 1 when max_iter steps end more than
// 1000 atol away (the reference warns).  On 1 and 2, x is put back to its start.
template <size_t N, class F, class IDF>
static int quasi_newton(const F &f, const IDF &inv_df, std::array<double, N> &x, const std::array<double, N> &atol,
                        int max_iter = 20) {
  const std::array<double, N> x0 = x;
  std::array<double, N> fx = f(x), dx;
  for (size_t k = 0; k < N; ++k) dx[k] = 2.0 * atol[k] + 1.0;
  auto within = [&](double factor) {
    for (size_t k = 0; k < N; ++k)
      if (!(std::fabs(dx[k]) <= factor * atol[k])) return false;
    return true;
  };
  std::vector<std::array<double, N>> hist;
  int iter = 0;
  while (!within(1.0) && iter < max_iter) {
    dx = inv_df(x, fx);
    for (size_t k = 0; k < N; ++k) x[k] -= dx[k];
    fx = f(x);
    hist.push_back(dx);
    if (iter >= 4) {
      const auto &a = hist[hist.size() - 3], &b = hist[hist.size() - 2], &c = hist[hist.size() - 1];
      bool conv = true;
      for (size_t k = 0; k < N; ++k) conv = conv && c[k] <= atol[k];
      if (!conv) {
        bool ok = true;
        for (size_t k = 0; k < N; ++k) {
          double r = std::log(std::fabs(c[k]) / std::fabs(b[k])) / std::log(std::fabs(b[k]) / std::fabs(a[k]));
          ok = ok && r >= 0.0;
        }
        if (!ok) {
          x = x0;
          return 2;
        }
      }
    }
    ++iter;
  }
  if (iter == max_iter && !within(1000.0)) {
    x = x0;
    return 1;
  }
  return 0;
}

// IsentropicEquilibrium + LocalEquilibriumBase (model/isentropic_equilibrium.hpp,
// local_equilibrium_impl.hpp:40-94,160-186), solved by quasi_newton.
struct LocalEq {
  const EOS *eos = nullptr;
  const Gravity *grav = nullptr;
  double h = 0, K = 0;
  XYZ x_ref;
  bool found = false;

  RhoE extrapolate_theta(double h_ref, double K_ref, const XYZ &xr, const XYZ &x) const {
    double hh = h_ref + grav->phi(xr) - grav->phi(x);
    return eos->rhoE_hK(hh, K_ref);
  }
  RhoE extrapolate(const XYZ &x) const {
    if (!found) return {0.0, 0.0};
    return extrapolate_theta(h, K, x_ref, x);
  }
  // (rhoE, (p, a)) -- full_variables (model/equilibrium_values.hpp:33-37)
  std::pair<RhoE, std::array<double, 2>> extrapolate_full(const XYZ &x) const {
    if (!found) return {{0.0, 0.0}, {0.0, 0.0}};
    RhoE r = extrapolate_theta(h, K, x_ref, x);
    return {r, eos->xvars_rhoE(r)};
  }
  RhoE extrapolate_cell(const QR &cell) const {
    if (!found) return {0.0, 0.0};
    return average<RhoE>(cell, [&](const XYZ &x) { return extrapolate(x); });
  }
  // returns 0 ok, 1 not found (warning), 2 diverging (the reference aborts)
  int solve(const RhoE &rbar, const QR &cell) {
    x_ref = cell.x[0];
    const auto guess = eos->hK_rhoE(rbar);  // full_extra_variables(rhoE_bar): (h, s)
    auto f = [&](const std::array<double, 2> &t) {
      RhoE avg = average<RhoE>(cell, [&](const XYZ &x) { return extrapolate_theta(t[0], t[1], x_ref, x); });
      return RhoE{rbar[0] - avg[0], rbar[1] - avg[1]};
    };
    // central differences of f with step 1e-6 |x_dir|, and the 2 x 2 inverse
    auto inv_df = [&](const std::array<double, 2> &x, const RhoE &fx) {
      double df[2][2];
      for (int dir = 0; dir < 2; ++dir) {
        double eps = 1e-6 * std::fabs(x[dir]);
        std::array<double, 2> xp = x, xm = x;
        xp[dir] = x[dir] + 0.5 * eps * 1.0;
        xm[dir] = x[dir] - 0.5 * eps * 1.0;
        RhoE a = f(xp), b = f(xm);
        df[dir][0] = (a[0] - b[0]) / eps;
        df[dir][1] = (a[1] - b[1]) / eps;
      }
      double inv_det = 1.0 / (df[0][0] * df[1][1] - df[0][1] * df[1][0]);
      return std::array<double, 2>{inv_det * (df[1][1] * fx[0] - df[1][0] * fx[1]),
                                   inv_det * (-df[0][1] * fx[0] + df[0][0] * fx[1])};
    };
    std::array<double, 2> x = guess;
    const int status = quasi_newton(f, inv_df, x, std::array<double, 2>{1e-13 * guess[0], 1e-13 * guess[1]});
    found = status == 0;
    h = x[0];
    K = x[1];
    return status;
  }
};

// ------------------------------------------------------------------ grid
struct Grid {
  int nd = 2, nb = 3;
  idx n_cells = 0, n_int_edges = 0, n_edges = 0;
  std::vector<XYZ> vertices;
  std::vector<idx> vi, nbr, edge_idx;
  std::vector<std::pair<idx, idx>> lr;
  std::vector<double> volumes, inradii, char_len;
  std::vector<XYZ> centers;
  std::vector<QR> cells;
  std::vector<QR> faces;
  std::vector<XYZ> fn, ft1, ft2;
  std::vector<std::vector<double>> moments;
  std::vector<uint8_t> interior, ghost, ghost_l1;
  std::vector<idx> source;
};

static int rel_vertex(int nd, int k, int rel) {
  if (nd == 2) return (k + rel) % 3;
  static const int t[4][3] = {{0, 1, 3}, {0, 2, 1}, {0, 3, 2}, {1, 2, 3}};
  return t[k][rel];
}

static double herons(double a, double b, double c) {
  return 0.25 * std::sqrt((a + b + c) * (-a + b + c) * (a - b + c) * (a + b - c));
}

// Grid::Grid (grid/grid.cpp:651-723)
static void build_grid(Grid &g, int qe, int qv, int qm) {
  const int nd = g.nd, nb = g.nb;
  const idx n = g.n_cells;
  auto V = [&](idx i, int k) -> XYZ & { return g.vertices[g.vi[i * nb + k]]; };
  // enforce_standard_vertex_order (grid.cpp:152-203)
  for (idx i = 0; i < n; ++i) {
    if (nd == 2) {
      XYZ c = cross(V(i, 1) - V(i, 0), V(i, 2) - V(i, 0));
      if (c[2] < 0.0) std::swap(g.vi[i * nb + 1], g.vi[i * nb + 2]);
    } else {
      XYZ cc = 0.25 * (V(i, 0) + V(i, 1) + V(i, 2) + V(i, 3));
      for (int k = 0; k < 4; ++k) {
        XYZ a = V(i, rel_vertex(3, k, 0)), b = V(i, rel_vertex(3, k, 1)), c = V(i, rel_vertex(3, k, 2));
        XYZ nn = cross(b - a, c - a);
        XYZ fc = 1.0 / 3.0 * (a + b + c);
        if (dot(nn, fc - cc) < 0.0) {
          std::swap(g.vi[i * nb + 2], g.vi[i * nb + 3]);
          break;
        }
      }
    }
  }
  // compute_neighbours via shared vertices (grid.cpp:486-540)
  g.nbr.assign(n * nb, -1);
  {
    idx nvtx = (idx)g.vertices.size();
    std::vector<std::vector<idx>> vn(nvtx);
    for (idx i = 0; i < n; ++i)
      for (int k = 0; k < nb; ++k) vn[g.vi[i * nb + k]].push_back(i);
    for (idx v = 0; v < nvtx; ++v) {
      auto &c = vn[v];
      for (size_t a = 0; a < c.size(); ++a)
        for (size_t b = a + 1; b < c.size(); ++b) {
          idx i = c[a], j = c[b];
          bool si[4] = {false, false, false, false}, sj[4] = {false, false, false, false};
          for (int k = 0; k < nb; ++k)
            for (int l = 0; l < nb; ++l)
              if (g.vi[i * nb + k] == g.vi[j * nb + l]) si[k] = sj[l] = true;
          auto face_of = [&](const bool *s) {
            if (nd == 2) {
              for (int k = 0; k < 3; ++k)
                if (s[k] && s[(k + 1) % 3]) return k;
              return -1;
            }
            if (s[0] && s[1] && s[3]) return 0;
            if (s[0] && s[2] && s[1]) return 1;
            if (s[0] && s[3] && s[2]) return 2;
            if (s[1] && s[2] && s[3]) return 3;
            return -1;
          };
          int ki = face_of(si), kj = face_of(sj);
          if (ki < 0) continue;
          g.nbr[i * nb + ki] = j;
          g.nbr[j * nb + kj] = i;
        }
    }
  }
  // compute_edge_indices / compute_left_right (grid.cpp:385-442)
  idx n_int = 0;
  for (idx i = 0; i < n; ++i)
    for (int k = 0; k < nb; ++k)
      if (g.nbr[i * nb + k] >= 0 && i < g.nbr[i * nb + k]) ++n_int;
  g.n_int_edges = n_int;
  g.edge_idx.assign(n * nb, -1);
  idx ci = 0, ce = n_int;
  for (idx i = 0; i < n; ++i)
    for (int k = 0; k < nb; ++k) {
      idx j = g.nbr[i * nb + k];
      if (j < 0)
        g.edge_idx[i * nb + k] = ce++;
      else if (i < j)
        g.edge_idx[i * nb + k] = ci++;
      else {
        int kj = 0;
        for (int l = 0; l < nb; ++l)
          if (g.nbr[j * nb + l] == i) kj = l;
        g.edge_idx[i * nb + k] = g.edge_idx[j * nb + kj];
      }
    }
  g.n_edges = ce;
  g.lr.assign(g.n_edges, {-1, -1});
  for (idx i = 0; i < n; ++i)
    for (int k = 0; k < nb; ++k) {
      idx e = g.edge_idx[i * nb + k], j = g.nbr[i * nb + k];
      if (j >= 0) {
        if (i < j) g.lr[e] = {i, j};
      } else {
        g.lr[e] = {i, -1};
      }
    }
  // volumes, inradii, characteristic lengths (math/triangle.cpp, tetrahedron.cpp)
  g.volumes.resize(n);
  g.inradii.resize(n);
  g.char_len.resize(n);
  for (idx i = 0; i < n; ++i) {
    if (nd == 2) {
      XYZ A = V(i, 0), B = V(i, 1), C = V(i, 2);
      double a = norm(B - C), b = norm(A - C), c = norm(A - B);
      g.volumes[i] = herons(a, b, c);
      g.inradii[i] = 0.5 * std::sqrt((b + c - a) * (c + a - b) * (a + b - c) / (a + b + c));
      XYZ bc = (A + B + C) / 3.0;
      g.char_len[i] = std::max(std::max(norm(A - bc), norm(B - bc)), norm(C - bc));
    } else {
      XYZ v[4] = {V(i, 0), V(i, 1), V(i, 2), V(i, 3)};
      XYZ d1 = v[1] - v[0], d2 = v[2] - v[0], d3 = v[3] - v[0];
      double vol = 1.0 / 6.0 *
                   (d1[0] * d2[1] * d3[2] + d2[0] * d3[1] * d1[2] + d3[0] * d1[1] * d2[2] - d1[0] * d3[1] * d2[2] -
                    d2[0] * d1[1] * d3[2] - d3[0] * d2[1] * d1[2]);
      g.volumes[i] = std::fabs(vol);
      XYZ c = 0.25 * (v[0] + v[1] + v[2] + v[3]);
      double rin = DBL_MAX, l = 0.0;
      for (int k = 0; k < 4; ++k) {
        XYZ fa = v[rel_vertex(3, k, 0)], fb = v[rel_vertex(3, k, 1)], fc = v[rel_vertex(3, k, 2)];
        rin = std::min(rin, norm((fa + fb + fc) / 3.0 - c));
      }
      for (int k = 0; k < 4; ++k) l += 2.0 * norm(c - v[k]);
      g.inradii[i] = rin;
      g.char_len[i] = 0.25 * l;
    }
  }
  // cells and centres
  Rule cr = nd == 2 ? tri_rule(qv) : tet_rule(qv);
  g.cells.resize(n);
  g.centers.resize(n);
  for (idx i = 0; i < n; ++i) {
    XYZ v[4];
    for (int k = 0; k < nb; ++k) v[k] = V(i, k);
    g.cells[i] = denormalize(cr, v, nb, g.volumes[i]);
    g.centers[i] = average<XYZ>(g.cells[i], [](const XYZ &x) { return x; });
  }
  // faces (grid.cpp:587-612, math/face_factory.cpp)
  Rule fr = nd == 2 ? edge_rule(qe) : tri_rule(qe);
  g.faces.resize(g.n_edges);
  g.fn.resize(g.n_edges);
  g.ft1.resize(g.n_edges);
  g.ft2.resize(g.n_edges);
  for (idx i = 0; i < n; ++i)
    for (int k = 0; k < nb; ++k) {
      idx j = g.nbr[i * nb + k];
      if (j >= 0 && !(i < j)) continue;
      idx e = g.edge_idx[i * nb + k];
      XYZ v[3];
      for (int r = 0; r < nd; ++r) v[r] = V(i, rel_vertex(nd, k, r));
      double area;
      XYZ nn, t1;
      if (nd == 2) {
        area = norm(v[1] - v[0]);
        XYZ t = normalize(v[1] - v[0]);
        nn = XYZ{{t[1], -t[0], t[2]}};
        t1 = normalize(v[1] - v[0]);
      } else {
        area = herons(norm(v[1] - v[2]), norm(v[0] - v[2]), norm(v[0] - v[1]));
        nn = normalize(cross(v[1] - v[0], v[2] - v[0]));
        t1 = normalize(v[1] - v[0]);
      }
      g.faces[e] = denormalize(fr, v, nd, area);
      g.fn[e] = nn;
      g.ft1[e] = t1;
      g.ft2[e] = cross(nn, t1);
    }
  // normalized moments (grid.cpp:1049-1098, math/cell.cpp)
  int mdeg = qm == -1 ? (nd == 2 ? 5 : 3) : qm;
  Rule mr = nd == 2 ? tri_rule(mdeg) : tet_rule(mdeg);
  g.moments.resize(n);
  for (idx i = 0; i < n; ++i) {
    XYZ v[4];
    for (int k = 0; k < nb; ++k) v[k] = V(i, k);
    QR cell = denormalize(mr, v, nb, g.volumes[i]);
    XYZ c = average<XYZ>(cell, [](const XYZ &x) { return x; });
    double len = g.char_len[i];
    std::vector<double> m(poly_dof(mdeg, nd), 0.0);
    double len_d = 1.0;
    for (int d = 0; d <= mdeg; ++d) {
      for (int a = 0; a <= d; ++a) {
        if (nd == 2) {
          int b = d - a;
          auto f = [&](const XYZ &x) {
            XYZ r = x - c;
            return std::pow(r[0], (double)a) * std::pow(r[1], (double)b) * std::pow(r[2], 0.0);
          };
          m[pidx2(a, b)] = average<double>(cell, f) / len_d;
        } else {
          for (int b = 0; b <= d - a; ++b) {
            int cc = d - a - b;
            auto f = [&](const XYZ &x) {
              XYZ r = x - c;
              return std::pow(r[0], (double)a) * std::pow(r[1], (double)b) * std::pow(r[2], (double)cc);
            };
            m[pidx3(a, b, cc)] = average<double>(cell, f) / len_d;
          }
        }
      }
      len_d *= len;
    }
    g.moments[i] = m;
  }
}

// ------------------------------------------------------------------- LSQ
// assemble_{2,3}d_weno_ao_matrix (reconstruction/lsq_solver.cpp:232-467)
static std::vector<double> assemble(const Grid &g, const std::vector<idx> &st, int order, int &rows, int &cols) {
  const int nd = g.nd;
  rows = (int)st.size() - 1;
  cols = poly_dof(order - 1, nd) - 1;
  std::vector<double> A((size_t)rows * cols, 0.0);
  idx i0 = st[0];
  XYZ x0 = g.centers[i0];
  double l0 = g.char_len[i0];
  const auto &C0 = g.moments[i0];
  auto idx2 = [&](int a, int b) { return nd == 2 ? pidx2(a, b) : pidx3(a, b, 0); };
  for (int ii = 0; ii < rows; ++ii) {
    idx j = st[ii + 1];
    XYZ d = (g.centers[j] - x0) / l0;
    double x = d[0], y = d[1], z = d[2];
    double lj = g.char_len[j] / l0;
    const auto &Cj = g.moments[j];
    auto at = [&](int c) -> double & { return A[(size_t)ii * cols + c - 1]; };
    if (order >= 2) {
      at(idx2(1, 0)) = x;
      at(idx2(0, 1)) = y;
    }
    if (order >= 3) {
      int i20 = idx2(2, 0), i11 = idx2(1, 1), i02 = idx2(0, 2);
      double lj2 = lj * lj;
      at(i20) = x * x - C0[i20] + lj2 * Cj[i20];
      at(i11) = x * y - C0[i11] + lj2 * Cj[i11];
      at(i02) = y * y - C0[i02] + lj2 * Cj[i02];
      if (order >= 4) {
        int i30 = idx2(3, 0), i21 = idx2(2, 1), i12 = idx2(1, 2), i03 = idx2(0, 3);
        double x20 = x * x, x11 = x * y, x02 = y * y;
        double lj3 = lj2 * lj;
        at(i30) = x20 * x - C0[i30] + 3.0 * x * lj2 * Cj[i20] + lj3 * Cj[i30];
        at(i21) = x20 * y - C0[i21] + y * lj2 * Cj[i20] + 2.0 * x * lj2 * Cj[i11] + lj3 * Cj[i21];
        at(i12) = x11 * y - C0[i12] + x * lj2 * Cj[i02] + 2.0 * y * lj2 * Cj[i11] + lj3 * Cj[i12];
        at(i03) = x02 * y - C0[i03] + 3.0 * y * lj2 * Cj[i02] + lj3 * Cj[i03];
      }
    }
    if (nd == 3) {
      at(pidx3(0, 0, 1)) = z;
      if (order >= 3) {
        int i002 = pidx3(0, 0, 2), i101 = pidx3(1, 0, 1), i011 = pidx3(0, 1, 1);
        double lj2 = lj * lj;
        at(i002) = z * z - C0[i002] + lj2 * Cj[i002];
        at(i101) = x * z - C0[i101] + lj2 * Cj[i101];
        at(i011) = y * z - C0[i011] + lj2 * Cj[i011];
      }
    }
  }
  return A;
}

// Robust Cholesky with diagonal pivoting, M = P^T L D L^T P: the factorisation
// Eigen::LDLT applies to A^T A (lsq_solver.cpp:110-111).
struct LDLT {
  int n = 0;
  std::vector<double> L, D;
  std::vector<int> perm;
  void compute(std::vector<double> M, int size) {
    n = size;
    perm.resize(n);
    for (int i = 0; i < n; ++i) perm[i] = i;
    for (int k = 0; k < n; ++k) {
      int p = k;
      double best = std::fabs(M[(size_t)k * n + k]);
      for (int j = k + 1; j < n; ++j)
        if (std::fabs(M[(size_t)j * n + j]) > best) best = std::fabs(M[(size_t)j * n + j]), p = j;
      if (p != k) {
        std::swap(perm[k], perm[p]);
        for (int j = 0; j < n; ++j) std::swap(M[(size_t)k * n + j], M[(size_t)p * n + j]);
        for (int j = 0; j < n; ++j) std::swap(M[(size_t)j * n + k], M[(size_t)j * n + p]);
      }
      double dk = M[(size_t)k * n + k];
      std::vector<double> col(n, 0.0);
      for (int i = k + 1; i < n; ++i) col[i] = M[(size_t)i * n + k];
      for (int i = k + 1; i < n; ++i) {
        double lik = dk != 0.0 ? col[i] / dk : 0.0;
        for (int j = k + 1; j <= i; ++j) M[(size_t)i * n + j] -= lik * col[j];
        M[(size_t)i * n + k] = lik;
      }
      for (int i = k + 1; i < n; ++i)
        for (int j = k + 1; j < i; ++j) M[(size_t)j * n + i] = M[(size_t)i * n + j];
    }
    L.assign((size_t)n * n, 0.0);
    D.assign(n, 0.0);
    for (int i = 0; i < n; ++i) {
      D[i] = M[(size_t)i * n + i];
      L[(size_t)i * n + i] = 1.0;
      for (int j = 0; j < i; ++j) L[(size_t)i * n + j] = M[(size_t)i * n + j];
    }
  }
  void solve(const double *b, double *x) const {
    std::vector<double> y(n);
    for (int i = 0; i < n; ++i) y[i] = b[perm[i]];
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < i; ++j) y[i] -= L[(size_t)i * n + j] * y[j];
    for (int i = 0; i < n; ++i) y[i] = D[i] != 0.0 ? y[i] / D[i] : 0.0;
    for (int i = n - 1; i >= 0; --i)
      for (int j = i + 1; j < n; ++j) y[i] -= L[(size_t)j * n + i] * y[j];
    for (int i = 0; i < n; ++i) x[perm[i]] = y[i];
  }
};

struct LSQ {
  int order = 1, rows = 0, cols = 0;
  std::vector<double> A, P;  // P: optional external pseudo-inverse (cols x rows)
  LDLT ldlt;
};

// ------------------------------------------------------------ scheme
struct Scheme {
  int flux = 0;
  EOS eos;
  std::vector<double> lw;
  double eps = 1e-6, expo = 4.0;
  int stages = 3;
  double cfl = 0.45;
  int equilibrium = 0;
  Gravity grav;
  int flux_bc = 0;
  int boundary = 0;
  int steps_per_recompute = 1;
  double recompute_threshold = 0.0;
  int weno_ao = 0;  // reconstruction.mode: 0 CWENO-AO, 1 WENO-AO
  double reject_drho = 0.0;  // RejectLargeDensityChange drho_crit_rel (0: RejectNothing)
  int reject_max_exponent = 0;
  double heat_rate = 0.0, heat_r0 = 0.0, heat_r1 = 0.0;  // heating.{rate, lower_boundary, upper_boundary}
  int na = 0;  // advected variables (AllVariables::avars columns)
};

struct CellRC {
  // stencil family (reconstruction/stencil_family.cpp) and its LSQ solvers
  int ns = 0, k_high = 0;
  std::vector<idx> l2g;
  std::vector<int> order, size;
  std::vector<std::vector<int>> local;
  std::vector<LSQ> lsq;
  std::vector<double> lin_w;
  // LocalReconstruction state (local_reconstruction.hpp:23-197)
  Cv scale{0, 0, 0, 0, 0};
  LocalEq eq;
  std::vector<RhoE> rhoEbar;
  std::vector<std::pair<RhoE, std::array<double, 2>>> pv_cell;  // cell quadrature points
  std::vector<std::vector<std::pair<RhoE, std::array<double, 2>>>> pv_face;  // per local face, qp
  Poly poly;
  std::vector<Poly> tpoly;  // scalar polynomials of the advected variables (variable 0 used)
  idx steps_since = 0;
};

struct Problem {
  Grid g;
  Scheme s;
  std::vector<CellRC> rc;
  std::vector<idx> interior_cells, exterior_cells, interior_faces, exterior_faces;
  int lsq_mode = 0;  // 0: LDLT of the normal equations per call; 1: external pseudo-inverse
  int threads = 1;
};

// ------------------------------------------------- local reconstruction
static Cv cv_div(const Cv &a, const Cv &b) {
  Cv r;
  for (int k = 0; k < 5; ++k) r[k] = a[k] / b[k];
  return r;
}

static int compute_equilibrium(Problem &pr, idx i, const std::vector<Cv> &ul) {
  auto &rc = pr.rc[i];
  const auto &g = pr.g;
  const EOS &eos = pr.s.eos;
  const Cv &u0 = ul[0];
  RhoE self{u0[0], eos.internal_energy(u0)};
  // EulerScaling (model/characteristic_scale.hpp:23-32)
  auto xv = eos.xvars_rhoE(self);
  if (self[0] <= 0.0 || self[1] <= 0.0) return 3;
  rc.scale = {self[0], xv[1], xv[1], xv[1], self[1]};
  int st = 0;
  if (pr.s.equilibrium) st = rc.eq.solve(self, g.cells[i]);
  if (st == 2) return 4;
  // point_values_cache.update (few_points_cache.hpp:72-79)
  const QR &cell = g.cells[i];
  rc.pv_cell.resize(cell.x.size());
  for (size_t q = 0; q < cell.x.size(); ++q)
    rc.pv_cell[q] = pr.s.equilibrium ? rc.eq.extrapolate_full(cell.x[q])
                                     : std::make_pair(RhoE{0, 0}, std::array<double, 2>{0, 0});
  rc.pv_face.resize(g.nb);
  for (int k = 0; k < g.nb; ++k) {
    const QR &f = g.faces[g.edge_idx[i * g.nb + k]];
    rc.pv_face[k].resize(f.x.size());
    for (size_t q = 0; q < f.x.size(); ++q)
      rc.pv_face[k][q] = pr.s.equilibrium ? rc.eq.extrapolate_full(f.x[q])
                                          : std::make_pair(RhoE{0, 0}, std::array<double, 2>{0, 0});
  }
  rc.rhoEbar.resize(rc.l2g.size());
  for (size_t il = 0; il < rc.l2g.size(); ++il)
    rc.rhoEbar[il] = pr.s.equilibrium ? rc.eq.extrapolate_cell(g.cells[rc.l2g[il]]) : RhoE{0.0, 0.0};
  rc.steps_since = 0;
  return 0;
}

static Poly hybrid_poly(const Problem &pr, idx i, const std::vector<Cv> &ul);

// LocalReconstruction::compute + CWENO_AO::reconstruct_impl + HybridWENO
static int local_reconstruct(Problem &pr, idx i, std::vector<Cv> &ul) {
  auto &rc = pr.rc[i];
  int st = 0;
  // recompute_equilibrium (local_reconstruction.hpp:87-100)
  if (rc.steps_since % pr.s.steps_per_recompute == 0) {
    st = compute_equilibrium(pr, i, ul);
  } else {
    const Cv &u0 = ul[0];
    double rho = u0[0], E = pr.s.eos.internal_energy(u0);
    double d0 = (rho - rc.rhoEbar[0][0]) / rc.scale[0], d1 = (E - rc.rhoEbar[0][1]) / rc.scale[4];
    if (std::sqrt(d0 * d0 + d1 * d1) >= pr.s.recompute_threshold) st = compute_equilibrium(pr, i, ul);
  }
  if (st) return st;
  for (size_t il = 0; il < rc.l2g.size(); ++il) {
    ul[il][0] -= rc.rhoEbar[il][0];
    ul[il][4] -= rc.rhoEbar[il][1];
    ul[il] = cv_div(ul[il], rc.scale);
  }
  rc.poly = hybrid_poly(pr, i, ul);
  ++rc.steps_since;
  return 0;
}

// HybridWENO::compute_polys + CWENO_AO::reconstruct_impl / WENO_AO::reconstruct
// + eno_hybridize of the stencil values ul (local stencil order), for a
// WENOPoly (five variables) or a ScalarPoly (variable 0, the others zero).
static Poly hybrid_poly(const Problem &pr, idx i, const std::vector<Cv> &ul) {
  const auto &rc = pr.rc[i];
  const auto &g = pr.g;
  // compute_polys (hybrid_weno.cpp:255-276)
  std::vector<Poly> polys(rc.ns);
  const XYZ &xc = g.centers[i];
  double len = g.char_len[i];
  for (int k = 0; k < rc.ns; ++k) {
    const LSQ &ls = rc.lsq[k];
    if (ls.order == 1) {
      polys[k] = Poly(0, {0.0}, xc, len, g.nd);
    } else {
      polys[k] = Poly(ls.order - 1, g.moments[i], xc, len, g.nd);
      const int rows = ls.rows, cols = ls.cols;
      std::vector<double> rhs((size_t)rows * 5);
      for (int ig = 0; ig < rows; ++ig) {
        int il = rc.local[k][ig + 1];
        for (int v = 0; v < 5; ++v) rhs[(size_t)ig * 5 + v] = ul[il][v] - ul[0][v];
      }
      if (pr.lsq_mode == 1 && !ls.P.empty()) {
        for (int c = 0; c < cols; ++c)
          for (int v = 0; v < 5; ++v) {
            double s = 0.0;
            for (int r = 0; r < rows; ++r) s += ls.P[(size_t)c * rows + r] * rhs[(size_t)r * 5 + v];
            polys[k].a[(c + 1) * 5 + v] = s;
          }
      } else {
        // coeffs = ldlt.solve(A^T rhs)  (lsq_solver.cpp:116-149)
        for (int v = 0; v < 5; ++v) {
          std::vector<double> atb(cols, 0.0), x(cols);
          for (int c = 0; c < cols; ++c) {
            double s = 0.0;
            for (int r = 0; r < rows; ++r) s += ls.A[(size_t)r * cols + c] * rhs[(size_t)r * 5 + v];
            atb[c] = s;
          }
          ls.ldlt.solve(atb.data(), x.data());
          for (int c = 0; c < cols; ++c) polys[k].a[(c + 1) * 5 + v] = x[c];
        }
      }
    }
    for (int v = 0; v < 5; ++v) polys[k].a[v] = ul[0][v];
  }
  // CWENO_AO::reconstruct_impl (cweno_ao.cpp:35-53); WENO_AO::reconstruct
  // (weno_ao.cpp:14-24) hybridizes the fitted polynomials as they are
  if (!pr.s.weno_ao) {
    const int kh = rc.k_high;
    for (int k = 0; k < rc.ns; ++k)
      if (k != kh) poly_axpy(polys[kh], rc.lin_w[k], polys[k], -1.0);
    double alpha = 1.0 / rc.lin_w[kh];
    for (int t = 0; t < 175; ++t) polys[kh].a[t] = alpha * polys[kh].a[t];
  }
  // eno_hybridize (hybrid_weno.cpp:109-128)
  std::vector<double> nlw(rc.ns);
  double al_tot = 0.0;
  for (int k = 0; k < rc.ns; ++k) {
    auto beta = smoothness_indicator(polys[k]);
    double IS = *std::max_element(beta.begin(), beta.end());
    double al = rc.lin_w[k] / (pr.s.eps + std::pow(IS, pr.s.expo));
    nlw[k] = al;
    al_tot += al;
  }
  Poly p(0, {0.0}, XYZ{}, 1.0, 2);
  for (int k = 0; k < rc.ns; ++k) poly_axpy(p, nlw[k] / al_tot, polys[k], 1.0);
  return p;
}

// LocalReconstruction::compute_tracer (local_reconstruction.hpp:127-147) with
// EulerGlobalReconstruction::set_tracer_local (global_reconstruction_impl.hpp:
// 178-192): every advected variable is reconstructed on its own, from its raw
// cell averages, without equilibrium or scaling.
static void tracer_reconstruct(Problem &pr, idx i, const std::vector<double> &aq) {
  auto &rc = pr.rc[i];
  const int na = pr.s.na;
  rc.tpoly.resize(na);
  std::vector<Cv> ul(rc.l2g.size());
  for (int t = 0; t < na; ++t) {
    for (size_t l = 0; l < rc.l2g.size(); ++l) ul[l] = Cv{aq[(size_t)rc.l2g[l] * na + t], 0.0, 0.0, 0.0, 0.0};
    rc.tpoly[t] = hybrid_poly(pr, i, ul);
  }
}

// LocalReconstruction::operator()(x) at cached point values
static Cv rc_value(const CellRC &rc, const XYZ &x, const std::pair<RhoE, std::array<double, 2>> &bg) {
  Cv pv = rc.poly.eval(x);
  Cv u;
  Cv b{bg.first[0], 0.0, 0.0, 0.0, bg.first[1]};
  for (int k = 0; k < 5; ++k) u[k] = b[k] + rc.scale[k] * pv[k];
  return u;
}

// ------------------------------------------------------------- problem
static void build_lists(Problem &pr) {
  // FluxLoop constructor (fvm_loops/flux_loop.hpp:41-90), including the loose
  // `contains` test (lower_bound != end).
  const auto &g = pr.g;
  pr.interior_cells.clear();
  pr.exterior_cells.clear();
  for (idx i = 0; i < g.n_cells; ++i) {
    bool ext = false;
    for (idx j : pr.rc[i].l2g)
      if (g.ghost[j]) {
        ext = true;
        break;
      }
    (ext ? pr.exterior_cells : pr.interior_cells).push_back(i);
  }
  auto contains = [](const std::vector<idx> &c, idx i) { return std::lower_bound(c.begin(), c.end(), i) != c.end(); };
  pr.interior_faces.clear();
  pr.exterior_faces.clear();
  for (idx e = 0; e < g.n_int_edges; ++e) {
    idx iL = g.lr[e].first, iR = g.lr[e].second;
    bool is_int = !contains(pr.exterior_cells, iL) && !contains(pr.exterior_cells, iR);
    if (is_int)
      pr.interior_faces.push_back(e);
    else if (!(g.ghost[iL] && g.ghost[iR]))
      pr.exterior_faces.push_back(e);
  }
}

static int local_face_of(const Grid &g, idx i, idx e) {
  for (int k = 0; k < g.nb; ++k)
    if (g.edge_idx[i * g.nb + k] == e) return k;
  return -1;
}

// EulerGlobalReconstruction::compute + FluxLoop::compute_patch; aq / atend are
// the advected variables and their tendency, n_cells x na row-major.
static int compute_patch(Problem &pr, std::vector<Cv> &tend, const std::vector<Cv> &state, const std::vector<idx> &cells,
                         const std::vector<idx> &faces, const std::vector<double> &aq, std::vector<double> &atend) {
  const int na = pr.s.na;
  const auto &g = pr.g;
  int err = 0;
  const idx nc = (idx)cells.size();
#pragma omp parallel for schedule(static, 8) num_threads(pr.threads)
  for (idx ii = 0; ii < nc; ++ii) {
    idx i = cells[ii];
    auto &rc = pr.rc[i];
    std::vector<Cv> ul(rc.l2g.size());
    for (size_t l = 0; l < rc.l2g.size(); ++l) ul[l] = state[rc.l2g[l]];
    int st = local_reconstruct(pr, i, ul);
    if (st) {
#pragma omp critical
      err = st;
    }
    if (na) tracer_reconstruct(pr, i, aq);
  }
  if (err) return err;
  const idx nf = (idx)faces.size();
#pragma omp parallel for schedule(static, 8) num_threads(pr.threads)
  for (idx ie = 0; ie < nf; ++ie) {
    idx e = faces[ie];
    const QR &face = g.faces[e];
    idx iL = g.lr[e].first, iR = g.lr[e].second;
    int kL = local_face_of(g, iL, e), kR = local_face_of(g, iR, e);
    Cv nf{0, 0, 0, 0, 0};
    std::vector<double> qnf(na, 0.0);
    for (size_t q = 0; q < face.w.size(); ++q) {
      double w = face.w[q];
      const XYZ &x = face.x[q];
      Cv uL = rc_value(pr.rc[iL], x, pr.rc[iL].pv_face[kL][q]);
      Cv uR = rc_value(pr.rc[iR], x, pr.rc[iR].pv_face[kR][q]);
      coord_transform(uL, g.fn[e], g.ft1[e], g.ft2[e]);
      coord_transform(uR, g.fn[e], g.ft1[e], g.ft2[e]);
      double speeds[3] = {0.0, 0.0, 0.0};
      Cv f = pr.s.flux == 0 ? hllc(pr.s.eos, uL, uR, speeds) : rusanov(pr.s.eos, uL, uR, speeds);
      for (int k = 0; k < 5; ++k) nf[k] += w * f[k];
      // the advected variables (flux_loop.hpp:157-161)
      for (int t = 0; t < na; ++t) {
        const double qL = pr.rc[iL].tpoly[t].eval(x)[0], qR = pr.rc[iR].tpoly[t].eval(x)[0];
        qnf[t] += w * (pr.s.flux == 0 ? tracer_flux_hllc(uL, uR, qL, qR, speeds)
                                      : tracer_flux_rusanov(uL, uR, qL, qR, speeds));
      }
    }
    for (int t = 0; t < na; ++t) {
      const double qfL = qnf[t] / g.volumes[iL];
#pragma omp atomic
      atend[(size_t)iL * na + t] -= qfL;
      const double qfR = qnf[t] / g.volumes[iR];
#pragma omp atomic
      atend[(size_t)iR * na + t] += qfR;
    }
    inv_coord_transform(nf, g.fn[e], g.ft1[e], g.ft2[e]);
    for (int k = 0; k < 5; ++k) {
      double nfL = nf[k] / g.volumes[iL];
#pragma omp atomic
      tend[iL][k] -= nfL;
      double nfR = nf[k] / g.volumes[iR];
#pragma omp atomic
      tend[iR][k] += nfR;
    }
  }
  return 0;
}

// GravitySourceLoop (fvm_loops/gravity_source_loop.hpp:32-148)
static void gravity_source(Problem &pr, std::vector<Cv> &tend) {
  const auto &g = pr.g;
  if (pr.s.grav.kind == 0) return;
#pragma omp parallel for schedule(static, 8) num_threads(pr.threads)
  for (idx i = 0; i < g.n_cells; ++i) {
    const auto &rc = pr.rc[i];
    const QR &cell = g.cells[i];
    if (pr.s.equilibrium) {
      const XYZ &x_cell = g.centers[i];
      Cv s{0, 0, 0, 0, 0};
      for (int k = 0; k < g.nb; ++k) {
        idx e = g.edge_idx[i * g.nb + k];
        const QR &face = g.faces[e];
        // unit_outward_normal (math/face.cpp:24-27)
        double sg = dot(g.fn[e], face.x[0] - x_cell);
        double sign = sg > 0 ? 1.0 : (sg < 0 ? -1.0 : 0.0);
        XYZ n = sign * g.fn[e];
        Cv sf{0, 0, 0, 0, 0};
        for (size_t q = 0; q < face.w.size(); ++q) {
          double p_eq = rc.pv_face[k][q].second[0];
          Cv v{0.0, p_eq * n[0], p_eq * n[1], p_eq * n[2], 0.0};
          sf = q == 0 ? mul(face.w[q], v) : add(sf, mul(face.w[q], v));
        }
        s = add(s, sf);
      }
      Cv sd{0, 0, 0, 0, 0};
      for (size_t q = 0; q < cell.w.size(); ++q) {
        const XYZ &x = cell.x[q];
        const auto &bg = rc.pv_cell[q];
        Cv pv = rc.poly.eval(x);
        Cv du;
        for (int k = 0; k < 5; ++k) du[k] = rc.scale[k] * pv[k];
        Cv ueq{bg.first[0], 0.0, 0.0, 0.0, bg.first[1]};
        Cv u;
        for (int k = 0; k < 5; ++k) u[k] = ueq[k] + du[k];
        double drho = du[0];
        XYZ gp = pr.s.grav.grad_phi(x);
        double mg = u[1] * gp[0] + u[2] * gp[1] + u[3] * gp[2];
        Cv v{0.0, -drho * gp[0], -drho * gp[1], -drho * gp[2], -mg};
        sd = q == 0 ? mul(cell.w[q], v) : add(sd, mul(cell.w[q], v));
      }
      s = add(s, sd);
      for (int k = 0; k < 5; ++k) tend[i][k] += s[k] / cell.volume;
    } else {
      auto f = [&](const XYZ &x) {
        Cv u = rc_value(rc, x, {{0, 0}, {0, 0}});
        XYZ gp = pr.s.grav.grad_phi(x);
        double mg = u[1] * gp[0] + u[2] * gp[1] + u[3] * gp[2];
        return Cv{0.0, -u[0] * gp[0], -u[0] * gp[1], -u[0] * gp[2], -mg};
      };
      Cv a = average<Cv>(cell, f);
      for (int k = 0; k < 5; ++k) tend[i][k] += a[k];
    }
  }
}

// FluxBC / EquilibriumFluxBC (boundary/flux_bc.hpp:25-42, equilibrium_flux_bc.hpp:36-62)
static int flux_bc(Problem &pr, std::vector<Cv> &tend, const std::vector<Cv> &state) {
  const auto &g = pr.g;
  if (pr.s.flux_bc == 0) return 0;
  for (idx e = g.n_int_edges; e < g.n_edges; ++e) {
    idx i = g.lr[e].first;
    const QR &face = g.faces[e];
    if (pr.s.flux_bc == 1) {
      Cv u = state[i];
      coord_transform(u, g.fn[e], g.ft1[e], g.ft2[e]);
      auto xv = pr.s.eos.xvars(u);
      Cv f = euler_flux(u, xv[0]);
      inv_coord_transform(f, g.fn[e], g.ft1[e], g.ft2[e]);
      double fac = face.volume / g.volumes[i];
      for (int k = 0; k < 5; ++k) tend[i][k] -= fac * f[k];
    } else {
      LocalEq eq;
      eq.eos = &pr.s.eos;
      eq.grav = &pr.s.grav;
      const Cv &u = state[i];
      int st = eq.solve(RhoE{u[0], pr.s.eos.internal_energy(u)}, g.cells[i]);
      if (st == 2) return 4;
      auto flux = [&](const XYZ &x) {
        RhoE r = eq.extrapolate(x);
        Cv uu{r[0], 0.0, 0.0, 0.0, r[1]};
        auto xv = pr.s.eos.xvars(uu);
        Cv f = euler_flux(uu, xv[0]);
        inv_coord_transform(f, g.fn[e], g.ft1[e], g.ft2[e]);
        return f;
      };
      Cv f = quadrature<Cv>(face, flux);
      for (int k = 0; k < 5; ++k) tend[i][k] -= f[k] / g.volumes[i];
    }
  }
  return 0;
}

// SumRatesOfChange{Zero, FluxLoop, GravitySource, FluxBC} (ode/rate_of_change.cpp:21-54)
// Heating (model/heating.hpp:29-77): dE/dt += average over the cell of
// rho(x) * rate(x), rho from the reconstruction of this stage, rate = epsilon on
// lower_boundary <= |x| <= upper_boundary.
static void heating_source(Problem &pr, std::vector<Cv> &tend) {
  if (pr.s.heat_rate == 0.0) return;
  const auto &g = pr.g;
#pragma omp parallel for schedule(static, 8) num_threads(pr.threads)
  for (idx i = 0; i < g.n_cells; ++i) {
    const auto &rc = pr.rc[i];
    const QR &cell = g.cells[i];
    double acc = 0.0;
    for (size_t q = 0; q < cell.w.size(); ++q) {
      const XYZ &x = cell.x[q];
      const double r = std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
      const double rate = (pr.s.heat_r0 <= r && r <= pr.s.heat_r1) ? pr.s.heat_rate : 0.0;
      const auto bg = pr.s.equilibrium ? rc.pv_cell[q] : std::make_pair(RhoE{0, 0}, std::array<double, 2>{0, 0});
      const double f = rc_value(rc, x, bg)[0] * rate;
      acc = q == 0 ? cell.w[q] * f : acc + cell.w[q] * f;
    }
    tend[i][4] += acc / cell.volume;
  }
}

static int rate_of_change(Problem &pr, std::vector<Cv> &tend, const std::vector<Cv> &state,
                          const std::vector<double> &aq, std::vector<double> &atend) {
  for (auto &t : tend) t = Cv{0, 0, 0, 0, 0};
  atend.assign(aq.size(), 0.0);  // ZeroRateOfChange (ode/rate_of_change.cpp:49-54)
  int st = compute_patch(pr, tend, state, pr.interior_cells, pr.interior_faces, aq, atend);
  if (st) return st;
  st = compute_patch(pr, tend, state, pr.exterior_cells, pr.exterior_faces, aq, atend);
  if (st) return st;
  gravity_source(pr, tend);
  heating_source(pr, tend);
  return flux_bc(pr, tend, state);
}

// Ghost cells after a stage: periodic images copy their source (boundary 1);
// FrozenBC::apply (boundary/frozen_boundary_condition.cpp:39-55) writes back the
// values the ghost cells had when the step started, which are the values they
// were set to (boundary 2).
static void apply_bc(Problem &pr, std::vector<Cv> &u, const std::vector<Cv> &u_step, std::vector<double> &aq,
                     const std::vector<double> &aq_step) {
  const auto &g = pr.g;
  const int na = pr.s.na;
  if (pr.s.boundary == 1) {
    for (idx i = 0; i < g.n_cells; ++i)
      if (g.ghost[i]) {
        u[i] = u[g.source[i]];
        for (int t = 0; t < na; ++t) aq[(size_t)i * na + t] = aq[(size_t)g.source[i] * na + t];
      }
  } else if (pr.s.boundary == 2) {
    for (idx i = 0; i < g.n_cells; ++i)
      if (g.ghost[i]) {
        u[i] = u_step[i];
        for (int t = 0; t < na; ++t) aq[(size_t)i * na + t] = aq_step[(size_t)i * na + t];
      }
  }
}

// LocalCFL (model/local_cfl_condition_impl.hpp:24-40) with reduce::min
static double cfl_dt(Problem &pr, const std::vector<Cv> &u) {
  const auto &g = pr.g;
  double ret = DBL_MAX;
#pragma omp parallel for reduction(min : ret) num_threads(pr.threads)
  for (idx i = 0; i < g.n_cells; ++i) {
    auto xv = pr.s.eos.xvars(u[i]);
    double v2 = (u[i][1] * u[i][1] + u[i][2] * u[i][2] + u[i][3] * u[i][3]) / (u[i][0] * u[i][0]);
    double ev = std::sqrt(v2) + xv[1];
    ret = std::min(ret, g.inradii[i] / ev);
  }
  return pr.s.cfl * ret;
}

// RungeKutta::compute_step (ode/runge_kutta.cpp:146-202)
static int rk_step(Problem &pr, std::vector<Cv> &u0, std::vector<double> &q0, double dt) {
  const int S = pr.s.stages;
  double a[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, b[3] = {0, 0, 0};
  if (S == 1) {
    b[0] = 1.0;
  } else if (S == 2) {
    a[1][0] = 1.0;
    b[0] = 0.5, b[1] = 0.5;
  } else {
    a[1][0] = 1.0;
    a[2][0] = 0.25, a[2][1] = 0.25;
    b[0] = 1.0 / 6, b[1] = 1.0 / 6, b[2] = 2.0 / 3;
  }
  const idx n = (idx)u0.size();
  const size_t nq = q0.size();
  std::vector<std::vector<Cv>> k(S, std::vector<Cv>(n));
  std::vector<std::vector<double>> kq(S, std::vector<double>(nq));
  std::vector<Cv> ux(n);
  std::vector<double> qx(nq);
  // runge_kutta_sum over all of AllVariables (ode/runge_kutta.cpp:181-202)
  auto rk_sum = [&](const double *coef) {
#pragma omp parallel for schedule(static, 8) num_threads(pr.threads)
    for (idx i = 0; i < n; ++i)
      for (int v = 0; v < 5; ++v) {
        double dudt = 0.0;
        for (int s = 0; s < S; ++s)
          if (coef[s] != 0.0) dudt += coef[s] * k[s][i][v];
        ux[i][v] = u0[i][v] + dt * dudt;
      }
    for (size_t j = 0; j < nq; ++j) {
      double dqdt = 0.0;
      for (int s = 0; s < S; ++s)
        if (coef[s] != 0.0) dqdt += coef[s] * kq[s][j];
      qx[j] = q0[j] + dt * dqdt;
    }
  };
  int st = rate_of_change(pr, k[0], u0, q0, kq[0]);
  if (st) return st;
  for (int s = 1; s < S; ++s) {
    rk_sum(a[s]);
    apply_bc(pr, ux, u0, qx, q0);
    st = rate_of_change(pr, k[s], ux, qx, kq[s]);
    if (st) return st;
  }
  rk_sum(b);
  apply_bc(pr, ux, u0, qx, q0);
  u0.swap(ux);
  q0.swap(qx);
  return 0;
}

}  // namespace oracle

// =================================================================== C ABI
using namespace oracle;

struct zfvm_oracle {
  Problem pr;
  std::string err;
};

static thread_local std::string g_oracle_err;

extern "C" {

const char *zfvm_oracle_last_error(void) { return g_oracle_err.c_str(); }

// Scheme parameter vector (doubles):
//  [0] flux (0 HLLC, 1 Rusanov)   [1] gamma        [2] R
//  [3..7] linear weights          [8] epsilon      [9] exponent
//  [10] rk stages                 [11] cfl         [12] equilibrium (0/1)
//  [13] gravity kind              [14] gravity strength
//  [15] flux bc (0/1/2)           [16] boundary (0 none, 1 periodic copy, 2 frozen)
//  [17] steps_per_recompute       [18] recompute_threshold
//  [19] reconstruction (0 CWENO-AO, 1 WENO-AO)
//  [20] step rejection drho_crit_rel [21] step rejection max exponent
//  [22] heating rate              [23] heating r0   [24] heating r1
//  [25] advected variables         [26..30] gravity parameters
//  [31] gravity table length n     [32..] n radii, then n potentials
int zfvm_oracle_create(int n_dims, int64_t n_vertices, const double *vertices, int64_t n_cells, const int64_t *vi,
                       const uint8_t *ghost, const int64_t *source, int qe, int qv, int qm,
                       const int8_t *n_stencils, const int8_t *k_high, const int8_t *n_l2g, const int32_t *l2g,
                       const int8_t *order, const int8_t *size, const int8_t *local, int max_l2g, int max_st,
                       int max_sz, const double *scheme, zfvm_oracle **out) {
  try {
    auto o = std::make_unique<zfvm_oracle>();
    Problem &pr = o->pr;
    Grid &g = pr.g;
    g.nd = n_dims;
    g.nb = n_dims + 1;
    g.n_cells = n_cells;
    g.vertices.resize(n_vertices);
    for (int64_t i = 0; i < n_vertices; ++i) g.vertices[i] = XYZ{{vertices[3 * i], vertices[3 * i + 1], vertices[3 * i + 2]}};
    g.vi.assign(vi, vi + n_cells * g.nb);
    build_grid(g, qe, qv, qm);
    g.ghost.assign(n_cells, 0);
    g.interior.assign(n_cells, 1);
    g.ghost_l1.assign(n_cells, 0);
    g.source.resize(n_cells);
    for (idx i = 0; i < n_cells; ++i) {
      g.source[i] = source ? source[i] : i;
      if (ghost && ghost[i]) g.ghost[i] = 1, g.interior[i] = 0;
    }
    // mask_ghost_cells (grid.cpp:1122-1137)
    for (idx i = 0; i < n_cells; ++i)
      if (g.ghost[i])
        for (int k = 0; k < g.nb; ++k) {
          idx j = g.nbr[i * g.nb + k];
          if (j >= 0 && !g.ghost[j]) g.ghost_l1[i] = 1;
        }
    Scheme &s = pr.s;
    s.flux = (int)scheme[0];
    s.eos.gamma = scheme[1];
    s.eos.R = scheme[2];
    s.eps = scheme[8];
    s.expo = scheme[9];
    s.stages = (int)scheme[10];
    s.cfl = scheme[11];
    s.equilibrium = (int)scheme[12];
    s.grav.kind = (int)scheme[13];
    s.grav.g = scheme[14];
    s.flux_bc = (int)scheme[15];
    s.boundary = (int)scheme[16];
    s.steps_per_recompute = (int)scheme[17];
    s.recompute_threshold = scheme[18];
    s.weno_ao = (int)scheme[19];
    s.reject_drho = scheme[20];
    s.reject_max_exponent = (int)scheme[21];
    s.heat_rate = scheme[22];
    s.heat_r0 = scheme[23];
    s.heat_r1 = scheme[24];
    s.na = (int)scheme[25];
    if (s.na < 0) throw Error{7, "negative number of advected variables"};
    // [26..30] gravity parameters, [31] table length n, then n radii and n potentials
    s.grav.set_params(scheme + 26);
    if (s.grav.kind == 6) {
      const int64_t nt = (int64_t)scheme[31];
      if (nt < 2) throw Error{7, "tabulated gravity needs at least two radii"};
      s.grav.tr.assign(scheme + 32, scheme + 32 + nt);
      s.grav.tphi.assign(scheme + 32 + nt, scheme + 32 + 2 * nt);
    }
    pr.rc.resize(n_cells);
    for (idx i = 0; i < n_cells; ++i) {
      CellRC &rc = pr.rc[i];
      rc.ns = n_stencils[i];
      rc.k_high = k_high[i];
      rc.l2g.assign(l2g + i * max_l2g, l2g + i * max_l2g + n_l2g[i]);
      rc.eq.eos = &s.eos;
      rc.eq.grav = &s.grav;
      // HybridWENO linear weights normalised by their sum (hybrid_weno.cpp:199-216)
      std::vector<double> lw;
      if (rc.ns == 1 && order[i * max_st] == 1 && g.ghost[i] && !g.ghost_l1[i]) {
        lw = {1.0};
      } else {
        for (int k = 0; k < rc.ns; ++k) lw.push_back(scheme[3 + k]);
        if (rc.ns == 1 && order[i * max_st] == 1) lw = {1.0};
      }
      double tot = 0.0;
      for (double w : lw) tot += w;
      for (double w : lw) rc.lin_w.push_back(w / tot);
      rc.order.resize(rc.ns);
      rc.size.resize(rc.ns);
      rc.local.resize(rc.ns);
      rc.lsq.resize(rc.ns);
      for (int k = 0; k < rc.ns; ++k) {
        rc.order[k] = order[i * max_st + k];
        rc.size[k] = size[i * max_st + k];
        rc.local[k].assign(local + (i * max_st + k) * max_sz, local + (i * max_st + k) * max_sz + rc.size[k]);
        LSQ &ls = rc.lsq[k];
        ls.order = rc.order[k];
        if (ls.order >= 2) {
          std::vector<idx> st(rc.size[k]);
          for (int r = 0; r < rc.size[k]; ++r) st[r] = rc.l2g[rc.local[k][r]];
          ls.A = assemble(g, st, ls.order, ls.rows, ls.cols);
          std::vector<double> M((size_t)ls.cols * ls.cols, 0.0);
          for (int a = 0; a < ls.cols; ++a)
            for (int b2 = 0; b2 < ls.cols; ++b2) {
              double t = 0.0;
              for (int r = 0; r < ls.rows; ++r) t += ls.A[(size_t)r * ls.cols + a] * ls.A[(size_t)r * ls.cols + b2];
              M[(size_t)a * ls.cols + b2] = t;
            }
          ls.ldlt.compute(M, ls.cols);
        }
      }
    }
    build_lists(pr);
    *out = o.release();
    return 0;
  } catch (const Error &e) {
    g_oracle_err = e.msg;
    return 7;
  } catch (const std::exception &e) {
    g_oracle_err = e.what();
    return 1;
  }
}

int zfvm_oracle_destroy(zfvm_oracle *o) {
  delete o;
  return 0;
}

int zfvm_oracle_set_threads(zfvm_oracle *o, int threads) {
  o->pr.threads = std::max(1, threads);
  return 0;
}

// Use a given pseudo-inverse for stencil k of cell i (cols x rows row-major).
int zfvm_oracle_set_pinv(zfvm_oracle *o, int64_t i, int k, const double *P, int rows, int cols) {
  auto &ls = o->pr.rc[i].lsq[k];
  if (rows != ls.rows || cols != ls.cols) {
    g_oracle_err = "pseudo-inverse shape mismatch";
    return 1;
  }
  ls.P.assign(P, P + (size_t)rows * cols);
  return 0;
}

int zfvm_oracle_set_lsq_mode(zfvm_oracle *o, int mode) {
  o->pr.lsq_mode = mode;
  return 0;
}

static std::vector<Cv> load(const double *aos, idx n) {
  std::vector<Cv> u(n);
  for (idx i = 0; i < n; ++i)
    for (int k = 0; k < 5; ++k) u[i][k] = aos[i * 5 + k];
  return u;
}
static void store(const std::vector<Cv> &u, double *aos) {
  for (size_t i = 0; i < u.size(); ++i)
    for (int k = 0; k < 5; ++k) aos[i * 5 + k] = u[i][k];
}

// Advected variables of a call: n_cells x na row-major, zero when the caller
// passes none (only allowed with na = 0).
static bool load_avars(const Problem &pr, const double *avars, std::vector<double> &q) {
  q.assign((size_t)pr.g.n_cells * pr.s.na, 0.0);
  if (pr.s.na == 0) return true;
  if (!avars) {
    g_oracle_err = "the scheme has advected variables: pass them";
    return false;
  }
  std::copy(avars, avars + q.size(), q.begin());
  return true;
}

int zfvm_oracle_rate_of_change_av(zfvm_oracle *o, const double *state, const double *avars, double *tendency,
                                  double *atend) {
  auto u = load(state, o->pr.g.n_cells);
  std::vector<double> q, tq;
  if (!load_avars(o->pr, avars, q)) return 1;
  apply_bc(o->pr, u, u, q, q);
  std::vector<Cv> t(u.size());
  int st = rate_of_change(o->pr, t, u, q, tq);
  if (st) {
    g_oracle_err = st == 4 ? "equilibrium solve is not converging" : "non-physical state";
    return st;
  }
  const int na = o->pr.s.na;
  for (idx i = 0; i < o->pr.g.n_cells; ++i)
    if (o->pr.g.ghost[i]) {
      t[i] = Cv{0, 0, 0, 0, 0};
      for (int k = 0; k < na; ++k) tq[(size_t)i * na + k] = 0.0;
    }
  store(t, tendency);
  if (na && atend) std::copy(tq.begin(), tq.end(), atend);
  return 0;
}

int zfvm_oracle_rate_of_change(zfvm_oracle *o, const double *state, double *tendency) {
  return zfvm_oracle_rate_of_change_av(o, state, nullptr, tendency, nullptr);
}

// EulerGlobalReconstruction::compute for the given cells, then
// LocalReconstruction::operator()(x) (local_reconstruction.hpp:149-163) at one
// point per entry: background equilibrium + scale * polynomial.
int zfvm_oracle_reconstruct_eval(zfvm_oracle *o, const double *state, int64_t n, const int64_t *cells,
                                 const double *x, double *u) {
  Problem &pr = o->pr;
  auto s = load(state, pr.g.n_cells);
  std::vector<double> q((size_t)pr.g.n_cells * pr.s.na, 0.0);
  apply_bc(pr, s, s, q, q);
  std::vector<char> done(pr.g.n_cells, 0);
  for (int64_t k = 0; k < n; ++k) {
    const idx i = cells[k];
    if (i < 0 || i >= pr.g.n_cells) {
      g_oracle_err = "cell index out of range";
      return 1;
    }
    if (done[i]) continue;
    std::vector<Cv> ul(pr.rc[i].l2g.size());
    for (size_t l = 0; l < ul.size(); ++l) ul[l] = s[pr.rc[i].l2g[l]];
    const int st = local_reconstruct(pr, i, ul);
    if (st) {
      g_oracle_err = st == 4 ? "equilibrium solve is not converging" : "non-physical state";
      return st;
    }
    done[i] = 1;
  }
  for (int64_t k = 0; k < n; ++k) {
    const idx i = cells[k];
    const XYZ xyz{{x[3 * k], x[3 * k + 1], x[3 * k + 2]}};
    const auto bg = pr.s.equilibrium ? pr.rc[i].eq.extrapolate_full(xyz)
                                     : std::make_pair(RhoE{0, 0}, std::array<double, 2>{0, 0});
    const Cv v = rc_value(pr.rc[i], xyz, bg);
    for (int c = 0; c < 5; ++c) u[5 * k + c] = v[c];
  }
  return 0;
}

int zfvm_oracle_cfl_dt(zfvm_oracle *o, const double *state, double *dt) {
  auto u = load(state, o->pr.g.n_cells);
  std::vector<double> q((size_t)o->pr.g.n_cells * o->pr.s.na, 0.0);
  apply_bc(o->pr, u, u, q, q);
  *dt = cfl_dt(o->pr, u);
  return 0;
}

int zfvm_oracle_step_av(zfvm_oracle *o, double *state, double *avars, double dt) {
  auto u = load(state, o->pr.g.n_cells);
  std::vector<double> q;
  if (!load_avars(o->pr, avars, q)) return 1;
  apply_bc(o->pr, u, u, q, q);
  int st = rk_step(o->pr, u, q, dt);
  if (st) {
    g_oracle_err = st == 4 ? "equilibrium solve is not converging" : "non-physical state";
    return st;
  }
  store(u, state);
  if (o->pr.s.na) std::copy(q.begin(), q.end(), avars);
  return 0;
}

int zfvm_oracle_step(zfvm_oracle *o, double *state, double dt) { return zfvm_oracle_step_av(o, state, nullptr, dt); }

// TimeLoop without IO (fvm_loops/time_loop.cpp:36-81); the clock of the
// unpinned ZisaTimeStepping is restated as dt = min(dt_cfl, t_end - t).
int zfvm_oracle_run_av(zfvm_oracle *o, double *state, double *avars, int64_t n_steps, double t_end, double *t_io,
                       int64_t *steps_out) {
  Problem &pr = o->pr;
  auto u = load(state, pr.g.n_cells);
  std::vector<double> q;
  if (!load_avars(pr, avars, q)) return 1;
  apply_bc(pr, u, u, q, q);
  double t = *t_io;
  int64_t step = 0;
  // RejectLargeDensityChange (ode/step_rejection.cpp:17-56): factor and is_good
  const bool rejecting = pr.s.reject_drho > 0.0;
  const double min_factor = std::pow(2.0, -(double)std::max(0, pr.s.reject_max_exponent));
  double factor = 1.0;
  bool is_good = true;
  double dt = cfl_dt(pr, u) * (rejecting ? factor : 1.0);
  while (true) {
    bool fin = (n_steps > 0 && step >= n_steps) || (t_end > 0.0 && t_end - t <= 1e-12 * t_end);
    if (fin) break;
    double dts = dt;
    if (t_end > 0.0) dts = std::min(dts, t_end - t);
    std::vector<Cv> u1 = u;
    std::vector<double> q1 = q;
    int st = rk_step(pr, u1, q1, dts);
    if (st) {
      g_oracle_err = st == 4 ? "equilibrium solve is not converging" : "non-physical state";
      return st;
    }
    if (rejecting) {
      bool good = true;
      for (idx i = 0; i < (idx)u.size(); ++i)
        if (std::abs(u[i][0] - u1[i][0]) > pr.s.reject_drho * u[i][0]) good = false;
      if (!good) {
        is_good = false;
        factor = std::max(min_factor, std::min(factor / 2.0, 1.0));
        dt = factor * dts;  // TimeLoop::reject_step (time_loop.cpp:182-198)
        continue;
      }
      if (is_good) factor *= 2.0;
      is_good = true;
      factor = std::max(min_factor, std::min(factor, 1.0));
    }
    u.swap(u1);
    q.swap(q1);
    t += dts;
    step += 1;
    dt = cfl_dt(pr, u) * (rejecting ? factor : 1.0);
  }
  store(u, state);
  if (pr.s.na) std::copy(q.begin(), q.end(), avars);
  *t_io = t;
  if (steps_out) *steps_out = step;
  return 0;
}

int zfvm_oracle_run(zfvm_oracle *o, double *state, int64_t n_steps, double t_end, double *t_io, int64_t *steps_out) {
  return zfvm_oracle_run_av(o, state, nullptr, n_steps, t_end, t_io, steps_out);
}

// ------------------------------------------------ known-answer helpers
int zfvm_oracle_flux(int kind, double gamma, const double *uL, const double *uR, double *f) {
  EOS eos;
  eos.gamma = gamma;
  Cv a, b;
  for (int k = 0; k < 5; ++k) a[k] = uL[k], b[k] = uR[k];
  Cv r = kind == 0 ? hllc(eos, a, b) : rusanov(eos, a, b);
  for (int k = 0; k < 5; ++k) f[k] = r[k];
  return 0;
}

// Flux of an advected variable through a face (face-frame states): the
// numerical flux's speeds, then tracer_flux.
int zfvm_oracle_tracer_flux(int kind, double gamma, const double *uL, const double *uR, double qL, double qR,
                            double *f) {
  EOS eos;
  eos.gamma = gamma;
  Cv a, b;
  for (int k = 0; k < 5; ++k) a[k] = uL[k], b[k] = uR[k];
  double speeds[3] = {0.0, 0.0, 0.0};
  if (kind == 0) {
    hllc(eos, a, b, speeds);
    *f = tracer_flux_hllc(a, b, qL, qR, speeds);
  } else {
    rusanov(eos, a, b, speeds);
    *f = tracer_flux_rusanov(a, b, qL, qR, speeds);
  }
  return 0;
}

int zfvm_oracle_euler_flux(double gamma, const double *u, double *f) {
  EOS eos;
  eos.gamma = gamma;
  Cv a;
  for (int k = 0; k < 5; ++k) a[k] = u[k];
  Cv r = euler_flux(a, eos.pressure(a));
  for (int k = 0; k < 5; ++k) f[k] = r[k];
  return 0;
}

// p(x) for a scalar polynomial given by its coefficients and moments.
int zfvm_oracle_poly_eval(int n_dims, int n_coeffs, const double *coeffs, const double *moments, const double *x_center,
                          double length, const double *x, double *out) {
  Poly p;
  p.n_dims = n_dims;
  int deg = 0;
  while (poly_dof(deg + 1, n_dims) <= n_coeffs) ++deg;
  p.degree = deg;
  for (int i = 0; i < n_coeffs; ++i) p.a[i * 5] = coeffs[i], p.c[i] = moments[i];
  p.xc = XYZ{{x_center[0], x_center[1], x_center[2]}};
  p.len = length;
  *out = p.eval(XYZ{{x[0], x[1], x[2]}})[0];
  return 0;
}

// The potential of a scheme vector (entries [13], [14], [26..]) and its
// gradient at n points (n x 3): phi n, grad n x 3.
int zfvm_oracle_gravity(const double *scheme, int64_t n, const double *x, double *phi, double *grad) {
  Gravity grav;
  grav.kind = (int)scheme[13];
  grav.g = scheme[14];
  grav.set_params(scheme + 26);
  if (grav.kind == 6) {
    const int64_t nt = (int64_t)scheme[31];
    if (nt < 2) {
      g_oracle_err = "tabulated gravity needs at least two radii";
      return 1;
    }
    grav.tr.assign(scheme + 32, scheme + 32 + nt);
    grav.tphi.assign(scheme + 32 + nt, scheme + 32 + 2 * nt);
  }
  for (int64_t k = 0; k < n; ++k) {
    const XYZ xk{{x[3 * k], x[3 * k + 1], x[3 * k + 2]}};
    phi[k] = grav.phi(xk);
    const XYZ gk = grav.grad_phi(xk);
    for (int d = 0; d < 3; ++d) grad[3 * k + d] = gk[d];
  }
  return 0;
}

// LocalEquilibrium test: solve from a cell average on an explicit triangle and
// extrapolate to a point (model/local_equilibrium.cpp in the reference tests).
int zfvm_oracle_local_equilibrium(double gamma, double R, int gravity_kind, double g, const double *tri, int quad_deg,
                                  const double *rhoE_bar, const double *x, double *rhoE_out, double *theta_out) {
  EOS eos;
  eos.gamma = gamma;
  eos.R = R;
  Gravity grav;
  grav.kind = gravity_kind;
  grav.g = g;
  XYZ v[3];
  for (int k = 0; k < 3; ++k) v[k] = XYZ{{tri[3 * k], tri[3 * k + 1], tri[3 * k + 2]}};
  double vol = herons(norm(v[1] - v[2]), norm(v[0] - v[2]), norm(v[0] - v[1]));
  QR cell = denormalize(tri_rule(quad_deg), v, 3, vol);
  LocalEq eq;
  eq.eos = &eos;
  eq.grav = &grav;
  int st = eq.solve(RhoE{rhoE_bar[0], rhoE_bar[1]}, cell);
  RhoE r = eq.extrapolate(XYZ{{x[0], x[1], x[2]}});
  rhoE_out[0] = r[0];
  rhoE_out[1] = r[1];
  theta_out[0] = eq.h;
  theta_out[1] = eq.K;
  return st;
}

// Average of the isentropic equilibrium theta = (h, K) at x_ref over a triangle.
int zfvm_oracle_equilibrium_average(double gamma, int gravity_kind, double g, const double *theta, const double *x_ref,
                                    const double *tri, int quad_deg, double *rhoE_out) {
  EOS eos;
  eos.gamma = gamma;
  Gravity grav;
  grav.kind = gravity_kind;
  grav.g = g;
  XYZ v[3];
  for (int k = 0; k < 3; ++k) v[k] = XYZ{{tri[3 * k], tri[3 * k + 1], tri[3 * k + 2]}};
  double vol = herons(norm(v[1] - v[2]), norm(v[0] - v[2]), norm(v[0] - v[1]));
  QR cell = denormalize(tri_rule(quad_deg), v, 3, vol);
  LocalEq eq;
  eq.eos = &eos;
  eq.grav = &grav;
  XYZ xr{{x_ref[0], x_ref[1], x_ref[2]}};
  RhoE r = average<RhoE>(cell, [&](const XYZ &x) { return eq.extrapolate_theta(theta[0], theta[1], xr, x); });
  rhoE_out[0] = r[0];
  rhoE_out[1] = r[1];
  return 0;
}

// Runge-Kutta on the reference's mock ODEs (test/.../ode/runge_kutta.cpp):
// ode 0 constant 0.1, 1 u' = u, 2 u' = t^2; returns the max error at t_final.
double zfvm_oracle_rk_ode_error(int stages, int ode, double dt, double t_final) {
  double a[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, b[3] = {0, 0, 0}, c[3] = {0, 0, 0};
  if (stages == 1) {
    b[0] = 1.0;
  } else if (stages == 2) {
    a[1][0] = 1.0;
    b[0] = 0.5, b[1] = 0.5;
  } else {
    a[1][0] = 1.0;
    a[2][0] = 0.25, a[2][1] = 0.25;
    b[0] = 1.0 / 6, b[1] = 1.0 / 6, b[2] = 2.0 / 3;
  }
  for (int s = 0; s < stages; ++s)
    for (int j = 0; j < stages; ++j) c[s] += a[s][j];
  auto rhs = [&](double t, double u) { return ode == 0 ? 0.1 : (ode == 1 ? u : t * t); };
  const int n = 30 * 2 + 30 * 3;
  std::vector<double> u(n, 1.0), ux(n);
  std::vector<std::vector<double>> k(stages, std::vector<double>(n));
  double t = 0.0;
  while (t < t_final - 0.5 * dt) {
    for (int i = 0; i < n; ++i) k[0][i] = rhs(t, u[i]);
    for (int s = 1; s < stages; ++s) {
      for (int i = 0; i < n; ++i) {
        double d = 0.0;
        for (int j = 0; j < stages; ++j)
          if (a[s][j] != 0.0) d += a[s][j] * k[j][i];
        ux[i] = u[i] + dt * d;
      }
      for (int i = 0; i < n; ++i) k[s][i] = rhs(t + c[s] * dt, ux[i]);
    }
    for (int i = 0; i < n; ++i) {
      double d = 0.0;
      for (int j = 0; j < stages; ++j)
        if (b[j] != 0.0) d += b[j] * k[j][i];
      ux[i] = u[i] + dt * d;
    }
    u.swap(ux);
    t += dt;
  }
  double exact = ode == 0 ? 1.0 + 0.1 * t_final : (ode == 1 ? std::exp(t_final) : 1.0 + t_final * t_final * t_final / 3.0);
  double err = 0.0;
  for (int i = 0; i < n; ++i) err = std::max(err, std::fabs(u[i] - exact));
  return err;
}

// A reference-element rule: kind 0 edge (x: n coordinates in [-1, 1]), 1
// triangle (x: n x 3 barycentric), 2 tetrahedron (x: n x 4 barycentric);
// weights normalised to sum 1.  At most max_n points are written; *n gets the
// rule's size.
int zfvm_oracle_rule(int kind, int deg, int max_n, int *n, double *w, double *x) {
  try {
    const Rule r = kind == 0 ? edge_rule(deg) : (kind == 1 ? tri_rule(deg) : tet_rule(deg));
    const int m = (int)r.w.size(), nc = kind == 0 ? 1 : kind + 2;
    *n = m;
    if (m > max_n) {
      g_oracle_err = "rule larger than the buffers";
      return 1;
    }
    for (int q = 0; q < m; ++q) {
      w[q] = r.w[q];
      for (int c = 0; c < nc; ++c) x[q * nc + c] = r.x[q][c];
    }
    return 0;
  } catch (const Error &e) {
    g_oracle_err = e.msg;
    return e.code;
  }
}

// The EOS round trips of test/zisa/unit_test/model/eos.cpp:7-23 at (rho, E):
// out = {rhoE(enthalpy_entropy(rhoE)), rhoE(rhoP(rhoE))}, four numbers.
int zfvm_oracle_eos_roundtrips(double gamma, double R, double rho, double E, double *out) {
  EOS eos;
  eos.gamma = gamma;
  eos.R = R;
  const RhoE r{rho, E};
  const auto hK = eos.hK_rhoE(r);
  const RhoE a = eos.rhoE_hK(hK[0], hK[1]);
  const RhoE b = eos.rhoE_rhoP(r[0], eos.pressure_rhoE(r[1]));
  out[0] = a[0], out[1] = a[1], out[2] = b[0], out[3] = b[1];
  return 0;
}

// The problems of test/zisa/unit_test/math/quasi_newton.cpp:9-54 solved by the
// quasi_newton above.  which 0: x^2 - 1.2345^2 from 1.9 with the Newton
// inverse fx / (2 x0), atol 1e-10; which 1: f(h, K) = (h K + h - K, K) from
// (0.2, -0.4) with its exact inverse Jacobian at the current point, atol 1e-10
// (root (0, 0)).  x gets the result (one or two numbers); returns
// quasi_newton's status.
int zfvm_oracle_quasi_newton_problem(int which, double *x) {
  if (which == 0) {
    const double root = 1.2345;
    auto f = [root](const std::array<double, 1> &v) { return std::array<double, 1>{v[0] * v[0] - root * root}; };
    auto inv_df = [](const std::array<double, 1> &v, const std::array<double, 1> &fx) {
      return std::array<double, 1>{fx[0] / (2.0 * v[0])};
    };
    std::array<double, 1> v{1.9};
    const int st = quasi_newton(f, inv_df, v, std::array<double, 1>{1e-10});
    x[0] = v[0];
    return st;
  }
  auto f = [](const std::array<double, 2> &t) { return std::array<double, 2>{t[0] * t[1] + t[0] - t[1], t[1]}; };
  auto inv_df = [](const std::array<double, 2> &t, const std::array<double, 2> &fx) {
    const double h = t[0], K = t[1], inv_det = 1.0 / (K + 1.0);
    return std::array<double, 2>{inv_det * (fx[0] + (-h + 1.0) * fx[1]), inv_det * ((K + 1.0) * fx[1])};
  };
  std::array<double, 2> v{0.2, -0.4};
  const int st = quasi_newton(f, inv_df, v, std::array<double, 2>{1e-10, 1e-10});
  x[0] = v[0], x[1] = v[1];
  return st;
}

}  // extern "C"
