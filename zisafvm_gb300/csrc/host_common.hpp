// Host-side geometry and quadrature primitives used by the mesh set-up.
//
// Everything in this header runs once per mesh on the host; the per-stage hot
// path lives in the CUDA kernels.  Quadrature tables are the published rules the
// reference uses (Gauss-Legendre on edges, Strang-Fix/Dunavant on triangles,
// Keast-type rules on tetrahedra); see math/edge_rule.cpp, math/triangular_rule.cpp
// and math/tetrahedral_rule.cpp in ZisaFVM.
#pragma once

#include <array>
#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

namespace zfvm {

using index_t = int64_t;

struct Vec3 {
  double x = 0.0, y = 0.0, z = 0.0;
  double &operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
  double operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

inline Vec3 operator+(const Vec3 &a, const Vec3 &b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline Vec3 operator-(const Vec3 &a, const Vec3 &b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline Vec3 operator*(double s, const Vec3 &a) { return {s * a.x, s * a.y, s * a.z}; }
inline Vec3 operator/(const Vec3 &a, double s) { return {a.x / s, a.y / s, a.z / s}; }
inline double dot(const Vec3 &a, const Vec3 &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline Vec3 cross(const Vec3 &a, const Vec3 &b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline double norm(const Vec3 &a) { return std::sqrt(dot(a, a)); }
inline Vec3 normalize(const Vec3 &a) { return a / norm(a); }
// (x, y, z) -> (y, -x, z): outward normal of a counter-clockwise edge.
inline Vec3 rotate_right(const Vec3 &a) { return {a.y, -a.x, a.z}; }
inline double det3(const Vec3 &a, const Vec3 &b, const Vec3 &c) { return dot(a, cross(b, c)); }

struct SetupError : std::runtime_error {
  int code;
  SetupError(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

// ---- polynomial indexing (math/poly2d_impl.hpp:11-41 in ZisaFVM) -------------
inline int poly_dof(int deg, int n_dims) {
  if (deg < 0) return 0;
  return n_dims == 2 ? ((deg + 1) * (deg + 2)) / 2 : ((deg + 1) * (deg + 2) * (deg + 3)) / 6;
}
inline int poly_index2(int a, int b) {
  int n = a + b;
  return ((n + 1) * n) / 2 + b;
}
inline int poly_index3(int a, int b, int c) { return poly_dof(a + b + c - 1, 3) + poly_index2(b, c); }

// ---- reference-element quadrature rules --------------------------------------
struct RefRule {
  std::vector<double> w;                   // weights, summing to 1
  std::vector<std::array<double, 4>> bary;  // barycentric coords (2 used on edges)
};

// Gauss-Legendre on [-1, 1], weights halved so they sum to one; `x` holds the
// point in bary[i][0].  n_points = deg / 2 + 1 (math/edge_rule.cpp:10-30).
RefRule edge_rule(int deg);
// Triangle rules of degree 1..5 (math/triangular_rule.cpp:33-90).
RefRule triangle_rule(int deg);
// Tetrahedron rules of degree 1..3 (math/tetrahedral_rule.cpp).
RefRule tetra_rule(int deg);

constexpr int kMaxTriangleRuleDegree = 5;
constexpr int kMaxTetraRuleDegree = 3;

// Relative vertex index of vertex `rel` on face `k` (grid/gmsh_reader.cpp:23-57).
inline int face_vertex(int n_dims, int k, int rel) {
  if (n_dims == 2) return (k + rel) % 3;
  static const int tab[4][3] = {{0, 1, 3}, {0, 2, 1}, {0, 3, 2}, {1, 2, 3}};
  return tab[k][rel];
}
// Vertex opposite to face `k` (grid/gmsh_reader.cpp:59-80).
inline int off_vertex(int n_dims, int k) {
  if (n_dims == 2) return (k + 2) % 3;
  static const int tab[4] = {2, 3, 1, 0};
  return tab[k];
}

}  // namespace zfvm
