// Stencil selection and least-squares operators, computed once per mesh.
// Follows reconstruction/stencil.cpp:159-399, stencil_family.cpp:15-136 and
// lsq_solver.cpp:139-403 of ZisaFVM.
#include <algorithm>
#include <cfloat>
#include <cstdint>
#include <numeric>
#include <random>
#include <utility>
#include <vector>

#include "grid.hpp"

namespace zfvm {

int_fast32_t required_stencil_size(int deg, double factor, int n_dims) {
  if (deg == 0) return 1;
  return (int_fast32_t)(double(poly_dof(deg, n_dims) - 1) * factor + 1);
}

int deduce_max_order(index_t stencil_size, double factor, int n_dims) {
  int deg = 0;
  while (required_stencil_size(deg + 1, factor, n_dims) <= stencil_size) deg += 1;
  return deg + 1;
}

// ------------------------------------------------------------------- LSQ
void assemble_weno_ao_matrix(const Grid &g, const int32_t *st, int n_points, int order,
                             std::vector<double> &A, int &rows, int &cols) {
  const int nd = g.n_dims;
  if (order <= 1) {
    rows = cols = 0;
    A.clear();
    return;
  }
  rows = n_points - 1;
  cols = poly_dof(order - 1, nd) - 1;
  A.assign((size_t)rows * cols, 0.0);
  const int nm = g.n_moments;
  index_t i0 = st[0];
  Vec3 x0 = g.cell_centers[i0];
  double l0 = g.char_length[i0];
  const double *C0 = &g.moments[i0 * nm];
  auto at = [&](int r, int c) -> double & { return A[(size_t)r * cols + (c - 1)]; };
  auto idx2 = [&](int a, int b) { return nd == 2 ? poly_index2(a, b) : poly_index3(a, b, 0); };
  for (int r = 0; r < rows; ++r) {
    index_t j = st[r + 1];
    Vec3 d = (g.cell_centers[j] - x0) / l0;
    double lj = g.char_length[j] / l0;
    const double *Cj = &g.moments[j * nm];
    double x = d.x, y = d.y, z = d.z;
    // two-dimensional part (lsq_solver.cpp:232-356)
    at(r, idx2(1, 0)) = x;
    at(r, idx2(0, 1)) = y;
    double lj2 = lj * lj;
    if (order >= 3) {
      int i20 = idx2(2, 0), i11 = idx2(1, 1), i02 = idx2(0, 2);
      at(r, i20) = x * x - C0[i20] + lj2 * Cj[i20];
      at(r, i11) = x * y - C0[i11] + lj2 * Cj[i11];
      at(r, i02) = y * y - C0[i02] + lj2 * Cj[i02];
    }
    if (order >= 4) {
      if (nd == 3) throw SetupError(1, "3D reconstruction above order 3 is not implemented");
      int i20 = idx2(2, 0), i11 = idx2(1, 1), i02 = idx2(0, 2);
      int i30 = idx2(3, 0), i21 = idx2(2, 1), i12 = idx2(1, 2), i03 = idx2(0, 3);
      double x20 = x * x, x11 = x * y, x02 = y * y;
      double x30 = x20 * x, x21 = x20 * y, x12 = x11 * y, x03 = x02 * y;
      double lj3 = lj2 * lj;
      at(r, i30) = x30 - C0[i30] + 3.0 * x * lj2 * Cj[i20] + lj3 * Cj[i30];
      at(r, i21) = x21 - C0[i21] + y * lj2 * Cj[i20] + 2.0 * x * lj2 * Cj[i11] + lj3 * Cj[i21];
      at(r, i12) = x12 - C0[i12] + x * lj2 * Cj[i02] + 2.0 * y * lj2 * Cj[i11] + lj3 * Cj[i12];
      at(r, i03) = x03 - C0[i03] + 3.0 * y * lj2 * Cj[i02] + lj3 * Cj[i03];
      if (order >= 5) throw SetupError(1, "reconstruction above order 4 is not implemented");
    }
    if (nd == 3) {
      // three-dimensional part (lsq_solver.cpp:358-467)
      at(r, poly_index3(0, 0, 1)) = z;
      if (order >= 3) {
        int i002 = poly_index3(0, 0, 2), i101 = poly_index3(1, 0, 1), i011 = poly_index3(0, 1, 1);
        at(r, i002) = z * z - C0[i002] + lj2 * Cj[i002];
        at(r, i101) = x * z - C0[i101] + lj2 * Cj[i101];
        at(r, i011) = y * z - C0[i011] + lj2 * Cj[i011];
      }
    }
  }
}

// One-sided Jacobi SVD; returns the singular values.
static std::vector<double> singular_values(std::vector<double> A, int m, int n) {
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0.0;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) {
        double alpha = 0, beta = 0, gamma = 0;
        for (int i = 0; i < m; ++i) {
          double ap = A[(size_t)i * n + p], aq = A[(size_t)i * n + q];
          alpha += ap * ap;
          beta += aq * aq;
          gamma += ap * aq;
        }
        if (gamma == 0.0) continue;
        off = std::max(off, std::fabs(gamma) / std::sqrt(alpha * beta));
        double zeta = (beta - alpha) / (2.0 * gamma);
        double t = (zeta >= 0 ? 1.0 : -1.0) / (std::fabs(zeta) + std::sqrt(1.0 + zeta * zeta));
        double c = 1.0 / std::sqrt(1.0 + t * t), s = c * t;
        for (int i = 0; i < m; ++i) {
          double ap = A[(size_t)i * n + p], aq = A[(size_t)i * n + q];
          A[(size_t)i * n + p] = c * ap - s * aq;
          A[(size_t)i * n + q] = s * ap + c * aq;
        }
      }
    if (off < 1e-15) break;
  }
  std::vector<double> sv(n);
  for (int j = 0; j < n; ++j) {
    double s = 0;
    for (int i = 0; i < m; ++i) s += A[(size_t)i * n + j] * A[(size_t)i * n + j];
    sv[j] = std::sqrt(s);
  }
  std::sort(sv.begin(), sv.end(), std::greater<double>());
  return sv;
}

int numerical_rank(const std::vector<double> &A, int rows, int cols) {
  if (cols == 0) return 0;
  if (rows < cols) {
    // rank <= rows; pad with zero rows to keep the Jacobi sweep simple
    std::vector<double> B((size_t)cols * cols, 0.0);
    std::copy(A.begin(), A.end(), B.begin());
    auto sv = singular_values(B, cols, cols);
    double thr = std::max(sv[0] * double(std::min(rows, cols)) * DBL_EPSILON, DBL_MIN);
    int r = 0;
    for (double s : sv) r += s > thr;
    return r;
  }
  auto sv = singular_values(A, rows, cols);
  double thr = std::max(sv[0] * double(std::min(rows, cols)) * DBL_EPSILON, DBL_MIN);
  int r = 0;
  for (double s : sv) r += s > thr;
  return r;
}

void pseudo_inverse(const std::vector<double> &A, int m, int n, std::vector<double> &P) {
  // Householder QR: A = Q R;  pinv = R^{-1} Q^T (n x m)
  std::vector<double> R(A);
  std::vector<double> Qt((size_t)m * m, 0.0);
  for (int i = 0; i < m; ++i) Qt[(size_t)i * m + i] = 1.0;
  for (int k = 0; k < n; ++k) {
    double s = 0;
    for (int i = k; i < m; ++i) s += R[(size_t)i * n + k] * R[(size_t)i * n + k];
    double nrm = std::sqrt(s);
    if (nrm == 0.0) continue;
    double akk = R[(size_t)k * n + k];
    double alpha = akk > 0 ? -nrm : nrm;
    std::vector<double> v(m, 0.0);
    v[k] = akk - alpha;
    for (int i = k + 1; i < m; ++i) v[i] = R[(size_t)i * n + k];
    double vv = 0;
    for (int i = k; i < m; ++i) vv += v[i] * v[i];
    if (vv == 0.0) continue;
    for (int j = 0; j < n; ++j) {
      double d = 0;
      for (int i = k; i < m; ++i) d += v[i] * R[(size_t)i * n + j];
      d = 2.0 * d / vv;
      for (int i = k; i < m; ++i) R[(size_t)i * n + j] -= d * v[i];
    }
    for (int j = 0; j < m; ++j) {
      double d = 0;
      for (int i = k; i < m; ++i) d += v[i] * Qt[(size_t)i * m + j];
      d = 2.0 * d / vv;
      for (int i = k; i < m; ++i) Qt[(size_t)i * m + j] -= d * v[i];
    }
  }
  // P = R^{-1} (Q^T)[0:n, :]
  P.assign((size_t)n * m, 0.0);
  for (int col = 0; col < m; ++col) {
    for (int i = n - 1; i >= 0; --i) {
      double s = Qt[(size_t)i * m + col];
      for (int j = i + 1; j < n; ++j) s -= R[(size_t)i * n + j] * P[(size_t)j * m + col];
      P[(size_t)i * m + col] = s / R[(size_t)i * n + i];
    }
  }
}

// -------------------------------------------------------------- selection
namespace {

struct Region {
  int kind = 0;  // 0 = everything, 2 = 2D cone, 3 = 3D cone
  Vec3 A, dB, dC, dD;
  bool inside(const Vec3 &x) const {
    if (kind == 0) return true;
    Vec3 dx = x - A;
    if (kind == 2) return cross(dB, dx).z >= 0.0 && cross(dx, dC).z >= 0.0;
    return det3(dB, dC, dx) >= 0.0 && det3(dC, dD, dx) >= 0.0 && det3(dD, dB, dx) >= 0.0;
  }
};

// Open-addressing set of cell ids for one candidate search (a few hundred
// entries at most).  The table is per thread and reused: a slot belongs to the
// current search when its stamp equals the search's epoch, so a new search
// clears nothing.  It grows by rehashing if a search ever fills half of it.
struct SmallSet {
  struct Table {
    std::vector<index_t> key = std::vector<index_t>(1024, -1);
    std::vector<uint32_t> stamp = std::vector<uint32_t>(1024, 0);
    uint32_t epoch = 0;
  };
  Table &t;
  size_t count = 0;
  static Table &table() {
    static thread_local Table tab;
    return tab;
  }
  SmallSet() : t(table()) {
    if (++t.epoch == 0) {  // stamps wrapped: start over
      std::fill(t.stamp.begin(), t.stamp.end(), 0u);
      t.epoch = 1;
    }
  }
  static size_t hash(index_t c) { return (size_t)((uint64_t)c * 0x9E3779B97F4A7C15ull >> 20); }
  bool contains(index_t c) const {
    const size_t mask = t.key.size() - 1;
    for (size_t h = hash(c) & mask;; h = (h + 1) & mask) {
      if (t.stamp[h] != t.epoch) return false;
      if (t.key[h] == c) return true;
    }
  }
  void insert(index_t c) {
    if (2 * (count + 1) > t.key.size()) grow();
    const size_t mask = t.key.size() - 1;
    size_t h = hash(c) & mask;
    while (t.stamp[h] == t.epoch && t.key[h] != c) h = (h + 1) & mask;
    if (t.stamp[h] != t.epoch) t.stamp[h] = t.epoch, t.key[h] = c, ++count;
  }
  void grow() {
    std::vector<index_t> live;
    for (size_t h = 0; h < t.key.size(); ++h)
      if (t.stamp[h] == t.epoch) live.push_back(t.key[h]);
    t.key.assign(2 * t.key.size(), -1);
    t.stamp.assign(t.key.size(), 0u);
    t.epoch = 1;
    count = 0;
    for (index_t x : live) insert(x);
  }
};

struct Selector {
  const Grid &g;
  RefRule query;  // highest-degree cell rule (stencil.cpp:178-190)
  explicit Selector(const Grid &grid)
      : g(grid), query(grid.n_dims == 2 ? triangle_rule(-1) : tetra_rule(-1)) {}

  // A cell is in the region when any of the query points or its centre is
  // (the centre, one test, is tried first; the answer is the same).
  bool cell_in_region(index_t c, const Region &reg) const {
    if (reg.kind == 0) return true;
    if (reg.inside(g.cell_centers[c])) return true;
    const int nb = g.max_nb;
    Vec3 v[4];
    for (int k = 0; k < nb; ++k) v[k] = g.vertex(c, k);
    for (size_t q = 0; q < query.w.size(); ++q) {
      Vec3 x = query.bary[q][0] * v[0];
      for (int k = 1; k < nb; ++k) x = x + query.bary[q][k] * v[k];
      if (reg.inside(x)) return true;
    }
    return false;
  }

  // Breadth-first candidates in discovery order; `seen` answers "already a
  // candidate?" in O(1) instead of a scan of the list.
  std::vector<index_t> candidates(index_t i, index_t n_points, const Region &reg) const {
    index_t max_points = 5 * n_points;
    std::vector<index_t> cand;
    cand.reserve((size_t)(max_points + 1) * g.max_nb);
    cand.push_back(i);
    SmallSet seen;
    seen.insert(i);
    for (index_t p = 0; p < max_points; ++p) {
      if (p >= (index_t)cand.size()) break;
      index_t j = cand[p];
      for (int k = 0; k < g.max_nb; ++k) {
        index_t c = g.neighbours[j * g.max_nb + k];
        if (c < 0) continue;
        if (!seen.contains(c) && cell_in_region(c, reg)) {
          cand.push_back(c);
          seen.insert(c);
        }
      }
    }
    return cand;
  }

  std::vector<index_t> region_stencil(index_t i, index_t n_points, const Region &reg) const {
    auto cand = candidates(i, n_points, reg);
    const Vec3 xc = g.cell_centers[i];
    // std::sort by distance in the reference; ties broken by candidate order
    // here, so the key is (distance, position in the candidate list), a total
    // order.  The distances are computed once, not in every comparison, and
    // only the nearest n_points are ordered.
    std::vector<std::pair<double, index_t>> key(cand.size());
    for (size_t r = 0; r < cand.size(); ++r) key[r] = {norm(g.cell_centers[cand[r]] - xc), (index_t)r};
    const size_t keep = std::min(cand.size(), (size_t)n_points);
    std::partial_sort(key.begin(), key.begin() + keep, key.end());
    std::vector<index_t> out(keep);
    for (size_t r = 0; r < keep; ++r) out[r] = cand[key[r].second];
    return out;
  }

  Region cone(index_t i, const Vec3 &apex, int k) const {
    Region r;
    r.kind = g.n_dims;
    r.A = apex;
    r.dB = g.vertex(i, face_vertex(g.n_dims, k, 0)) - apex;
    r.dC = g.vertex(i, face_vertex(g.n_dims, k, 1)) - apex;
    if (g.n_dims == 3) r.dD = g.vertex(i, face_vertex(3, k, 2)) - apex;
    return r;
  }

  bool is_good(const std::vector<index_t> &s, index_t n, int order) const {
    std::vector<int32_t> st(s.begin(), s.begin() + n);
    std::vector<double> A;
    int rows, cols;
    assemble_weno_ao_matrix(g, st.data(), (int)n, order, A, rows, cols);
    return numerical_rank(A, rows, cols) == cols;
  }

  std::vector<index_t> biased(index_t i, int k, index_t n_points, int order) const {
    // conservative: apex at the vertex opposite face k
    auto s = region_stencil(i, n_points, cone(i, g.vertex(i, off_vertex(g.n_dims, k)), k));
    if ((index_t)s.size() == n_points && is_good(s, n_points, order)) return s;
    // less conservative: apex at the cell centre
    s = region_stencil(i, n_points, cone(i, g.cell_centers[i], k));
    if ((index_t)s.size() == n_points && is_good(s, n_points, order)) return s;
    // last resort: apex at the face centre, random subsets of the candidates
    index_t e = g.edge_indices[i * g.max_nb + k];
    Vec3 fc = g.face_qw[e * g.n_face_qp] * g.face_qx[e * g.n_face_qp];
    for (int q = 1; q < g.n_face_qp; ++q)
      fc = fc + g.face_qw[e * g.n_face_qp + q] * g.face_qx[e * g.n_face_qp + q];
    fc = fc / g.face_area[e];
    auto cand = candidates(i, n_points, cone(i, fc, k));
    if ((index_t)cand.size() < n_points) return {i};
    if (!is_good(cand, (index_t)cand.size(), order))
      throw SetupError(1, "impossible to find a suitable stencil for cell " + std::to_string(i));
    std::mt19937 rng((uint32_t)(i * 7919 + k * 104729 + 17));
    for (int iter = 0; iter < 100; ++iter) {
      std::shuffle(cand.begin() + 1, cand.end(), rng);
      if (is_good(cand, n_points, order)) {
        cand.resize(n_points);
        return cand;
      }
    }
    throw SetupError(1, "did not find a suitable stencil for cell " + std::to_string(i));
  }
};

}  // namespace

StencilFamilies compute_stencil_families(const Grid &g, const StencilParams &params) {
  const index_t n = g.n_cells;
  StencilFamilies f;
  f.n_cells = n;
  f.n_stencils.assign(n, 0);
  f.k_high.assign(n, 0);
  f.n_l2g.assign(n, 0);
  f.l2g.assign(n * kMaxL2G, -1);
  f.order.assign(n * kMaxStencils, 1);
  f.size.assign(n * kMaxStencils, 1);
  f.bias.assign(n * kMaxStencils, 0);
  f.overfit.assign(n * kMaxStencils, 1.0);
  f.local.assign(n * kMaxStencils * kMaxStencilSize, 0);
  if ((int)params.orders.size() > kMaxStencils) throw SetupError(1, "too many stencils");
  Selector sel(g);
  std::vector<SetupError> errors;

#pragma omp parallel for schedule(dynamic, 64)
  for (index_t i = 0; i < n; ++i) {
    try {
      bool full = (g.flags[i] & kInterior) || (g.flags[i] & kGhostL1);
      StencilParams p = full ? params : StencilParams{{1}, {0}, {1.0}};
      std::vector<index_t> l2g;
      int ns = (int)p.orders.size();
      int k_biased = 0;
      for (int s = 0; s < ns; ++s) {
        double fac = p.overfit[s];
        int max_order = p.orders[s];
        index_t max_size = required_stencil_size(max_order - 1, fac, g.n_dims);
        std::vector<index_t> glob =
            p.biased[s] ? sel.biased(i, k_biased++, max_size, max_order) : sel.region_stencil(i, max_size, Region{});
        if ((int)glob.size() > kMaxStencilSize) throw SetupError(1, "stencil too large");
        for (size_t r = 0; r < glob.size(); ++r) {
          auto it = std::find(l2g.begin(), l2g.end(), glob[r]);
          f.local[(i * kMaxStencils + s) * kMaxStencilSize + r] = (int8_t)(it - l2g.begin());
          if (it == l2g.end()) l2g.push_back(glob[r]);
        }
        int ord = deduce_max_order((index_t)glob.size(), fac, g.n_dims);
        f.order[i * kMaxStencils + s] = (int8_t)ord;
        f.size[i * kMaxStencils + s] = (int8_t)required_stencil_size(ord - 1, fac, g.n_dims);
        f.bias[i * kMaxStencils + s] = (int8_t)p.biased[s];
        f.overfit[i * kMaxStencils + s] = fac;
      }
      if ((int)l2g.size() > kMaxL2G) throw SetupError(1, "combined stencil too large");
      f.n_stencils[i] = (int8_t)ns;
      f.n_l2g[i] = (int8_t)l2g.size();
      for (size_t l = 0; l < l2g.size(); ++l) f.l2g[i * kMaxL2G + l] = (int32_t)l2g[l];
      // highest-order stencil, central preferred on ties (stencil_family.cpp:120-136)
      int kh = 0;
      for (int s = 1; s < ns; ++s) {
        int ko = f.order[i * kMaxStencils + kh], so = f.order[i * kMaxStencils + s];
        if (so > ko || (so == ko && !f.bias[i * kMaxStencils + s])) kh = s;
      }
      f.k_high[i] = (int8_t)kh;
    } catch (const SetupError &e) {
#pragma omp critical
      errors.push_back(e);
    }
  }
  if (!errors.empty()) throw errors.front();
  return f;
}

}  // namespace zfvm
