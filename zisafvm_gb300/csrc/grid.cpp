// Set-up-time geometry: quadrature rules and the Grid restatement.
// Follows grid/grid.cpp:103-723,1049-1137, math/triangle.cpp, math/tetrahedron.cpp,
// math/face_factory.cpp and math/cell.cpp of ZisaFVM.
#include "grid.hpp"

#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif
#include <map>

namespace zfvm {

// ---------------------------------------------------------------- quadrature
RefRule edge_rule(int deg) {
  if (deg < 0) deg = 7;
  int n = deg / 2 + 1;
  RefRule r;
  std::vector<double> x, w;
  if (n == 1) {
    x = {0.0};
    w = {2.0};
  } else if (n == 2) {
    double a = 1.0 / std::sqrt(3.0);
    x = {-a, a};
    w = {1.0, 1.0};
  } else if (n == 3) {
    double a = std::sqrt(0.6);
    // The reference's middle node is cos(pi/2) (math/gauss_legendre.hpp:93-95).
    x = {-a, std::cos(M_PI / 2), a};
    w = {5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0};
  } else if (n == 4) {
    double s = 2.0 / 7.0 * std::sqrt(6.0 / 5.0);
    double a = std::sqrt(3.0 / 7.0 - s), b = std::sqrt(3.0 / 7.0 + s);
    double wa = (18.0 + std::sqrt(30.0)) / 36.0, wb = (18.0 - std::sqrt(30.0)) / 36.0;
    x = {-b, -a, a, b};
    w = {wb, wa, wa, wb};
  } else {
    throw SetupError(1, "edge rule degree not implemented");
  }
  for (int i = 0; i < n; ++i) {
    r.w.push_back(0.5 * w[i]);
    r.bary.push_back({x[i], 0.0, 0.0, 0.0});
  }
  return r;
}

static void permute2(RefRule &r, double w, double a, double b) {
  r.w.insert(r.w.end(), {w, w, w});
  r.bary.push_back({a, b, b, 0.0});
  r.bary.push_back({b, a, b, 0.0});
  r.bary.push_back({b, b, a, 0.0});
}

RefRule triangle_rule(int deg) {
  if (deg < 0) deg = kMaxTriangleRuleDegree;
  RefRule r;
  if (deg == 1) {
    r.w = {1.0};
    r.bary = {{1.0 / 3.0, 1.0 / 3.0, 1.0 / 3.0, 0.0}};
  } else if (deg == 2) {
    permute2(r, 1.0 / 3.0, 2.0 / 3.0, 1.0 / 6.0);
  } else if (deg == 3) {
    r.w = {-0.5625};
    r.bary = {{1.0 / 3.0, 1.0 / 3.0, 1.0 / 3.0, 0.0}};
    permute2(r, 1.5625 / 3.0, 0.6, 0.2);
  } else if (deg == 4) {
    permute2(r, 0.109951743655322, 0.816847572980459, 0.091576213509771);
    permute2(r, 0.223381589678011, 0.108103018168070, 0.445948490915965);
  } else if (deg == 5) {
    r.w = {0.225};
    r.bary = {{1.0 / 3.0, 1.0 / 3.0, 1.0 / 3.0, 0.0}};
    permute2(r, 0.132394152788506, 0.059715871789770, 0.470142064105115);
    permute2(r, 0.125939180544827, 0.797426985353087, 0.101286507323456);
  } else {
    throw SetupError(1, "triangle rule degree not implemented");
  }
  return r;
}

RefRule tetra_rule(int deg) {
  if (deg < 0) deg = kMaxTetraRuleDegree;
  RefRule r;
  if (deg <= 1) {
    r.w = {1.0};
    r.bary = {{0.25, 0.25, 0.25, 0.25}};
  } else if (deg == 2) {
    const double a = 0.5854101966249680, b = 0.1381966011250110;
    r.w = {0.25, 0.25, 0.25, 0.25};
    r.bary = {{a, b, b, b}, {b, a, b, b}, {b, b, a, b}, {b, b, b, a}};
  } else if (deg == 3) {
    const double a = 0.7784952948213300, b = 0.0738349017262234;
    const double c = 0.4062443438840510, d = 0.0937556561159491;
    const double wa = 0.0476331348432089, wc = 0.1349112434378610;
    r.w = {wa, wa, wa, wa, wc, wc, wc, wc, wc, wc};
    r.bary = {{a, b, b, b}, {b, a, b, b}, {b, b, a, b}, {b, b, b, a}, {c, c, d, d},
              {c, d, c, d}, {c, d, d, c}, {d, c, c, d}, {d, c, d, c}, {d, d, c, c}};
  } else {
    throw SetupError(1, "tetrahedron rule degree not implemented");
  }
  return r;
}

// ------------------------------------------------------------------ elements
static double herons_formula(double a, double b, double c) {
  return 0.25 * std::sqrt((a + b + c) * (-a + b + c) * (a - b + c) * (a + b - c));
}

static double triangle_area(const Vec3 &A, const Vec3 &B, const Vec3 &C) {
  return herons_formula(norm(B - C), norm(A - C), norm(A - B));
}

static double tetra_volume(const Vec3 &v0, const Vec3 &v1, const Vec3 &v2, const Vec3 &v3) {
  Vec3 d1 = v1 - v0, d2 = v2 - v0, d3 = v3 - v0;
  double vol = 1.0 / 6.0 *
               (d1.x * d2.y * d3.z + d2.x * d3.y * d1.z + d3.x * d1.y * d2.z - d1.x * d3.y * d2.z -
                d2.x * d1.y * d3.z - d3.x * d2.y * d1.z);
  return std::fabs(vol);
}

// Quadrature points / weights of `rule` on the simplex with vertices `v`.
static void denormalize(const RefRule &rule, const Vec3 *v, int n_vertices, double vol,
                        double *w_out, Vec3 *x_out) {
  for (size_t q = 0; q < rule.w.size(); ++q) {
    w_out[q] = vol * rule.w[q];
    if (n_vertices == 2) {
      double xr = rule.bary[q][0];
      x_out[q] = (0.5 - 0.5 * xr) * v[0] + (0.5 + 0.5 * xr) * v[1];
    } else {
      Vec3 x = rule.bary[q][0] * v[0];
      for (int k = 1; k < n_vertices; ++k) x = x + rule.bary[q][k] * v[k];
      x_out[q] = x;
    }
  }
}

// average over a denormalised rule: (sum_i w_i f_i) / vol, summed from i = 0
// (math/quadrature.hpp:33-62).
template <class F>
static auto qr_average(const double *w, const Vec3 *x, int n, double vol, const F &f) {
  auto ret = w[0] * f(x[0]);
  for (int i = 1; i < n; ++i) ret = ret + w[i] * f(x[i]);
  return ret / vol;
}

static Vec3 qr_barycenter(const double *w, const Vec3 *x, int n, double vol) {
  Vec3 r = w[0] * x[0];
  for (int i = 1; i < n; ++i) r = r + w[i] * x[i];
  return r / vol;
}

// ---------------------------------------------------------------- build_grid
Grid build_grid(int n_dims, std::vector<Vec3> vertices, std::vector<index_t> vi,
                const QuadDegrees &deg) {
  Grid g;
  g.n_dims = n_dims;
  g.max_nb = n_dims + 1;
  const int nb = g.max_nb;
  g.n_cells = (index_t)vi.size() / nb;
  g.n_vertices = (index_t)vertices.size();
  g.vertices = std::move(vertices);
  g.vertex_indices = std::move(vi);
  const index_t n = g.n_cells;
  auto V = [&](index_t i, int k) -> const Vec3 & { return g.vertices[g.vertex_indices[i * nb + k]]; };

  // standard vertex order
#pragma omp parallel for schedule(static)
  for (index_t i = 0; i < n; ++i) {
    if (n_dims == 2) {
      Vec3 c = cross(V(i, 1) - V(i, 0), V(i, 2) - V(i, 0));
      if (c.z < 0.0) std::swap(g.vertex_indices[i * nb + 1], g.vertex_indices[i * nb + 2]);
    } else {
      Vec3 cc = 0.25 * (V(i, 0) + V(i, 1) + V(i, 2) + V(i, 3));
      for (int k = 0; k < 4; ++k) {
        const Vec3 &a = V(i, face_vertex(3, k, 0)), &b = V(i, face_vertex(3, k, 1)),
                   &c = V(i, face_vertex(3, k, 2));
        Vec3 nn = cross(b - a, c - a);
        Vec3 fc = 1.0 / 3.0 * (a + b + c);
        if (dot(nn, fc - cc) < 0.0) {
          std::swap(g.vertex_indices[i * nb + 2], g.vertex_indices[i * nb + 3]);
          break;
        }
      }
    }
  }

  // neighbours across each face: every (cell, local face) is keyed by the
  // face's sorted vertex ids; a face meets the earlier unmatched entry with
  // the same vertices, if there is one, else waits for a later one (so with
  // more than two equal faces, consecutive ones pair up in cell order).  The
  // entries are split by hash into buckets, each matched on its own in cell
  // order by an open-addressing table with tombstones for consumed entries;
  // equal faces share a bucket, so the pairing is the serial one.
  g.neighbours.assign(n * nb, -1);
  {
    const int fv = n_dims;  // vertices per face
    auto sorted_face = [&](index_t i, int k, index_t *a) {
      for (int r = 0; r < fv; ++r) a[r] = g.vertex_indices[i * nb + face_vertex(n_dims, k, r)];
      if (a[0] > a[1]) std::swap(a[0], a[1]);
      if (fv == 3) {
        if (a[1] > a[2]) std::swap(a[1], a[2]);
        if (a[0] > a[1]) std::swap(a[0], a[1]);
      }
    };
    const index_t total = n * nb;
    std::vector<uint64_t> hv(total);
#pragma omp parallel for schedule(static)
    for (index_t i = 0; i < n; ++i)
      for (int k = 0; k < nb; ++k) {
        index_t a[3] = {0, 0, 0};
        sorted_face(i, k, a);
        uint64_t h = 1469598103934665603ull;
        for (int r = 0; r < fv; ++r) h = (h ^ (uint64_t)a[r]) * 1099511628211ull;
        hv[i * nb + k] = h;
      }
    constexpr int kBucketBits = 10, kBuckets = 1 << kBucketBits;
    auto bucket_of = [](uint64_t h) { return (int)((h * 0x9E3779B97F4A7C15ull) >> (64 - kBucketBits)); };
    // stable counting sort of the entries by bucket
    std::vector<index_t> order(total), start(kBuckets + 1, 0);
    int max_threads = 1;
#ifdef _OPENMP
    max_threads = omp_get_max_threads();
#endif
    std::vector<index_t> cnt((size_t)max_threads * kBuckets, 0);
#pragma omp parallel
    {
      int t = 0, T = 1;
#ifdef _OPENMP
      t = omp_get_thread_num(), T = omp_get_num_threads();
#endif
      const index_t lo = total * t / T, hi = total * (t + 1) / T;
      index_t *c = &cnt[(size_t)t * kBuckets];
      for (index_t e = lo; e < hi; ++e) ++c[bucket_of(hv[e])];
#pragma omp barrier
#pragma omp single
      {
        index_t off = 0;
        for (int b = 0; b < kBuckets; ++b) {
          start[b] = off;
          for (int u = 0; u < T; ++u) {
            const index_t m = cnt[(size_t)u * kBuckets + b];
            cnt[(size_t)u * kBuckets + b] = off;
            off += m;
          }
        }
        start[kBuckets] = off;
      }
      for (index_t e = lo; e < hi; ++e) order[c[bucket_of(hv[e])]++] = e;
    }
    constexpr int64_t kEmpty = -1, kConsumed = -2;
#pragma omp parallel
    {
      std::vector<int64_t> table;  // entry i * nb + k of a face still waiting for its partner
#pragma omp for schedule(dynamic, 8)
      for (int bk = 0; bk < kBuckets; ++bk) {
        size_t cap = 16;
        while (cap < 2 * (size_t)(start[bk + 1] - start[bk])) cap <<= 1;
        const size_t mask = cap - 1;
        table.assign(cap, kEmpty);
        for (index_t o = start[bk]; o < start[bk + 1]; ++o) {
          const index_t ent = order[o];
          const index_t i = ent / nb;
          const int k = (int)(ent % nb);
          index_t a[3] = {0, 0, 0};
          sorted_face(i, k, a);
          const uint64_t h = hv[ent];
          for (size_t s = (size_t)(h ^ (h >> 29)) & mask;; s = (s + 1) & mask) {
            const int64_t e = table[s];
            if (e == kEmpty) {
              table[s] = ent;
              break;
            }
            if (e == kConsumed || hv[e] != h) continue;
            index_t b[3] = {0, 0, 0};
            const index_t j = e / nb;
            const int l = (int)(e % nb);
            sorted_face(j, l, b);
            bool same = true;
            for (int r = 0; r < fv; ++r) same = same && a[r] == b[r];
            if (same) {
              g.neighbours[i * nb + k] = j;
              g.neighbours[j * nb + l] = i;
              table[s] = kConsumed;
              break;
            }
          }
        }
      }
    }
  }

  // interior-first edge numbering (grid/grid.cpp:385-413): interior faces in
  // the order of their lower cell, then boundary faces in cell order; the
  // numbers come from per-cell prefix counts, so every cell is numbered on
  // its own
  {
    std::vector<index_t> int_off(n + 1, 0), ext_off(n + 1, 0);
#pragma omp parallel for schedule(static)
    for (index_t i = 0; i < n; ++i) {
      index_t ni = 0, ne = 0;
      for (int k = 0; k < nb; ++k) {
        const index_t j = g.neighbours[i * nb + k];
        ni += (j >= 0 && i < j);
        ne += (j < 0);
      }
      int_off[i + 1] = ni;
      ext_off[i + 1] = ne;
    }
    for (index_t i = 0; i < n; ++i) int_off[i + 1] += int_off[i], ext_off[i + 1] += ext_off[i];
    const index_t n_int = int_off[n];
    g.n_interior_edges = n_int;
    g.n_edges = n_int + ext_off[n];
    g.edge_indices.assign(n * nb, -1);
    g.left.assign(g.n_edges, -1);
    g.right.assign(g.n_edges, -1);
#pragma omp parallel for schedule(static)
    for (index_t i = 0; i < n; ++i) {
      index_t next_int = int_off[i], next_ext = n_int + ext_off[i];
      for (int k = 0; k < nb; ++k) {
        const index_t j = g.neighbours[i * nb + k];
        if (j < 0) {
          g.edge_indices[i * nb + k] = next_ext;
          g.left[next_ext++] = i;
        } else if (i < j) {
          g.edge_indices[i * nb + k] = next_int;
          g.left[next_int] = i;
          g.right[next_int++] = j;
        }
      }
    }
    int bad = 0;
#pragma omp parallel for schedule(static) reduction(| : bad)
    for (index_t i = 0; i < n; ++i)
      for (int k = 0; k < nb; ++k) {
        const index_t j = g.neighbours[i * nb + k];
        if (j < 0 || i < j) continue;
        int kj = -1;
        for (int l = 0; l < nb; ++l)
          if (g.neighbours[j * nb + l] == i) kj = l;
        if (kj < 0 || g.edge_indices[j * nb + kj] < 0) {
          bad = 1;
          continue;
        }
        g.edge_indices[i * nb + k] = g.edge_indices[j * nb + kj];
      }
    if (bad) throw SetupError(1, "inconsistent neighbours");
  }

  // cell measures
  g.volumes.resize(n);
  g.inradii.resize(n);
  g.circum_radii.resize(n);
  g.char_length.resize(n);
#pragma omp parallel for schedule(static)
  for (index_t i = 0; i < n; ++i) {
    if (n_dims == 2) {
      const Vec3 &A = V(i, 0), &B = V(i, 1), &C = V(i, 2);
      double a = norm(B - C), b = norm(A - C), c = norm(A - B);
      g.volumes[i] = herons_formula(a, b, c);
      g.inradii[i] = 0.5 * std::sqrt((b + c - a) * (c + a - b) * (a + b - c) / (a + b + c));
      Vec3 bc = (A + B + C) / 3.0;
      g.circum_radii[i] = std::max(norm(A - bc), std::max(norm(B - bc), norm(C - bc)));
      g.char_length[i] = g.circum_radii[i];
    } else {
      Vec3 v[4] = {V(i, 0), V(i, 1), V(i, 2), V(i, 3)};
      g.volumes[i] = tetra_volume(v[0], v[1], v[2], v[3]);
      Vec3 c = 0.25 * (v[0] + v[1] + v[2] + v[3]);
      double r_in = 1e300, r_out = 0.0, l = 0.0;
      for (int k = 0; k < 4; ++k) {
        Vec3 fa = v[face_vertex(3, k, 0)], fb = v[face_vertex(3, k, 1)], fc = v[face_vertex(3, k, 2)];
        r_in = std::min(r_in, norm((fa + fb + fc) / 3.0 - c));
        r_out = std::max(r_out, norm(v[k] - c));
        l += 2.0 * norm(c - v[k]);
      }
      g.inradii[i] = r_in;
      g.circum_radii[i] = r_out;
      g.char_length[i] = 0.25 * l;
    }
  }

  // cell quadrature and centres
  RefRule crule = n_dims == 2 ? triangle_rule(deg.volume) : tetra_rule(deg.volume);
  g.n_cell_qp = (int)crule.w.size();
  g.cell_qw.resize(n * g.n_cell_qp);
  g.cell_qx.resize(n * g.n_cell_qp);
  g.cell_centers.resize(n);
#pragma omp parallel for schedule(static)
  for (index_t i = 0; i < n; ++i) {
    Vec3 v[4];
    for (int k = 0; k < nb; ++k) v[k] = V(i, k);
    double *w = &g.cell_qw[i * g.n_cell_qp];
    Vec3 *x = &g.cell_qx[i * g.n_cell_qp];
    denormalize(crule, v, nb, g.volumes[i], w, x);
    g.cell_centers[i] = qr_barycenter(w, x, g.n_cell_qp, g.volumes[i]);
  }

  // faces (grid/grid.cpp:587-612, math/face_factory.cpp)
  RefRule frule = n_dims == 2 ? edge_rule(deg.edge) : triangle_rule(deg.edge);
  g.n_face_qp = (int)frule.w.size();
  g.face_qw.resize(g.n_edges * g.n_face_qp);
  g.face_qx.resize(g.n_edges * g.n_face_qp);
  g.face_area.resize(g.n_edges);
  g.face_normal.resize(g.n_edges);
  g.face_t1.resize(g.n_edges);
  g.face_t2.resize(g.n_edges);
  // every face is set up once, by its lower-numbered cell
#pragma omp parallel for schedule(static)
  for (index_t i = 0; i < n; ++i)
    for (int k = 0; k < nb; ++k) {
      index_t j = g.neighbours[i * nb + k];
      if (j >= 0 && j < i) continue;
      index_t e = g.edge_indices[i * nb + k];
      Vec3 fv[3];
      for (int r = 0; r < n_dims; ++r) fv[r] = V(i, face_vertex(n_dims, k, r));
      double area;
      Vec3 nn, t1;
      if (n_dims == 2) {
        area = norm(fv[1] - fv[0]);
        nn = rotate_right(normalize(fv[1] - fv[0]));
        t1 = normalize(fv[1] - fv[0]);
      } else {
        area = triangle_area(fv[0], fv[1], fv[2]);
        nn = normalize(cross(fv[1] - fv[0], fv[2] - fv[0]));
        t1 = normalize(fv[1] - fv[0]);
      }
      g.face_area[e] = area;
      g.face_normal[e] = nn;
      g.face_t1[e] = t1;
      g.face_t2[e] = cross(nn, t1);
      denormalize(frule, fv, n_dims, area, &g.face_qw[e * g.n_face_qp], &g.face_qx[e * g.n_face_qp]);
    }

  // normalized moments (grid/grid.cpp:1049-1098)
  int mdeg = deg.moments;
  if (mdeg < 0) mdeg = n_dims == 2 ? kMaxTriangleRuleDegree : kMaxTetraRuleDegree;
  RefRule mrule = n_dims == 2 ? triangle_rule(mdeg) : tetra_rule(mdeg);
  const int nmq = (int)mrule.w.size();
  g.n_moments = poly_dof(mdeg, n_dims);
  g.moments.assign(n * g.n_moments, 0.0);
#pragma omp parallel
  {
  std::vector<double> mw(nmq);
  std::vector<Vec3> mx(nmq);
#pragma omp for schedule(static)
  for (index_t i = 0; i < n; ++i) {
    Vec3 v[4];
    for (int k = 0; k < nb; ++k) v[k] = V(i, k);
    denormalize(mrule, v, nb, g.volumes[i], mw.data(), mx.data());
    Vec3 c = qr_barycenter(mw.data(), mx.data(), nmq, g.volumes[i]);
    double len = g.char_length[i];
    double len_d = 1.0;
    for (int d = 0; d <= mdeg; ++d) {
      for (int a = 0; a <= d; ++a) {
        if (n_dims == 2) {
          int b = d - a;
          auto f = [&](const Vec3 &x) {
            Vec3 r = x - c;
            return std::pow(r.x, (double)a) * std::pow(r.y, (double)b) * std::pow(r.z, 0.0);
          };
          g.moments[i * g.n_moments + poly_index2(a, b)] =
              qr_average(mw.data(), mx.data(), nmq, g.volumes[i], f) / len_d;
        } else {
          for (int b = 0; b <= d - a; ++b) {
            int cc = d - a - b;
            auto f = [&](const Vec3 &x) {
              Vec3 r = x - c;
              return std::pow(r.x, (double)a) * std::pow(r.y, (double)b) * std::pow(r.z, (double)cc);
            };
            g.moments[i * g.n_moments + poly_index3(a, b, cc)] =
                qr_average(mw.data(), mx.data(), nmq, g.volumes[i], f) / len_d;
          }
        }
      }
      len_d *= len;
    }
  }
  }

  g.flags.assign(n, kInterior);
  g.source.resize(n);
  for (index_t i = 0; i < n; ++i) g.source[i] = i;
  return g;
}

void mask_ghost_cells(Grid &g, const std::vector<uint8_t> &is_ghost) {
  if (is_ghost.empty()) return;
  for (index_t i = 0; i < g.n_cells; ++i) {
    if (!is_ghost[i]) continue;
    uint8_t f = kGhost;
    for (int k = 0; k < g.max_nb; ++k) {
      index_t j = g.neighbours[i * g.max_nb + k];
      if (j >= 0 && !is_ghost[j]) f |= kGhostL1;
    }
    g.flags[i] = f;
  }
}

}  // namespace zfvm
