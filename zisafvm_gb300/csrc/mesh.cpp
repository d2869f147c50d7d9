// Synthetic mesh generators and space-filling-curve renumbering.
//
// The reference reads gmsh meshes (grid/grid.cpp:889-922) and renumbers them
// with src/renumber_grid.cpp; these generators produce meshes in the same
// vertices / vertex_indices form so every downstream step is unchanged.
#include <algorithm>
#include <cmath>
#include <numeric>
#include <random>
#include <unordered_map>

#include "grid.hpp"

namespace zfvm {

// Portable uniform double in [0, 1) from a 64-bit engine.
static double uniform01(std::mt19937_64 &rng) { return double(rng() >> 11) * 0x1.0p-53; }

RawMesh periodic_square_mesh(int n, int halo, double jitter, uint64_t seed) {
  if (n < 2 || halo < 0) throw SetupError(1, "invalid square mesh size");
  RawMesh m;
  m.n_dims = 2;
  const double h = 1.0 / n;
  std::mt19937_64 rng(seed);
  std::vector<double> jx((size_t)n * n), jy((size_t)n * n);
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      jx[(size_t)j * n + i] = (2.0 * uniform01(rng) - 1.0) * jitter * h;
      jy[(size_t)j * n + i] = (2.0 * uniform01(rng) - 1.0) * jitter * h;
    }
  const int nv = n + 2 * halo + 1;
  auto wrap = [n](int a) { return ((a % n) + n) % n; };
  m.vertices.resize((size_t)nv * nv);
  for (int J = -halo; J <= n + halo; ++J)
    for (int I = -halo; I <= n + halo; ++I) {
      size_t id = (size_t)(J + halo) * nv + (I + halo);
      size_t jj = (size_t)wrap(J) * n + wrap(I);
      m.vertices[id] = {double(I) / double(n) + jx[jj], double(J) / double(n) + jy[jj], 0.0};
    }
  const int nc = n + 2 * halo;
  auto vid = [&](int I, int J) { return (index_t)(J + halo) * nv + (I + halo); };
  auto cid = [&](int I, int J, int t) { return ((index_t)(J + halo) * nc + (I + halo)) * 2 + t; };
  m.vertex_indices.resize((size_t)nc * nc * 2 * 3);
  m.ghost.resize((size_t)nc * nc * 2);
  m.source.resize((size_t)nc * nc * 2);
  for (int J = -halo; J < n + halo; ++J)
    for (int I = -halo; I < n + halo; ++I) {
      index_t v00 = vid(I, J), v10 = vid(I + 1, J), v11 = vid(I + 1, J + 1), v01 = vid(I, J + 1);
      index_t c0 = cid(I, J, 0), c1 = cid(I, J, 1);
      index_t *a = &m.vertex_indices[c0 * 3];
      a[0] = v00, a[1] = v10, a[2] = v11;
      index_t *b = &m.vertex_indices[c1 * 3];
      b[0] = v00, b[1] = v11, b[2] = v01;
      bool ghost = I < 0 || J < 0 || I >= n || J >= n;
      m.ghost[c0] = m.ghost[c1] = ghost;
      m.source[c0] = cid(wrap(I), wrap(J), 0);
      m.source[c1] = cid(wrap(I), wrap(J), 1);
    }
  return m;
}

// ---------------------------------------------------------------- disk mesh
namespace {
struct Tri {
  index_t v[3];
};

double orient(const Vec3 &a, const Vec3 &b, const Vec3 &c) {
  return (b.x - a.x) * (c.y - a.y) - (b.y - a.y) * (c.x - a.x);
}

// > 0 if d lies inside the circumcircle of the counter-clockwise triangle abc.
double incircle(const Vec3 &a, const Vec3 &b, const Vec3 &c, const Vec3 &d) {
  double adx = a.x - d.x, ady = a.y - d.y, bdx = b.x - d.x, bdy = b.y - d.y, cdx = c.x - d.x,
         cdy = c.y - d.y;
  double ad = adx * adx + ady * ady, bd = bdx * bdx + bdy * bdy, cd = cdx * cdx + cdy * cdy;
  return adx * (bdy * cd - bd * cdy) - ady * (bdx * cd - bd * cdx) + ad * (bdx * cdy - bdy * cdx);
}
}  // namespace

RawMesh disk_mesh(int K, double R, double jitter, uint64_t seed) {
  if (K < 2) throw SetupError(1, "invalid disk mesh size");
  RawMesh m;
  m.n_dims = 2;
  const double h = R / K;
  std::vector<int> start(K + 2), count(K + 1);
  m.vertices.push_back({0.0, 0.0, 0.0});
  count[0] = 1;
  start[0] = 0;
  for (int k = 1; k <= K; ++k) {
    int nk = std::max(6, (int)std::lround(2.0 * M_PI * k));
    start[k] = (int)m.vertices.size();
    count[k] = nk;
    double off = (k % 2) ? 0.0 : 0.5;
    for (int j = 0; j < nk; ++j) {
      double th = 2.0 * M_PI * (j + off) / nk;
      m.vertices.push_back({k * h * std::cos(th), k * h * std::sin(th), 0.0});
    }
  }
  std::vector<Tri> tris;
  // centre fan
  for (int j = 0; j < count[1]; ++j)
    tris.push_back({{0, start[1] + j, start[1] + (j + 1) % count[1]}});
  // annuli, zipped by angle
  for (int k = 1; k < K; ++k) {
    int na = count[k], nb = count[k + 1];
    auto ang = [&](int ring, int j) {
      const Vec3 &p = m.vertices[start[ring] + (j % count[ring])];
      double a = std::atan2(p.y, p.x);
      if (a < 0) a += 2 * M_PI;
      return a + 2 * M_PI * (j / count[ring]);
    };
    // begin both walks at the point with the smallest angle
    int a = 0, b = 0;
    while (a < na || b < nb) {
      index_t A0 = start[k] + a % na, A1 = start[k] + (a + 1) % na;
      index_t B0 = start[k + 1] + b % nb, B1 = start[k + 1] + (b + 1) % nb;
      bool advance_b;
      if (a >= na)
        advance_b = true;
      else if (b >= nb)
        advance_b = false;
      else
        advance_b = ang(k + 1, b + 1) < ang(k, a + 1);
      if (advance_b) {
        tris.push_back({{A0, B0, B1}});
        ++b;
      } else {
        tris.push_back({{A0, B0, A1}});
        ++a;
      }
    }
  }
  // jitter the interior points (the centre and rings 1..K-1)
  std::mt19937_64 rng(seed);
  for (int k = 0; k < K; ++k)
    for (int j = 0; j < count[k]; ++j) {
      Vec3 &p = m.vertices[start[k] + j];
      p.x += (2.0 * uniform01(rng) - 1.0) * jitter * h;
      p.y += (2.0 * uniform01(rng) - 1.0) * jitter * h;
    }
  for (auto &t : tris)
    if (orient(m.vertices[t.v[0]], m.vertices[t.v[1]], m.vertices[t.v[2]]) < 0) std::swap(t.v[1], t.v[2]);

  // Lawson flips until Delaunay
  const index_t nt = (index_t)tris.size();
  for (int pass = 0; pass < 200; ++pass) {
    std::unordered_map<uint64_t, std::pair<index_t, int>> edges;
    edges.reserve(nt * 3);
    auto ekey = [](index_t a, index_t b) {
      if (a > b) std::swap(a, b);
      return (uint64_t)a << 32 | (uint64_t)b;
    };
    index_t flips = 0;
    std::vector<char> touched(nt, 0);
    for (index_t t = 0; t < nt; ++t)
      for (int e = 0; e < 3; ++e) {
        index_t a = tris[t].v[e], b = tris[t].v[(e + 1) % 3];
        auto key = ekey(a, b);
        auto it = edges.find(key);
        if (it == edges.end()) {
          edges[key] = {t, e};
          continue;
        }
        index_t u = it->second.first;
        edges.erase(it);
        if (touched[t] || touched[u]) continue;
        index_t c = tris[t].v[(e + 2) % 3];
        index_t d = -1;
        for (int f = 0; f < 3; ++f) {
          index_t x = tris[u].v[f];
          if (x != a && x != b) d = x;
        }
        const Vec3 &A = m.vertices[a], &B = m.vertices[b], &C = m.vertices[c], &D = m.vertices[d];
        double scale = h * h * h * h;
        if (incircle(A, B, C, D) > 1e-12 * scale) {
          // triangle t = (a, b, c) ccw, u contains (b, a, d): flip edge ab -> cd
          // only a convex quadrilateral a-d-b-c can be flipped
          if (orient(C, A, D) <= 0 || orient(D, B, C) <= 0) continue;
          tris[t] = {{c, a, d}};
          tris[u] = {{d, b, c}};
          touched[t] = touched[u] = 1;
          ++flips;
        }
      }
    if (flips == 0) break;
  }
  m.vertex_indices.resize(nt * 3);
  for (index_t t = 0; t < nt; ++t)
    for (int e = 0; e < 3; ++e) m.vertex_indices[t * 3 + e] = tris[t].v[e];
  return m;
}

// ------------------------------------------------------------- cube tets
RawMesh cube_tet_mesh(int n, double jitter, uint64_t seed) {
  if (n < 1) throw SetupError(1, "invalid cube mesh size");
  RawMesh m;
  m.n_dims = 3;
  const double h = 1.0 / n;
  const int nv = n + 1;
  std::mt19937_64 rng(seed);
  m.vertices.resize((size_t)nv * nv * nv);
  for (int k = 0; k <= n; ++k)
    for (int j = 0; j <= n; ++j)
      for (int i = 0; i <= n; ++i) {
        Vec3 p{double(i) / n, double(j) / n, double(k) / n};
        bool interior = i > 0 && j > 0 && k > 0 && i < n && j < n && k < n;
        double dx = (2.0 * uniform01(rng) - 1.0) * jitter * h;
        double dy = (2.0 * uniform01(rng) - 1.0) * jitter * h;
        double dz = (2.0 * uniform01(rng) - 1.0) * jitter * h;
        if (interior) p = {p.x + dx, p.y + dy, p.z + dz};
        m.vertices[((size_t)k * nv + j) * nv + i] = p;
      }
  // Kuhn split: one tetrahedron per permutation of the axes
  static const int perms[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
  m.vertex_indices.reserve((size_t)n * n * n * 24);
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i)
        for (auto &p : perms) {
          int c[3] = {i, j, k};
          auto id = [&]() { return (index_t)(((size_t)c[2] * nv + c[1]) * nv + c[0]); };
          m.vertex_indices.push_back(id());
          for (int s = 0; s < 3; ++s) {
            c[p[s]] += 1;
            m.vertex_indices.push_back(id());
          }
        }
  return m;
}

// ---------------------------------------------------------------- Hilbert
uint64_t hilbert_key_2d(double xf, double yf, int bits) {
  const uint64_t side = 1ull << bits;
  uint64_t x = (uint64_t)std::min(std::max(xf, 0.0) * double(side), double(side - 1));
  uint64_t y = (uint64_t)std::min(std::max(yf, 0.0) * double(side), double(side - 1));
  uint64_t d = 0;
  for (uint64_t s = side >> 1; s > 0; s >>= 1) {
    uint64_t rx = (x & s) ? 1 : 0, ry = (y & s) ? 1 : 0;
    d += s * s * ((3 * rx) ^ ry);
    if (ry == 0) {
      if (rx == 1) {
        x = side - 1 - x;
        y = side - 1 - y;
      }
      std::swap(x, y);
    }
  }
  return d;
}

// Skilling's transpose form of the Hilbert index (AIP Conf. Proc. 707, 2004).
uint64_t hilbert_key_3d(double xf, double yf, double zf, int bits) {
  const uint64_t side = 1ull << bits;
  uint64_t X[3];
  double in[3] = {xf, yf, zf};
  for (int a = 0; a < 3; ++a)
    X[a] = (uint64_t)std::min(std::max(in[a], 0.0) * double(side), double(side - 1));
  uint64_t M = 1ull << (bits - 1);
  for (uint64_t Q = M; Q > 1; Q >>= 1) {
    uint64_t P = Q - 1;
    for (int i = 0; i < 3; ++i) {
      if (X[i] & Q)
        X[0] ^= P;
      else {
        uint64_t t = (X[0] ^ X[i]) & P;
        X[0] ^= t;
        X[i] ^= t;
      }
    }
  }
  for (int i = 1; i < 3; ++i) X[i] ^= X[i - 1];
  uint64_t t = 0;
  for (uint64_t Q = M; Q > 1; Q >>= 1)
    if (X[2] & Q) t ^= Q - 1;
  for (int i = 0; i < 3; ++i) X[i] ^= t;
  uint64_t d = 0;
  for (int b = bits - 1; b >= 0; --b)
    for (int i = 0; i < 3; ++i) d = (d << 1) | ((X[i] >> b) & 1ull);
  return d;
}

std::vector<index_t> renumber_hilbert(RawMesh &m) {
  const int nb = m.n_dims + 1;
  const index_t n = (index_t)m.vertex_indices.size() / nb;
  std::vector<Vec3> c(n);
  Vec3 lo{1e300, 1e300, 1e300}, hi{-1e300, -1e300, -1e300};
  for (index_t i = 0; i < n; ++i) {
    // vertex 0 is counted twice, as in src/renumber_grid.cpp:68-72
    Vec3 s = m.vertices[m.vertex_indices[i * nb]];
    for (int k = 0; k < nb; ++k) s = s + m.vertices[m.vertex_indices[i * nb + k]];
    c[i] = s / double(nb);
    for (int a = 0; a < 3; ++a) {
      lo[a] = std::min(lo[a], c[i][a]);
      hi[a] = std::max(hi[a], c[i][a]);
    }
  }
  std::vector<uint64_t> key(n);
  for (index_t i = 0; i < n; ++i) {
    double x = (c[i].x - lo.x) / (hi.x - lo.x + 1e-10 * std::fabs(hi.x));
    double y = (c[i].y - lo.y) / (hi.y - lo.y + 1e-10 * std::fabs(hi.y));
    if (m.n_dims == 2) {
      key[i] = hilbert_key_2d(x, y, 32);
    } else {
      double z = (c[i].z - lo.z) / (hi.z - lo.z + 1e-10 * std::fabs(hi.z));
      key[i] = hilbert_key_3d(x, y, z, 21);
    }
  }
  std::vector<index_t> sigma(n);
  std::iota(sigma.begin(), sigma.end(), 0);
  std::stable_sort(sigma.begin(), sigma.end(), [&](index_t a, index_t b) { return key[a] < key[b]; });
  std::vector<index_t> inv(n);
  for (index_t k = 0; k < n; ++k) inv[sigma[k]] = k;
  std::vector<index_t> vi(m.vertex_indices.size());
  for (index_t k = 0; k < n; ++k)
    for (int a = 0; a < nb; ++a) vi[k * nb + a] = m.vertex_indices[sigma[k] * nb + a];
  m.vertex_indices.swap(vi);
  if (!m.ghost.empty()) {
    std::vector<uint8_t> g(n);
    for (index_t k = 0; k < n; ++k) g[k] = m.ghost[sigma[k]];
    m.ghost.swap(g);
  }
  if (!m.source.empty()) {
    std::vector<index_t> s(n);
    for (index_t k = 0; k < n; ++k) s[k] = inv[m.source[sigma[k]]];
    m.source.swap(s);
  }
  return sigma;
}

}  // namespace zfvm
