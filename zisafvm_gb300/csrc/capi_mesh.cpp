// C ABI: mesh generation, mesh set-up (geometry, stencils, LSQ operators) and
// initial data.  All of it is host work done once per mesh.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>
#include <new>

#include "gravity.hpp"
#include "mesh_obj.hpp"

namespace zfvm {

static thread_local std::string g_last_error;

void set_last_error(const std::string &msg) { g_last_error = msg; }

int fail(int code, const std::string &msg) {
  g_last_error = msg;
  return code;
}

}  // namespace zfvm

using namespace zfvm;

extern "C" const char *zfvm_last_error(void) { return g_last_error.c_str(); }

#define ZFVM_GUARD_BEGIN try {
#define ZFVM_GUARD_END                                   \
  }                                                      \
  catch (const SetupError &e) {                          \
    return fail(ZFVM_ESETUP, e.what());                  \
  }                                                      \
  catch (const std::bad_alloc &) {                       \
    return fail(ZFVM_ENOMEM, "host allocation failed");  \
  }                                                      \
  catch (const std::exception &e) {                      \
    return fail(ZFVM_EINVAL, e.what());                  \
  }

extern "C" int zfvm_rawmesh_generate(int32_t kind, const int64_t *ip, const double *dp, uint64_t seed,
                                     int32_t renumber, zfvm_rawmesh **out) {
  if (!out || !ip || !dp) return fail(ZFVM_EINVAL, "null argument");
  ZFVM_GUARD_BEGIN
  auto m = std::make_unique<zfvm_rawmesh>();
  if (kind == 0) {
    m->mesh = periodic_square_mesh((int)ip[0], (int)ip[1], dp[0], seed);
  } else if (kind == 1) {
    m->mesh = disk_mesh((int)ip[0], dp[0], dp[1], seed);
  } else if (kind == 2) {
    m->mesh = cube_tet_mesh((int)ip[0], dp[0], seed);
  } else {
    return fail(ZFVM_EINVAL, "unknown mesh kind");
  }
  if (renumber) renumber_hilbert(m->mesh);
  *out = m.release();
  return ZFVM_OK;
  ZFVM_GUARD_END
}

extern "C" int zfvm_rawmesh_sizes(const zfvm_rawmesh *m, int32_t *n_dims, int64_t *n_vertices,
                                  int64_t *n_cells, int32_t *has_ghosts) {
  if (!m) return fail(ZFVM_EINVAL, "null mesh");
  const int nb = m->mesh.n_dims + 1;
  if (n_dims) *n_dims = m->mesh.n_dims;
  if (n_vertices) *n_vertices = (int64_t)m->mesh.vertices.size();
  if (n_cells) *n_cells = (int64_t)m->mesh.vertex_indices.size() / nb;
  if (has_ghosts) *has_ghosts = !m->mesh.ghost.empty();
  return ZFVM_OK;
}

extern "C" int zfvm_rawmesh_copy(const zfvm_rawmesh *m, double *vertices, int64_t *vi, uint8_t *ghost,
                                 int64_t *source) {
  if (!m) return fail(ZFVM_EINVAL, "null mesh");
  const auto &r = m->mesh;
  if (vertices)
    for (size_t i = 0; i < r.vertices.size(); ++i) {
      vertices[3 * i] = r.vertices[i].x;
      vertices[3 * i + 1] = r.vertices[i].y;
      vertices[3 * i + 2] = r.vertices[i].z;
    }
  if (vi) std::copy(r.vertex_indices.begin(), r.vertex_indices.end(), vi);
  const size_t n = r.vertex_indices.size() / (r.n_dims + 1);
  if (ghost) {
    if (r.ghost.empty())
      std::fill(ghost, ghost + n, 0);
    else
      std::copy(r.ghost.begin(), r.ghost.end(), ghost);
  }
  if (source) {
    if (r.source.empty())
      for (size_t i = 0; i < n; ++i) source[i] = (int64_t)i;
    else
      std::copy(r.source.begin(), r.source.end(), source);
  }
  return ZFVM_OK;
}

extern "C" int zfvm_rawmesh_destroy(zfvm_rawmesh *m) {
  delete m;
  return ZFVM_OK;
}

extern "C" int zfvm_mesh_create(const zfvm_mesh_desc *d, zfvm_mesh **out) {
  if (!d || !out || !d->vertices || !d->vertex_indices) return fail(ZFVM_EINVAL, "null argument");
  if (d->n_dims != 2 && d->n_dims != 3) return fail(ZFVM_EINVAL, "n_dims must be 2 or 3");
  if (d->n_cells <= 0 || d->n_vertices <= 0) return fail(ZFVM_EINVAL, "empty mesh");
  if (d->n_stencils < 1 || d->n_stencils > ZFVM_MAX_STENCILS) return fail(ZFVM_EINVAL, "bad n_stencils");
  ZFVM_GUARD_BEGIN
  const int nb = d->n_dims + 1;
  std::vector<Vec3> v(d->n_vertices);
  for (int64_t i = 0; i < d->n_vertices; ++i)
    v[i] = {d->vertices[3 * i], d->vertices[3 * i + 1], d->vertices[3 * i + 2]};
  std::vector<index_t> vi(d->vertex_indices, d->vertex_indices + d->n_cells * nb);
  for (auto x : vi)
    if (x < 0 || x >= d->n_vertices) return fail(ZFVM_EINVAL, "vertex index out of range");
  for (int64_t i = 0; i < d->n_cells; ++i)
    for (int a = 0; a < nb; ++a)
      for (int b = a + 1; b < nb; ++b)
        if (vi[i * nb + a] == vi[i * nb + b])
          return fail(ZFVM_EINVAL, "cell " + std::to_string(i) + " repeats a vertex");
  for (const Vec3 &x : v)
    if (!std::isfinite(x.x) || !std::isfinite(x.y) || !std::isfinite(x.z))
      return fail(ZFVM_EINVAL, "non-finite vertex coordinate");
  auto m = std::make_unique<zfvm_mesh>();
  m->quad = {d->quad_edge, d->quad_volume, d->quad_moments};
  int max_order = 1;
  for (int s = 0; s < d->n_stencils; ++s) {
    m->sparams.orders.push_back(d->orders[s]);
    m->sparams.biased.push_back(d->biased[s] ? 1 : 0);
    m->sparams.overfit.push_back(d->overfit[s]);
    max_order = std::max(max_order, d->orders[s]);
    if (d->orders[s] < 1 || d->orders[s] > 4) return fail(ZFVM_EINVAL, "stencil order must be 1..4");
  }
  if (m->quad.moments >= 0 && m->quad.moments < max_order - 1)
    return fail(ZFVM_EINVAL, "quadrature.moments must be at least the polynomial degree");
  using Clk = std::chrono::steady_clock;
  auto secs = [](Clk::time_point a, Clk::time_point b) { return std::chrono::duration<double>(b - a).count(); };
  const auto t0 = Clk::now();
  m->grid = build_grid(d->n_dims, std::move(v), std::move(vi), m->quad);
  for (int64_t i = 0; i < d->n_cells; ++i)
    if (!(m->grid.volumes[i] > 0.0) || !std::isfinite(m->grid.volumes[i]))
      return fail(ZFVM_EINVAL, "cell " + std::to_string(i) + " has no volume (degenerate or flat)");
  if (d->ghost) {
    std::vector<uint8_t> g(d->ghost, d->ghost + d->n_cells);
    mask_ghost_cells(m->grid, g);
  }
  if (d->source) {
    for (int64_t i = 0; i < d->n_cells; ++i) {
      int64_t s = d->source[i];
      if (s < 0 || s >= d->n_cells) return fail(ZFVM_EINVAL, "periodic source out of range");
      // a ghost cell is either a periodic image of an interior cell or, as its
      // own source, frozen (FrozenBC, boundary/frozen_boundary_condition.cpp:39-55)
      if (!(m->grid.flags[s] & kInterior) && s != i)
        return fail(ZFVM_EINVAL, "periodic source is a ghost cell");
      if ((m->grid.flags[i] & kInterior) && s != i) return fail(ZFVM_EINVAL, "interior cell with a periodic source");
      m->grid.source[i] = s;
    }
  }
  for (int64_t i = 0; i < d->n_cells; ++i) m->n_interior += (m->grid.flags[i] & kInterior) ? 1 : 0;
  const auto t1 = Clk::now();
  m->fam = compute_stencil_families(m->grid, m->sparams);
  const auto t2 = Clk::now();
  const index_t n = m->grid.n_cells;
  m->pinv.resize(n * kMaxStencils);
  m->pinv_rows.assign(n * kMaxStencils, 0);
  m->pinv_cols.assign(n * kMaxStencils, 0);
#pragma omp parallel for schedule(dynamic, 256)
  for (index_t i = 0; i < n; ++i) {
    std::vector<double> A;
    for (int k = 0; k < m->fam.n_stencils[i]; ++k) {
      int ord = m->fam.order[i * kMaxStencils + k];
      int sz = m->fam.size[i * kMaxStencils + k];
      if (ord < 2) continue;
      int32_t glob[kMaxStencilSize];
      for (int r = 0; r < sz; ++r)
        glob[r] = m->fam.l2g[i * kMaxL2G + m->fam.local[(i * kMaxStencils + k) * kMaxStencilSize + r]];
      int rows, cols;
      assemble_weno_ao_matrix(m->grid, glob, sz, ord, A, rows, cols);
      pseudo_inverse(A, rows, cols, m->pinv[i * kMaxStencils + k]);
      m->pinv_rows[i * kMaxStencils + k] = rows;
      m->pinv_cols[i * kMaxStencils + k] = cols;
    }
  }
  const auto t3 = Clk::now();
  m->t_geometry = secs(t0, t1);
  m->t_stencils = secs(t1, t2);
  m->t_lsq = secs(t2, t3);
  *out = m.release();
  return ZFVM_OK;
  ZFVM_GUARD_END
}

extern "C" int zfvm_mesh_destroy(zfvm_mesh *m) {
  delete m;
  return ZFVM_OK;
}

extern "C" int zfvm_mesh_get_info(const zfvm_mesh *m, zfvm_mesh_info *info) {
  if (!m || !info) return fail(ZFVM_EINVAL, "null argument");
  const auto &g = m->grid;
  info->n_dims = g.n_dims;
  info->n_cells = g.n_cells;
  info->n_interior_cells = m->n_interior;
  info->n_edges = g.n_edges;
  info->n_interior_edges = g.n_interior_edges;
  info->n_cell_qp = g.n_cell_qp;
  info->n_face_qp = g.n_face_qp;
  info->n_moments = g.n_moments;
  double rmin = 1e300, rmax = 0, vol = 0;
  for (index_t i = 0; i < g.n_cells; ++i) {
    rmin = std::min(rmin, g.inradii[i]);
    rmax = std::max(rmax, g.circum_radii[i]);
    if (g.flags[i] & kInterior) vol += g.volumes[i];
  }
  info->min_inradius = rmin;
  info->max_circum_radius = rmax;
  info->total_volume = vol;
  info->setup_geometry_s = m->t_geometry;
  info->setup_stencils_s = m->t_stencils;
  info->setup_lsq_s = m->t_lsq;
  return ZFVM_OK;
}

extern "C" int zfvm_mesh_get_stencils(const zfvm_mesh *m, int8_t *n_stencils, int8_t *k_high,
                                      int8_t *n_l2g, int32_t *l2g, int8_t *order, int8_t *size,
                                      int8_t *bias, int8_t *local) {
  if (!m) return fail(ZFVM_EINVAL, "null mesh");
  const auto &f = m->fam;
  if (n_stencils) std::copy(f.n_stencils.begin(), f.n_stencils.end(), n_stencils);
  if (k_high) std::copy(f.k_high.begin(), f.k_high.end(), k_high);
  if (n_l2g) std::copy(f.n_l2g.begin(), f.n_l2g.end(), n_l2g);
  if (l2g) std::copy(f.l2g.begin(), f.l2g.end(), l2g);
  if (order) std::copy(f.order.begin(), f.order.end(), order);
  if (size) std::copy(f.size.begin(), f.size.end(), size);
  if (bias) std::copy(f.bias.begin(), f.bias.end(), bias);
  if (local) std::copy(f.local.begin(), f.local.end(), local);
  return ZFVM_OK;
}

extern "C" int zfvm_mesh_get_pinv(const zfvm_mesh *m, int64_t cell, int32_t k, double *P, int32_t *rows,
                                  int32_t *cols) {
  if (!m || cell < 0 || cell >= m->grid.n_cells || k < 0 || k >= kMaxStencils)
    return fail(ZFVM_EINVAL, "bad argument");
  size_t id = cell * kMaxStencils + k;
  if (rows) *rows = m->pinv_rows[id];
  if (cols) *cols = m->pinv_cols[id];
  if (P) std::copy(m->pinv[id].begin(), m->pinv[id].end(), P);
  return ZFVM_OK;
}

extern "C" int zfvm_mesh_get_geometry(const zfvm_mesh *m, double *volumes, double *inradii,
                                      double *centers, uint8_t *flags) {
  if (!m) return fail(ZFVM_EINVAL, "null mesh");
  const auto &g = m->grid;
  for (index_t i = 0; i < g.n_cells; ++i) {
    if (volumes) volumes[i] = g.volumes[i];
    if (inradii) inradii[i] = g.inradii[i];
    if (centers) {
      centers[3 * i] = g.cell_centers[i].x;
      centers[3 * i + 1] = g.cell_centers[i].y;
      centers[3 * i + 2] = g.cell_centers[i].z;
    }
    if (flags) flags[i] = g.flags[i];
  }
  return ZFVM_OK;
}

extern "C" int zfvm_mesh_get_connectivity(const zfvm_mesh *m, int64_t *neighbours, int64_t *edge_indices) {
  if (!m) return fail(ZFVM_EINVAL, "null mesh");
  const auto &g = m->grid;
  if (neighbours) std::copy(g.neighbours.begin(), g.neighbours.end(), neighbours);
  if (edge_indices) std::copy(g.edge_indices.begin(), g.edge_indices.end(), edge_indices);
  return ZFVM_OK;
}

extern "C" int zfvm_mesh_get_faces(const zfvm_mesh *m, int64_t *left, int64_t *right, double *normals,
                                   double *areas) {
  if (!m) return fail(ZFVM_EINVAL, "null mesh");
  const auto &g = m->grid;
  for (index_t e = 0; e < g.n_edges; ++e) {
    if (left) left[e] = g.left[e];
    if (right) right[e] = g.right[e];
    if (normals) {
      normals[3 * e] = g.face_normal[e].x;
      normals[3 * e + 1] = g.face_normal[e].y;
      normals[3 * e + 2] = g.face_normal[e].z;
    }
    if (areas) areas[e] = g.face_area[e];
  }
  return ZFVM_OK;
}

// Initial data as cell averages over the volume quadrature
// (the averaging pattern of experiments/polytrope.cpp:25-53).
extern "C" int zfvm_initial_conditions(const zfvm_mesh *m, int32_t kind, const double *p, double *cv) {
  if (!m || !p || !cv) return fail(ZFVM_EINVAL, "null argument");
  const auto &g = m->grid;
  // kind 2: the potential of the polytrope
  RadialPotential pot;
  double h_top = 0.0;  // h_c + phi(0)
  if (kind == 2) {
    zfvm_scheme_desc sc{};
    sc.gravity = (int32_t)p[7];
    sc.gravity_strength = p[8];
    for (int k = 0; k < 5; ++k) sc.gravity_params[k] = p[9 + k];
    if (sc.gravity == ZFVM_GRAVITY_RADIAL_TABLE) return fail(ZFVM_EINVAL, "no polytrope initial data for a tabulated potential");
    try {
      pot = RadialPotential::from_scheme(sc);
    } catch (const SetupError &e) {
      return fail(ZFVM_EINVAL, e.what());
    }
    const double gamma = p[0], K = p[1], rho_c = p[2];
    h_top = gamma / (gamma - 1.0) * K * std::pow(rho_c, gamma - 1.0) + pot.phi_r(0.0);
  }
  const int nq = g.n_cell_qp;
  for (index_t i = 0; i < g.n_cells; ++i) {
    double acc[5] = {0, 0, 0, 0, 0};
    for (int q = 0; q < nq; ++q) {
      const Vec3 &x = g.cell_qx[i * nq + q];
      double w = g.cell_qw[i * nq + q];
      double u[5];
      if (kind == 0) {
        // isentropic vortex (Shu) with core length scale p[4], uniform along z
        double gamma = p[0], beta = p[1], x0 = p[2], y0 = p[3], L = p[4];
        double rho_inf = p[5], u_inf = p[6], v_inf = p[7], p_inf = p[8];
        double dx = (x.x - x0) / L, dy = (x.y - y0) / L;
        double r2 = dx * dx + dy * dy;
        double e = std::exp(0.5 * (1.0 - r2));
        double du = -beta / (2.0 * M_PI) * e * dy, dv = beta / (2.0 * M_PI) * e * dx;
        double T_inf = p_inf / rho_inf;
        double dT = -(gamma - 1.0) * beta * beta / (8.0 * gamma * M_PI * M_PI) * e * e;
        double T = T_inf + dT;
        double rho = rho_inf * std::pow(T / T_inf, 1.0 / (gamma - 1.0));
        double pr = rho * T;
        double vx = u_inf + du, vy = v_inf + dv;
        u[0] = rho;
        u[1] = rho * vx;
        u[2] = rho * vy;
        u[3] = 0.0;
        u[4] = pr / (gamma - 1.0) + 0.5 * rho * (vx * vx + vy * vy);
      } else if (kind == 1) {
        // polytrope rho_eq = (h_c - phi) (gamma-1)/(gamma K) ... with phi = k r^2 / 2
        double gamma = p[0], K = p[1], rho_c = p[2], kphi = p[3], A = p[4], width = p[5];
        double x0 = p[6], y0 = p[7];
        double r2 = x.x * x.x + x.y * x.y + x.z * x.z;
        double h_c = gamma / (gamma - 1.0) * K * std::pow(rho_c, gamma - 1.0);
        double h = h_c - 0.5 * kphi * r2;
        double rho = std::pow((gamma - 1.0) / (gamma * K) * h, 1.0 / (gamma - 1.0));
        double pr = K * std::pow(rho, gamma);
        double d2 = ((x.x - x0) * (x.x - x0) + (x.y - y0) * (x.y - y0)) / (width * width);
        pr *= 1.0 + A * std::exp(-d2);
        u[0] = rho;
        u[1] = u[2] = u[3] = 0.0;
        u[4] = pr / (gamma - 1.0);
      } else if (kind == 2) {
        // isentropic polytrope in the potential: h + phi = h_c + phi(0)
        double gamma = p[0], K = p[1], A = p[3], width = p[4], x0 = p[5], y0 = p[6];
        double h = h_top - pot.phi(x);
        double rho = std::pow((gamma - 1.0) / (gamma * K) * h, 1.0 / (gamma - 1.0));
        double pr = K * std::pow(rho, gamma);
        double d2 = ((x.x - x0) * (x.x - x0) + (x.y - y0) * (x.y - y0)) / (width * width);
        pr *= 1.0 + A * std::exp(-d2);
        u[0] = rho;
        u[1] = u[2] = u[3] = 0.0;
        u[4] = pr / (gamma - 1.0);
      } else {
        return fail(ZFVM_EINVAL, "unknown initial condition kind");
      }
      for (int v = 0; v < 5; ++v) acc[v] = q == 0 ? w * u[v] : acc[v] + w * u[v];
    }
    for (int v = 0; v < 5; ++v) cv[i * 5 + v] = acc[v] / g.volumes[i];
  }
  return ZFVM_OK;
}
