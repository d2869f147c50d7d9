// Host mesh, geometry and stencil data for the GB300 solver.
//
// A `Grid` is the set-up-time restatement of ZisaFVM's `Grid`
// (grid/grid_decl.hpp:34-107, grid/grid.cpp:651-723): neighbours, interior-first
// edge numbering with left = lower cell index, outward normals, volumes,
// in-radii, characteristic lengths, per-cell / per-face quadrature (weights
// pre-multiplied by the element volume) and normalized moments.  It also carries
// the ghost-cell flags of grid/cell_flags.hpp and, for periodic halos, the
// index of the interior cell each ghost cell copies.
#pragma once

#include "host_common.hpp"

namespace zfvm {

// kFrozen: a ghost cell that is its own source keeps its values (FrozenBC)
enum CellFlag : uint8_t { kInterior = 1, kGhost = 2, kGhostL1 = 4, kFrozen = 8 };

struct QuadDegrees {
  int edge = 3;
  int volume = 3;
  int moments = 2;
};

struct Grid {
  int n_dims = 2;
  int max_nb = 3;  // faces per cell
  index_t n_cells = 0, n_vertices = 0;
  index_t n_interior_edges = 0, n_edges = 0;

  std::vector<Vec3> vertices;
  std::vector<index_t> vertex_indices;  // n_cells * max_nb
  std::vector<index_t> neighbours;      // -1 where there is no neighbour
  std::vector<index_t> edge_indices;    // n_cells * max_nb
  std::vector<index_t> left, right;     // per edge; right = -1 on the boundary

  std::vector<double> volumes, inradii, circum_radii, char_length;
  std::vector<Vec3> cell_centers;

  int n_cell_qp = 0, n_face_qp = 0, n_moments = 0;
  std::vector<double> cell_qw;  // n_cells * n_cell_qp (times the cell volume)
  std::vector<Vec3> cell_qx;
  std::vector<double> face_qw;  // n_edges * n_face_qp (times the face area)
  std::vector<Vec3> face_qx;
  std::vector<double> face_area;
  std::vector<Vec3> face_normal, face_t1, face_t2;
  std::vector<double> moments;  // n_cells * n_moments

  std::vector<uint8_t> flags;    // CellFlag bits
  std::vector<index_t> source;   // periodic source cell (identity if none)

  int face_of_cell(index_t i, int k) const { return (int)edge_indices[i * max_nb + k]; }
  const Vec3 &vertex(index_t i, int k) const { return vertices[vertex_indices[i * max_nb + k]]; }
};

// Build all geometry from vertices and cell->vertex indices.  Vertex order is
// normalised as in grid/grid.cpp:152-203 (counter-clockwise triangles, tetrahedra
// with outward face normals).
Grid build_grid(int n_dims, std::vector<Vec3> vertices, std::vector<index_t> vertex_indices,
                const QuadDegrees &deg);

// Mark ghost cells (grid/grid.cpp:1122-1137): ghost cells are not interior, and a
// ghost cell with an interior neighbour is a first-layer ghost cell.
void mask_ghost_cells(Grid &grid, const std::vector<uint8_t> &is_ghost);

// ---- stencils (reconstruction/stencil.cpp, stencil_family.cpp) ----------------
constexpr int kMaxStencils = 5;
constexpr int kMaxL2G = 40;
constexpr int kMaxStencilSize = 24;

struct StencilParams {
  std::vector<int> orders;
  std::vector<int> biased;  // 1 = one-sided ("b"), 0 = central ("c")
  std::vector<double> overfit;
};

struct StencilFamilies {
  index_t n_cells = 0;
  std::vector<int8_t> n_stencils, k_high, n_l2g;
  std::vector<int32_t> l2g;       // n_cells * kMaxL2G
  std::vector<int8_t> order;      // n_cells * kMaxStencils
  std::vector<int8_t> size;       // n_cells * kMaxStencils (cells used by the LSQ fit)
  std::vector<int8_t> bias;       // n_cells * kMaxStencils
  std::vector<double> overfit;    // n_cells * kMaxStencils
  std::vector<int8_t> local;      // n_cells * kMaxStencils * kMaxStencilSize
};

int_fast32_t required_stencil_size(int deg, double factor, int n_dims);
int deduce_max_order(index_t stencil_size, double factor, int n_dims);

// Stencil families for every cell; interior and first-layer ghost cells get the
// requested family, deeper ghost cells a first-order one (stencil_family.cpp:99-118).
// The reference's last-resort stencil shuffles with std::random_device
// (stencil.cpp:332-334); here the shuffle is seeded per (cell, face) so the
// families are reproducible.
StencilFamilies compute_stencil_families(const Grid &grid, const StencilParams &params);

// ---- least squares (reconstruction/lsq_solver.cpp) ----------------------------
// WENO-AO matrix of a stencil (rows = stencil size - 1, cols = dof - 1), row-major.
void assemble_weno_ao_matrix(const Grid &grid, const int32_t *stencil, int n_points, int order,
                             std::vector<double> &A, int &rows, int &cols);
// Pseudo-inverse (A^T A)^{-1} A^T, cols x rows, row-major, by Householder QR.
void pseudo_inverse(const std::vector<double> &A, int rows, int cols, std::vector<double> &P);
// Numerical rank with Eigen's default JacobiSVD threshold (diag * eps * sigma_max).
int numerical_rank(const std::vector<double> &A, int rows, int cols);

// ---- meshes -------------------------------------------------------------------
struct RawMesh {
  int n_dims = 2;
  std::vector<Vec3> vertices;
  std::vector<index_t> vertex_indices;
  std::vector<uint8_t> ghost;    // optional ghost mask (empty = none)
  std::vector<index_t> source;   // optional periodic source per cell
};

// Unit square split into n x n squares of two triangles each, surrounded by a
// halo of `halo` squares; vertices jittered by U(-jitter h, jitter h) with a
// periodic jitter pattern, so halo cells are exact translates of interior cells.
RawMesh periodic_square_mesh(int n, int halo, double jitter, uint64_t seed);
// Disk of radius `radius` from concentric rings of spacing h = radius / n_rings,
// jittered interior points, made Delaunay by edge flips.
RawMesh disk_mesh(int n_rings, double radius, double jitter, uint64_t seed);
// Unit cube split into n^3 sub-cubes of six tetrahedra, interior vertices jittered.
RawMesh cube_tet_mesh(int n, double jitter, uint64_t seed);

// Hilbert renumbering of the cells (src/renumber_grid.cpp:46-135): min-max
// normalised vertex-mean centres, Hilbert key, stable sort.  Returns the new->old
// permutation and applies it to the mesh (ghost mask and sources included).
std::vector<index_t> renumber_hilbert(RawMesh &mesh);

uint64_t hilbert_key_2d(double x, double y, int bits);
uint64_t hilbert_key_3d(double x, double y, double z, int bits);

}  // namespace zfvm
