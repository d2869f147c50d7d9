// Host-side mesh handle behind the C ABI: geometry, stencil families and the
// per-stencil least-squares pseudo-inverses, computed once per mesh.
#pragma once

#include <string>
#include <vector>

#include "../../include/zfvm.h"
#include "grid.hpp"

struct zfvm_mesh {
  zfvm::Grid grid;
  zfvm::QuadDegrees quad;
  zfvm::StencilParams sparams;
  zfvm::StencilFamilies fam;
  // pinv[(i * kMaxStencils + k)] is (cols x rows) row-major, empty for order 1
  std::vector<std::vector<double>> pinv;
  std::vector<int> pinv_rows, pinv_cols;
  zfvm::index_t n_interior = 0;
  double t_geometry = 0.0, t_stencils = 0.0, t_lsq = 0.0;  // set-up phase wall times (s)
};

struct zfvm_rawmesh {
  zfvm::RawMesh mesh;
};

namespace zfvm {
void set_last_error(const std::string &msg);
int fail(int code, const std::string &msg);
}  // namespace zfvm
