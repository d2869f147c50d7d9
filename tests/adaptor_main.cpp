// Drives the solver through the C++ adaptors of include/zfvm_zisa.hpp, the way
// a ZisaFVM time loop would: LocalCFL, RateOfChange, RungeKutta::compute_step
// and GlobalReconstruction, then DumpSnapshot / LoadSnapshot, the numerical
// flux interface and the BoundaryCondition object.  Prints the results for
// tests/test_adaptors.py.
#define ZFVM_STANDALONE 1
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "zfvm_zisa.hpp"

int main(int argc, char **argv) {
  const int rings = argc > 1 ? std::atoi(argv[1]) : 10;
  zfvm_rawmesh *raw = nullptr;
  const int64_t ip[2] = {rings, 0};
  const double dp[2] = {1.0, 0.2};
  zfvm::check(zfvm_rawmesh_generate(1, ip, dp, 7, 1, &raw));
  int32_t nd, hg;
  int64_t nv, nc;
  zfvm::check(zfvm_rawmesh_sizes(raw, &nd, &nv, &nc, &hg));
  std::vector<double> v(nv * 3);
  std::vector<int64_t> vi(nc * (nd + 1));
  zfvm::check(zfvm_rawmesh_copy(raw, v.data(), vi.data(), nullptr, nullptr));
  zfvm_rawmesh_destroy(raw);

  zfvm_mesh_desc md{};
  md.n_dims = nd;
  md.n_vertices = nv;
  md.n_cells = nc;
  md.vertices = v.data();
  md.vertex_indices = vi.data();
  md.quad_edge = 3;
  md.quad_volume = 3;
  md.quad_moments = 2;
  md.n_stencils = 4;
  const int orders[4] = {3, 2, 2, 2};
  const double over[4] = {2.0, 1.5, 1.5, 1.5};
  for (int k = 0; k < 4; ++k) {
    md.orders[k] = orders[k];
    md.biased[k] = k > 0;
    md.overfit[k] = over[k];
  }
  zfvm_mesh *mesh = nullptr;
  zfvm::check(zfvm_mesh_create(&md, &mesh));

  zfvm_scheme_desc sc{};
  sc.flux = ZFVM_FLUX_HLLC;
  sc.gamma = 2.0;
  sc.specific_gas_constant = 1.0;
  const double lw[4] = {100.0, 1.0, 1.0, 1.0};
  for (int k = 0; k < 4; ++k) sc.linear_weights[k] = lw[k];
  sc.epsilon = 1e-6;
  sc.exponent = 4.0;
  sc.rk_stages = 3;
  sc.cfl_number = 0.45;
  sc.equilibrium = ZFVM_EQ_ISENTROPIC;
  sc.gravity = ZFVM_GRAVITY_HARMONIC_RADIAL;
  sc.gravity_strength = 1.0;
  sc.flux_bc = ZFVM_FLUX_BC_ISENTROPIC;
  sc.boundary = ZFVM_BC_NONE;
  sc.precision = ZFVM_FP64;
  sc.steps_per_recompute = 1;
  sc.n_avars = 1;

  auto u0 = std::make_shared<zfvm::AllVariables>(nc, 1);
  const double ic[8] = {2.0, 1.0, 1.0, 1.0, 1e-2, 0.05, 0.3, 0.0};
  zfvm::check(zfvm_initial_conditions(mesh, 1, ic, zfvm::cvars_data(*u0)));
  // one advected variable: a mass fraction of 0.25 + 0.5 x
  for (int64_t i = 0; i < nc; ++i) {
    double cx = 0.0;
    for (int k = 0; k < 3; ++k) cx += v[3 * vi[3 * i + k]] / 3.0;
    u0->avars[i] = u0->cvars[5 * i] * (0.25 + 0.5 * cx);
  }

  auto ds = std::make_shared<zfvm::DeviceSolver>(mesh, sc);
  zfvm::GpuLocalCFL cfl(ds);
  zfvm::GpuRateOfChange roc(ds);
  zfvm::GpuRungeKutta rk(ds, nc);
  zfvm::GpuGlobalReconstruction grc(ds);

  const double dt = cfl(*u0);
  zfvm::AllVariables tend(nc, 1);
  roc.compute(tend, *u0, 0.0);
  auto u1 = rk.compute_step(u0, 0.0, dt);
  if (u1 == u0) return 2;  // compute_step must return a different buffer
  grc.compute(*u0);
  const zfvm::XYZ x = {0.25, 0.1, 0.0};
  int64_t cell = -1;
  // the cell whose centroid is nearest to x
  double best = 1e300;
  for (int64_t i = 0; i < nc; ++i) {
    double c[2] = {0, 0};
    for (int k = 0; k < 3; ++k)
      for (int d = 0; d < 2; ++d) c[d] += v[3 * vi[3 * i + k] + d] / 3.0;
    const double r2 = (c[0] - x[0]) * (c[0] - x[0]) + (c[1] - x[1]) * (c[1] - x[1]);
    if (r2 < best) best = r2, cell = i;
  }
  const auto ux = grc(cell, x);
  const auto st = grc.stencil(cell);

  std::printf("dt %.17g\n", dt);
  std::printf("cell %lld stencil %lld\n", (long long)cell, (long long)zfvm::view_size(st));
  std::printf("recon");
  for (int k = 0; k < 5; ++k) std::printf(" %.17g", ux[k]);
  std::printf("\n");
  double s_t = 0, s_u = 0, s_tq = 0, s_q = 0;
  for (double a : tend.cvars) s_t += a;
  for (double a : u1->cvars) s_u += a;
  for (double a : tend.avars) s_tq += a;
  for (double a : u1->avars) s_q += a;
  std::printf("sums %.17g %.17g\n", s_t, s_u);
  std::printf("avars %.17g %.17g\n", s_tq, s_q);

  // DumpSnapshot / LoadSnapshot round trip of the stepped state
  const std::string dir = argc > 2 ? argv[2] : ".";
  zfvm::NpzDumpSnapshot dump(dir + "/snapshot_%04d.npz", dir + "/steady_state.npz");
  zfvm::SimulationClock clock;
  clock.advance_to(dt, 1);
  dump(*u1, clock);
  zfvm::NpzLoadSnapshot load(dump.filename(0));
  zfvm::AllVariables back(nc, 1);
  zfvm::SimulationClock clock2;
  load(back, clock2);
  std::printf("snapshot %d %.17g %lld\n", int(back.cvars == u1->cvars && back.avars == u1->avars), clock2.current_time(),
              (long long)clock2.current_step());

  // the numerical flux as a FluxLoop template argument would call it
  const zfvm::euler_var_t fl = {1.0, 0.3, -0.2, 0.1, 2.5}, fr = {0.8, 0.1, 0.05, -0.1, 1.9};
  const zfvm::IdealGasEOS eos{1.4, 1.0};
  const auto [nf, speeds] = zfvm::GpuHLLCBatten::flux(zfvm::Euler{}, eos, fl, eos, fr);
  std::printf("hllc");
  for (int k = 0; k < 5; ++k) std::printf(" %.17g", nf[k]);
  std::printf(" %.17g %.17g %.17g\n", std::get<0>(speeds), std::get<1>(speeds), std::get<2>(speeds));
  std::printf("tracer %.17g\n", zfvm::GpuHLLCBatten::tracer_flux(fl, fr, 0.4, 0.6, speeds));
  const auto [rf, rs] = zfvm::GpuRusanov::flux(zfvm::Euler{}, eos, fl, eos, fr);
  std::printf("rusanov");
  for (int k = 0; k < 5; ++k) std::printf(" %.17g", rf[k]);
  std::printf(" %.17g\n", std::get<2>(rs));

  // the boundary condition object the reference's RungeKutta applies after
  // every stage; this mesh has no ghost cells, so the state is unchanged
  zfvm::GpuBoundaryCondition bc(ds, *u0);
  zfvm::AllVariables w = *u1;
  bc.apply(w, dt);
  std::printf("bc %d\n", int(w.cvars == u1->cvars && w.avars == u1->avars));

  ds.reset();
  zfvm_mesh_destroy(mesh);
  return 0;
}
