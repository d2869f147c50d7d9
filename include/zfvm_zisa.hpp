// zfvm_zisa.hpp -- C++ adaptors that put the GB300 solver behind ZisaFVM's own
// interfaces.  Header-only, on top of the C ABI in zfvm.h.
//
// Inside a ZisaFVM build (its headers on the include path) the adaptors derive
// from the reference's abstract classes:
//   GpuRateOfChange         : zisa::RateOfChange      (ode/rate_of_change.hpp:23-43)
//   GpuRungeKutta           : zisa::TimeIntegration   (ode/time_integration.hpp:13-48)
//   GpuLocalCFL             : zisa::CFLCondition      (model/cfl_condition.hpp:12-18)
//   GpuGlobalReconstruction : zisa::GlobalReconstruction<euler_var_t>
//                             (reconstruction/global_reconstruction_decl.hpp:20-32)
//   GpuBoundaryCondition    : zisa::BoundaryCondition (boundary/boundary_condition.hpp:12-21)
//   GpuHLLCBatten, GpuRusanov: HLLCBatten's static numerical-flux interface
//                             (flux/hllc.hpp:142-202), a FluxLoop template argument
// Outside it (ZFVM_STANDALONE) they implement the same member signatures on a
// minimal AllVariables stand-in so the boundary compiles and tests on its own.
//
// Ownership follows the reference: compute_step never modifies *u0 and returns
// a different buffer; it keeps the state resident on the device and copies it
// to the host AllVariables only at the interface.  Errors from the C ABI are
// thrown as std::runtime_error, the equivalent of the reference's LOG_ERR.
#pragma once

#include <array>
#include <cstdio>
#include <memory>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include "zfvm.h"

#if __has_include(<zisa/ode/rate_of_change.hpp>) && !defined(ZFVM_STANDALONE)
#include <zisa/boundary/boundary_condition.hpp>
#include <zisa/model/all_variables.hpp>
#include <zisa/model/cfl_condition.hpp>
#include <zisa/ode/rate_of_change.hpp>
#include <zisa/ode/time_integration.hpp>
#include <zisa/reconstruction/global_reconstruction_decl.hpp>
#include <zisa/io/data_source.hpp>
#include <zisa/io/visualization.hpp>
#define ZFVM_HAVE_ZISA 1
#else
#define ZFVM_HAVE_ZISA 0
#endif

namespace zfvm {

inline void check(int status) {
  if (status != ZFVM_OK) throw std::runtime_error(std::string("zfvm: ") + zfvm_last_error());
}

#if ZFVM_HAVE_ZISA
using AllVariables = zisa::AllVariables;
using RateOfChangeBase = zisa::RateOfChange;
using TimeIntegrationBase = zisa::TimeIntegration;
using CFLConditionBase = zisa::CFLCondition;
inline double *cvars_data(AllVariables &u) { return u.cvars.raw(); }
inline const double *cvars_data(const AllVariables &u) { return u.cvars.raw(); }
inline double *avars_data(AllVariables &u) { return u.avars.raw(); }
inline const double *avars_data(const AllVariables &u) { return u.avars.raw(); }
inline int64_t n_cells_of(const AllVariables &u) { return int64_t(u.cvars.shape(0)); }
inline int32_t n_avars_of(const AllVariables &u) { return int32_t(u.avars.shape(1)); }
using BoundaryConditionBase = zisa::BoundaryCondition;
using VisualizationBase = zisa::Visualization;
using DataSourceBase = zisa::DataSource;
using SimulationClock = zisa::SimulationClock;
using XYZ = zisa::XYZ;
using euler_var_t = zisa::euler_var_t;
using GlobalReconstructionBase = zisa::GlobalReconstruction<zisa::euler_var_t>;
using CellsView = zisa::array_const_view<zisa::int_t, 1>;
inline CellsView cells_view(const int64_t *p, int64_t n) {
  return CellsView(zisa::shape_t<1>{zisa::int_t(n)}, reinterpret_cast<const zisa::int_t *>(p),
                   zisa::device_type::cpu);
}
inline double coord(const XYZ &x, int k) { return x[k]; }
inline euler_var_t to_cvars(const double *u) {
  euler_var_t r;
  for (int k = 0; k < 5; ++k) r[k] = u[k];
  return r;
}
inline int64_t view_size(const CellsView &v) { return int64_t(v.shape(0)); }
inline const int64_t *view_data(const CellsView &v) { return reinterpret_cast<const int64_t *>(v.raw()); }
#else
// Stand-in with the reference's layout: cvars is n_cells x 5 and avars
// n_cells x n_avars, both row-major.
struct AllVariables {
  std::vector<double> cvars, avars;
  int32_t n_avars = 0;
  explicit AllVariables(size_t n_cells = 0, int32_t n_avars_ = 0)
      : cvars(n_cells * 5, 0.0), avars(n_cells * n_avars_, 0.0), n_avars(n_avars_) {}
};
inline double *cvars_data(AllVariables &u) { return u.cvars.data(); }
inline const double *cvars_data(const AllVariables &u) { return u.cvars.data(); }
inline double *avars_data(AllVariables &u) { return u.avars.data(); }
inline const double *avars_data(const AllVariables &u) { return u.avars.data(); }
inline int64_t n_cells_of(const AllVariables &u) { return int64_t(u.cvars.size() / 5); }
inline int32_t n_avars_of(const AllVariables &u) { return u.n_avars; }
// SimulationClock's time and step count, as DumpSnapshot and LoadSnapshot use them.
struct SimulationClock {
  double t = 0.0;
  int64_t n_steps = 0;
  double current_time() const { return t; }
  int64_t current_step() const { return n_steps; }
  void advance_to(double t_, int64_t n_) { t = t_, n_steps = n_; }
};
struct VisualizationBase {
  virtual ~VisualizationBase() = default;
  void operator()(const AllVariables &u, const SimulationClock &clock) { do_visualization(u, clock); }
  void steady_state(const AllVariables &u) { do_steady_state(u); }

 protected:
  virtual void do_visualization(const AllVariables &u, const SimulationClock &clock) = 0;
  virtual void do_steady_state(const AllVariables &u) = 0;
};
struct DataSourceBase {
  virtual ~DataSourceBase() = default;
  void operator()(AllVariables &u, SimulationClock &clock) { do_load(u, clock); }

 protected:
  virtual void do_load(AllVariables &u, SimulationClock &clock) = 0;
};
struct RateOfChangeBase {
  virtual ~RateOfChangeBase() = default;
  virtual void compute(AllVariables &tendency, const AllVariables &current_state, double t) const = 0;
  virtual std::string str() const = 0;
};
struct TimeIntegrationBase {
  virtual ~TimeIntegrationBase() = default;
  virtual std::shared_ptr<AllVariables> compute_step(const std::shared_ptr<AllVariables> &u0, double t,
                                                     double dt) = 0;
  virtual std::string str() const = 0;
};
struct CFLConditionBase {
  virtual ~CFLConditionBase() = default;
  virtual double operator()(const AllVariables &all_variables) = 0;
};
struct BoundaryConditionBase {
  virtual ~BoundaryConditionBase() = default;
  virtual void apply(AllVariables &u, double t) = 0;
  virtual std::string str() const = 0;
};
// IdealGasEOS and Euler as the numerical flux receives them (only gamma is read).
struct IdealGasEOS {
  double gamma_ = 1.4, specific_gas_constant_ = 1.0;
  double gamma() const { return gamma_; }
};
struct Euler {};
using XYZ = std::array<double, 3>;
using euler_var_t = std::array<double, 5>;  // rho, m1, m2, m3, E
struct CellsView {
  const int64_t *ptr = nullptr;
  int64_t n = 0;
};
inline CellsView cells_view(const int64_t *p, int64_t n) { return CellsView{p, n}; }
inline double coord(const XYZ &x, int k) { return x[k]; }
inline euler_var_t to_cvars(const double *u) { return {u[0], u[1], u[2], u[3], u[4]}; }
inline int64_t view_size(const CellsView &v) { return v.n; }
inline const int64_t *view_data(const CellsView &v) { return v.ptr; }
struct GlobalReconstructionBase {
  virtual ~GlobalReconstructionBase() = default;
  virtual void compute(const AllVariables &current_state) = 0;
  virtual void compute(const AllVariables &current_state, const CellsView &cells) = 0;
  virtual euler_var_t operator()(int64_t i, const XYZ &x) const = 0;
  virtual CellsView stencil(int64_t i) const = 0;
};
#endif

// Shared device solver (one mesh + scheme); the adaptors below hold it.
class DeviceSolver {
 public:
  DeviceSolver(zfvm_mesh *mesh, const zfvm_scheme_desc &scheme) : mesh_(mesh), n_avars_(scheme.n_avars) {
    check(zfvm_solver_create(mesh, &scheme, &s_));
  }
  ~DeviceSolver() { zfvm_solver_destroy(s_); }
  DeviceSolver(const DeviceSolver &) = delete;
  DeviceSolver &operator=(const DeviceSolver &) = delete;
  zfvm_solver *get() const { return s_; }
  zfvm_mesh *mesh() const { return mesh_; }
  int32_t n_avars() const { return n_avars_; }
  // upload / download a whole AllVariables (cvars, and avars when the scheme has them)
  void set(const AllVariables &u, double t) const {
    if (n_avars_of(u) != n_avars_) throw std::runtime_error("zfvm: AllVariables has the wrong number of avars");
    check(zfvm_set_state(s_, cvars_data(u), t));
    if (n_avars_) check(zfvm_set_avars(s_, avars_data(u)));
  }
  double get_into(AllVariables &u) const {
    double t;
    check(zfvm_get_state(s_, cvars_data(u), &t));
    if (n_avars_) check(zfvm_get_avars(s_, avars_data(u)));
    return t;
  }

 private:
  zfvm_mesh *mesh_ = nullptr;
  zfvm_solver *s_ = nullptr;
  int32_t n_avars_ = 0;
};

// SumRatesOfChange{Zero, FluxLoop, GravitySource, FluxBC} of the configured scheme.
class GpuRateOfChange : public RateOfChangeBase {
 public:
  explicit GpuRateOfChange(std::shared_ptr<DeviceSolver> s) : s_(std::move(s)) {}
  void compute(AllVariables &tendency, const AllVariables &current_state, double t) const override {
    s_->set(current_state, t);
    check(zfvm_rate_of_change_all(s_->get(), cvars_data(tendency), avars_data(tendency)));
  }
  std::string str() const override { return "GB300 rate of change (`GpuRateOfChange`)"; }

 private:
  std::shared_ptr<DeviceSolver> s_;
};

// RungeKutta (SSP-RK) with the rate of change on the device.
class GpuRungeKutta : public TimeIntegrationBase {
 public:
  GpuRungeKutta(std::shared_ptr<DeviceSolver> s, size_t n_cells) : s_(std::move(s)), n_cells_(n_cells) {}
  std::shared_ptr<AllVariables> compute_step(const std::shared_ptr<AllVariables> &u0, double t,
                                             double dt) override {
    // the reference keeps u0 for reuse and returns its other buffer
    if (!ux_ || ux_ == u0) ux_ = std::make_shared<AllVariables>(*u0);
    if (s_->n_avars()) {
      s_->set(*u0, t);
      check(zfvm_step(s_->get(), dt));
      s_->get_into(*ux_);
    } else {
      // upload, one step of dt, download: one call, one synchronisation
      double t_new;
      int64_t steps;
      check(zfvm_step_host(s_->get(), cvars_data(*u0), t, 1, 0.0, dt, cvars_data(*ux_), &t_new, &steps));
    }
    auto out = ux_;
    ux_ = u0;
    return out;
  }
  std::string str() const override { return "GB300 SSP Runge-Kutta (`GpuRungeKutta`)"; }

 private:
  std::shared_ptr<DeviceSolver> s_;
  size_t n_cells_;
  std::shared_ptr<AllVariables> ux_;
};

// LocalCFL on the device.
class GpuLocalCFL : public CFLConditionBase {
 public:
  explicit GpuLocalCFL(std::shared_ptr<DeviceSolver> s) : s_(std::move(s)) {}
  double operator()(const AllVariables &u) override {
    check(zfvm_set_state(s_->get(), cvars_data(u), 0.0));
    double dt;
    check(zfvm_cfl_dt(s_->get(), &dt));
    return dt;
  }

 private:
  std::shared_ptr<DeviceSolver> s_;
};

// EulerGlobalReconstruction on the device: compute() reconstructs the state in
// every cell (the reference's `cells` subset is reconstructed along with the
// rest), operator()(i, x) evaluates the limited polynomial plus the
// equilibrium at x on the host, stencil(i) is the cell's combined stencil.
class GpuGlobalReconstruction : public GlobalReconstructionBase {
 public:
  explicit GpuGlobalReconstruction(std::shared_ptr<DeviceSolver> s) : s_(std::move(s)) {
    zfvm_mesh_info info;
    check(zfvm_mesh_get_info(s_->mesh(), &info));
    const int64_t n = info.n_cells;
    std::vector<int8_t> ns(n), kh(n), nl(n), order(n * ZFVM_MAX_STENCILS), size(n * ZFVM_MAX_STENCILS),
        bias(n * ZFVM_MAX_STENCILS), local(n * ZFVM_MAX_STENCILS * ZFVM_MAX_STENCIL_SIZE);
    std::vector<int32_t> l2g(n * ZFVM_MAX_L2G);
    check(zfvm_mesh_get_stencils(s_->mesh(), ns.data(), kh.data(), nl.data(), l2g.data(), order.data(),
                                 size.data(), bias.data(), local.data()));
    l2g_.resize(l2g.size());
    for (size_t k = 0; k < l2g.size(); ++k) l2g_[k] = l2g[k];
    n_l2g_.assign(nl.begin(), nl.end());
  }
  void compute(const AllVariables &current_state) override {
    check(zfvm_set_state(s_->get(), cvars_data(current_state), 0.0));
    check(zfvm_reconstruct(s_->get()));
  }
  void compute(const AllVariables &current_state, const CellsView &) override { compute(current_state); }
  euler_var_t operator()(int64_t i, const XYZ &x) const override {
    const double p[3] = {coord(x, 0), coord(x, 1), coord(x, 2)};
    double u[5];
    check(zfvm_reconstruction_eval(s_->get(), 1, &i, p, u));
    return to_cvars(u);
  }
  CellsView stencil(int64_t i) const override {
    return cells_view(l2g_.data() + i * ZFVM_MAX_L2G, n_l2g_[i]);
  }
  std::string str() const { return "GB300 global reconstruction (`GpuGlobalReconstruction`)"; }

 private:
  std::shared_ptr<DeviceSolver> s_;
  std::vector<int64_t> l2g_;
  std::vector<int64_t> n_l2g_;
};

// A numerical flux with HLLCBatten's static interface (flux/hllc.hpp:142-202),
// evaluated by the same device code as the solver's face kernel: the flux of
// two face states (normal momentum first) with the wave speeds of the fan, and
// the flux of an advected variable for those speeds.  One call is one launch;
// flux_batch evaluates many face points in one.
template <int32_t FLUX>
struct GpuNumericalFlux {
  using speeds_t = std::tuple<double, double, double>;

  template <class EulerT, class EOS>
  static std::tuple<euler_var_t, speeds_t> flux(const EulerT &, const EOS &eosL, const euler_var_t &uL,
                                                const EOS &eosR, const euler_var_t &uR) {
    if (eosL.gamma() != eosR.gamma()) throw std::runtime_error("zfvm: the flux needs one ideal gas on both sides");
    double a[5], b[5], f[5], sp[3];
    for (int k = 0; k < 5; ++k) a[k] = uL[k], b[k] = uR[k];
    check(zfvm_numerical_flux(FLUX, eosL.gamma(), 1, a, b, f, sp));
    return {to_cvars(f), speeds_t{sp[0], sp[1], sp[2]}};
  }
  static double tracer_flux(const euler_var_t &uL, const euler_var_t &uR, double mqL, double mqR,
                            const speeds_t &speeds) {
    double a[5], b[5], f;
    for (int k = 0; k < 5; ++k) a[k] = uL[k], b[k] = uR[k];
    const double sp[3] = {std::get<0>(speeds), std::get<1>(speeds), std::get<2>(speeds)};
    check(zfvm_tracer_flux(FLUX, 1, a, b, &mqL, &mqR, sp, &f));
    return f;
  }
  // n face points (rows of 5) in one launch; speeds n x 3 (may be null)
  static void flux_batch(double gamma, int64_t n, const double *uL, const double *uR, double *f, double *speeds) {
    check(zfvm_numerical_flux(FLUX, gamma, n, uL, uR, f, speeds));
  }
  static std::string str() {
    return FLUX == ZFVM_FLUX_HLLC ? "HLLC with Batten wavespeeds on the GPU (`GpuHLLCBatten`)"
                                  : "Rusanov on the GPU (`GpuRusanov`)";
  }
};
using GpuHLLCBatten = GpuNumericalFlux<ZFVM_FLUX_HLLC>;
using GpuRusanov = GpuNumericalFlux<ZFVM_FLUX_RUSANOV>;

// The solver's ghost-cell boundary condition as a BoundaryCondition object for
// the reference's RungeKutta: frozen ghost cells are reset to the rows of the
// state given at construction (FrozenBC, boundary/frozen_boundary_condition.cpp:11-55),
// periodic images take their source cells' rows.
class GpuBoundaryCondition : public BoundaryConditionBase {
 public:
  GpuBoundaryCondition(std::shared_ptr<DeviceSolver> s, const AllVariables &frozen)
      : s_(std::move(s)), frozen_(frozen) {}
  void apply(AllVariables &u, double /* t */) override {
    const bool q = s_->n_avars() > 0;
    check(zfvm_apply_boundary(s_->get(), cvars_data(frozen_), q ? avars_data(frozen_) : nullptr, cvars_data(u),
                              q ? avars_data(u) : nullptr));
  }
  std::string str() const override { return "GB300 ghost-cell boundary conditions (`GpuBoundaryCondition`)"; }

 private:
  std::shared_ptr<DeviceSolver> s_;
  AllVariables frozen_;
};

// DumpSnapshot (io/dump_snapshot_impl.hpp:21-38) writing .npz snapshot files
// with the reference's dataset names.  `pattern` is a printf pattern of the
// generation number, the FileNameGenerator's dir + stem + pattern + suffix
// (io/file_name_generator.cpp:9-27), e.g. "out/snapshot_%04d.npz".
class NpzDumpSnapshot : public VisualizationBase {
 public:
  NpzDumpSnapshot(std::string pattern, std::string steady_state_name, int first_generation = 0)
      : pattern_(std::move(pattern)), steady_(std::move(steady_state_name)), count_(first_generation) {}
  std::string filename(int generation) const {
    std::vector<char> buf(pattern_.size() + 32);
    std::snprintf(buf.data(), buf.size(), pattern_.c_str(), generation);
    return std::string(buf.data());
  }

 protected:
  void do_visualization(const AllVariables &u, const SimulationClock &clock) override {
    write(filename(count_++), u, 1, clock.current_time(), int64_t(clock.current_step()));
  }
  void do_steady_state(const AllVariables &u) override { write(steady_, u, 0, 0.0, 0); }

 private:
  static void write(const std::string &name, const AllVariables &u, int32_t with_clock, double t, int64_t n) {
    check(zfvm_snapshot_write(name.c_str(), n_cells_of(u), cvars_data(u), n_avars_of(u), avars_data(u), with_clock,
                              t, n));
  }
  std::string pattern_, steady_;
  int count_;
};

// LoadSnapshot (io/load_snapshot.cpp:9-13): the state from a snapshot file and
// the clock advanced to its time and step count.  The AllVariables must have
// the file's numbers of cells and advected variables.
class NpzLoadSnapshot : public DataSourceBase {
 public:
  explicit NpzLoadSnapshot(std::string file_name) : file_(std::move(file_name)) {}

 protected:
  void do_load(AllVariables &u, SimulationClock &clock) override {
    double t = 0.0;
    int64_t n = 0;
    check(zfvm_snapshot_read(file_.c_str(), n_cells_of(u), cvars_data(u), n_avars_of(u), avars_data(u), &t, &n));
    clock.advance_to(t, n);
  }

 private:
  std::string file_;
};

}  // namespace zfvm
