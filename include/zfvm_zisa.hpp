// zfvm_zisa.hpp -- C++ adaptors that put the GB300 solver behind ZisaFVM's own
// interfaces.  Header-only, on top of the C ABI in zfvm.h.
//
// Inside a ZisaFVM build (its headers on the include path) the adaptors derive
// from the reference's abstract classes:
//   GpuRateOfChange      : zisa::RateOfChange      (ode/rate_of_change.hpp:23-43)
//   GpuRungeKutta        : zisa::TimeIntegration   (ode/time_integration.hpp:13-48)
//   GpuLocalCFL          : zisa::CFLCondition      (model/cfl_condition.hpp:12-18)
// Outside it (ZFVM_STANDALONE) they implement the same member signatures on a
// minimal AllVariables stand-in so the boundary compiles and tests on its own.
//
// Ownership follows the reference: compute_step never modifies *u0 and returns
// a different buffer; it keeps the state resident on the device and copies it
// to the host AllVariables only at the interface.  Errors from the C ABI are
// thrown as std::runtime_error, the equivalent of the reference's LOG_ERR.
#pragma once

#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "zfvm.h"

#if __has_include(<zisa/ode/rate_of_change.hpp>) && !defined(ZFVM_STANDALONE)
#include <zisa/model/all_variables.hpp>
#include <zisa/model/cfl_condition.hpp>
#include <zisa/ode/rate_of_change.hpp>
#include <zisa/ode/time_integration.hpp>
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
#else
// Stand-in with the reference's layout: cvars is n_cells x 5, row-major.
struct AllVariables {
  std::vector<double> cvars;
  explicit AllVariables(size_t n_cells = 0) : cvars(n_cells * 5, 0.0) {}
};
inline double *cvars_data(AllVariables &u) { return u.cvars.data(); }
inline const double *cvars_data(const AllVariables &u) { return u.cvars.data(); }
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
#endif

// Shared device solver (one mesh + scheme); the adaptors below hold it.
class DeviceSolver {
 public:
  DeviceSolver(zfvm_mesh *mesh, const zfvm_scheme_desc &scheme) { check(zfvm_solver_create(mesh, &scheme, &s_)); }
  ~DeviceSolver() { zfvm_solver_destroy(s_); }
  DeviceSolver(const DeviceSolver &) = delete;
  DeviceSolver &operator=(const DeviceSolver &) = delete;
  zfvm_solver *get() const { return s_; }

 private:
  zfvm_solver *s_ = nullptr;
};

// SumRatesOfChange{Zero, FluxLoop, GravitySource, FluxBC} of the configured scheme.
class GpuRateOfChange : public RateOfChangeBase {
 public:
  explicit GpuRateOfChange(std::shared_ptr<DeviceSolver> s) : s_(std::move(s)) {}
  void compute(AllVariables &tendency, const AllVariables &current_state, double t) const override {
    check(zfvm_set_state(s_->get(), cvars_data(current_state), t));
    check(zfvm_rate_of_change(s_->get(), cvars_data(tendency)));
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
    check(zfvm_set_state(s_->get(), cvars_data(*u0), t));
    check(zfvm_step(s_->get(), dt));
    double t_new;
    check(zfvm_get_state(s_->get(), cvars_data(*ux_), &t_new));
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

}  // namespace zfvm
