// include/vibe_gb300.hpp
//
// C++ interfaces of the GB300 dynamics step, mirroring the reference's
// stepper interfaces over the C ABI (header-only; link libvibe_gb300.so):
//   vibe::gb300::StepContext, IntegratorStats  timeint::StepContext /
//                                              IntegratorStats (integrator.hpp:34-59)
//   vibe::gb300::Integrator                    timeint::Integrator (integrator.hpp:62-82)
//   vibe::gb300::Rk3Integrator                 RungeKutta3Integrator (runge_kutta.hpp:46-80)
//   vibe::gb300::SemiImplicitIntegrator        SemiImplicitIntegrator (semi_implicit.hpp:48-91)
//   vibe::gb300::AcousticSubstepper            AcousticSubstepper (acoustic_substep.hpp:55-85)
//   vibe::gb300::HelmholtzSolver,
//   make_helmholtz_solver                      HelmholtzSolver (helmholtz.hpp:63-98)
//   vibe::gb300::TangentLinearModel /
//   AdjointModel                               da::TangentLinearModel / AdjointModel
//                                              (tangent_linear.hpp:80-150)
//   vibe::gb300::NumericalError                NumericalError (error.hpp)
// The state is device-resident: State owns the GPU model (grid metrics,
// reference state, fields); field() / set_field() copy one species in the
// reference's FieldT storage layout. As in the reference, failures throw
// (NumericalError for non-finite states and singular solves, std::runtime_error
// for bad arguments and device errors) and one object is not thread-safe.
#ifndef VIBE_GB300_HPP
#define VIBE_GB300_HPP

#include <cmath>
#include <functional>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "vibe_gb300.h"
#include "vibe_helmholtz.h"
#include "vibe_tlad.h"

namespace vibe::gb300 {

class NumericalError : public std::runtime_error {
 public:
  using std::runtime_error::runtime_error;
};

inline void check(int rc) {
  if (rc == VIBE_GB300_OK) return;
  const std::string msg = vibe_gb300_last_error();
  if (rc == VIBE_GB300_ENONFINITE || rc == VIBE_GB300_ESINGULAR) throw NumericalError(msg);
  throw std::runtime_error(msg);
}

enum class Precision { FP64 = VIBE_GB300_FP64, Mixed = VIBE_GB300_MIXED, FP64Exact = VIBE_GB300_FP64_EXACT };

// timeint::StepContext (integrator.hpp:34-50)
struct StepContext {
  double dt = 1.0;
  double dt_acoustic = 1.0;
  int acoustic_substeps = 1;
  double time = 0.0;
  bool physics_on = true;
  static StepContext make(double dt, int substeps, double time) {
    StepContext c;
    c.dt = dt;
    c.acoustic_substeps = substeps;
    c.dt_acoustic = dt / static_cast<double>(substeps);
    c.time = time;
    return c;
  }
};

// timeint::IntegratorStats (integrator.hpp:53-59)
struct IntegratorStats {
  long steps = 0, acoustic_substeps = 0;
  double wall_time = 0.0;
  int helmholtz_iterations = 0;
  double helmholtz_residual = 0.0;
  bool diverged = false;
};

// The device-resident state of one domain.
class State {
 public:
  static vibe_gb300_setup defaults() {
    vibe_gb300_setup s;
    vibe_gb300_setup_defaults(&s);
    return s;
  }
  State(const vibe_gb300_setup& s, Precision p) : setup_(s) {
    vibe_gb300_model* m = nullptr;
    check(vibe_gb300_model_create(&s, static_cast<int>(p), &m));
    m_.reset(m);
  }
  vibe_gb300_model* model() const { return m_.get(); }
  const vibe_gb300_setup& setup() const { return setup_; }
  size_t size(int species) const { return vibe_gb300_storage_size(m_.get(), species); }
  std::vector<double> field(int species) const {
    std::vector<double> out(size(species));
    check(vibe_gb300_get_field(m_.get(), species, out.data()));
    return out;
  }
  void set_field(int species, const std::vector<double>& v) {
    if (v.size() != size(species)) throw std::runtime_error("set_field: wrong storage size");
    check(vibe_gb300_set_field(m_.get(), species, v.data()));
  }
  double time = 0.0;
  long step = 0;

 private:
  struct Del {
    void operator()(vibe_gb300_model* m) const { vibe_gb300_model_destroy(m); }
  };
  vibe_gb300_setup setup_;
  std::unique_ptr<vibe_gb300_model, Del> m_;
};

// A device physics package for Integrator::set_physics: the built-in Kessler
// warm-rain scheme with PhysicsOptions' defaults (vibe_gb300_physics_kessler).
struct KesslerPhysics {
  vibe_gb300_kessler options{};
  KesslerPhysics() { vibe_gb300_kessler_defaults(&options); }
  vibe_gb300_physics_fn fn() const { return vibe_gb300_physics_kessler; }
  void* user() { return &options; }
};

// timeint::Integrator (integrator.hpp:62-82). set_physics takes a device
// package (vibe_gb300_set_physics) in place of a host PhysicsDriver*; it is
// installed on the state's model at the next step.
class Integrator {
 public:
  using BoundaryCallback = std::function<void(State&, const StepContext&)>;
  virtual ~Integrator() = default;
  virtual void step(State& s, const StepContext& ctx) = 0;
  virtual const char* name() const noexcept = 0;
  const IntegratorStats& stats() const noexcept { return stats_; }
  void reset_stats() { stats_ = {}; }
  virtual double max_stable_dt(const State& s) const {
    double dt = 0.0;
    check(vibe_gb300_max_stable_dt(s.model(), &dt));
    return dt;
  }
  virtual void set_boundary_callback(BoundaryCallback cb) { boundary_ = std::move(cb); }
  virtual void set_physics(vibe_gb300_physics_fn fn, void* user) {
    phys_fn_ = fn;
    phys_user_ = user;
    phys_dirty_ = true;
    phys_ever_ = phys_ever_ || fn != nullptr;
  }

 protected:
  // the package goes onto a model once per change (installing drops the
  // step graphs); a removed package is taken off the next state stepped
  void install_physics(State& s) {
    if (!phys_dirty_ && phys_model_ == s.model()) return;
    if (!phys_ever_) return;
    check(vibe_gb300_set_physics(s.model(), phys_fn_, phys_user_));
    phys_model_ = s.model();
    phys_dirty_ = false;
  }
  IntegratorStats stats_{};
  BoundaryCallback boundary_;
  vibe_gb300_physics_fn phys_fn_ = nullptr;
  void* phys_user_ = nullptr;
  vibe_gb300_model* phys_model_ = nullptr;
  bool phys_dirty_ = false, phys_ever_ = false;
};

// RungeKutta3Integrator: SSP-RK3 with n_sub acoustic substeps per stage and
// the sponge, on the device (vibe_gb300_step).
class Rk3Integrator final : public Integrator {
 public:
  void step(State& s, const StepContext& ctx) override {
    install_physics(s);
    const int rc = vibe_gb300_step(s.model(), ctx.dt, ctx.acoustic_substeps, 1);
    if (rc == VIBE_GB300_ENONFINITE) stats_.diverged = true;
    check(rc);
    stats_.steps += 1;
    stats_.acoustic_substeps += 3 * ctx.acoustic_substeps;
    s.time = ctx.time + ctx.dt;
    s.step += 1;
    if (boundary_) boundary_(s, ctx);
  }
  const char* name() const noexcept override { return "runge_kutta3"; }
};

// SemiImplicitIntegrator (vibe_gb300_si_step) with the Helmholtz solver kind,
// max_iter and tol of cfg.numerics (helmholtz_solver / _max_iter / _tol).
class SemiImplicitIntegrator final : public Integrator {
 public:
  explicit SemiImplicitIntegrator(int helmholtz_kind = VIBE_HZ_KRYLOV_MULTIGRID, int max_iter = 200,
                                  double tol = 1e-8)
      : kind_(helmholtz_kind), max_iter_(max_iter), tol_(tol) {}
  void step(State& s, const StepContext& ctx) override {
    int it = 0;
    double res = 0.0;
    const int rc = vibe_gb300_si_step(s.model(), ctx.dt, kind_, max_iter_, tol_, &it, &res, nullptr);
    if (rc == VIBE_GB300_ENONFINITE) stats_.diverged = true;
    check(rc);
    stats_.helmholtz_iterations += it;
    stats_.helmholtz_residual = res;
    stats_.steps += 1;
    s.time = ctx.time + ctx.dt;
    s.step += 1;
    if (boundary_) boundary_(s, ctx);
  }
  const char* name() const noexcept override { return "semi_implicit"; }

 private:
  int kind_, max_iter_;
  double tol_;
};

// AcousticSubstepper (acoustic_substep.hpp:55-85) on the device state.
class AcousticSubstepper {
 public:
  // one substep: HEVI (acoustic_mode 1 or 2 of the setup) or explicit FB
  void step(State& s, double dtau) const {
    if (s.setup().acoustic_mode == 0) check(vibe_gb300_acoustic_substep(s.model(), dtau));
    else check(vibe_gb300_hevi_substep(s.model(), dtau));
  }
  double acoustic_cfl(const State& s, double dtau) const {
    double ac = 0.0;
    check(vibe_gb300_cfl(s.model(), 1.0, dtau, nullptr, nullptr, &ac));
    return ac;
  }
  int required_substeps(const State& s, double dt, double safety = 0.8) const {
    const double cfl = acoustic_cfl(s, dt);
    if (cfl <= safety || cfl <= 0.0) return 1;
    return static_cast<int>(std::ceil(cfl / safety));
  }
};

// HelmholtzSolver (helmholtz.hpp:63-98). Fields: FieldT cell storage.
class HelmholtzSolver {
 public:
  HelmholtzSolver(int kind, int nx, int ny, int nz, double dx, double dy, double z_top,
                  const std::vector<double>& dzeta, const std::vector<double>& zs, int max_iter, double tol) {
    vibe_helmholtz* h = nullptr;
    const int rc = vibe_helmholtz_create(kind, nx, ny, nz, dx, dy, z_top, dzeta.data(),
                                         zs.empty() ? nullptr : zs.data(), max_iter, tol, &h);
    if (rc != VIBE_C_OK) throw std::runtime_error(vibe_helmholtz_last_error());
    h_.reset(h);
  }
  void set_coefficients(const std::vector<double>& a, const std::vector<double>& b) {
    if (vibe_helmholtz_set_coefficients(h_.get(), a.data(), b.data()) != VIBE_C_OK)
      throw std::runtime_error(vibe_helmholtz_last_error());
  }
  void solve(const std::vector<double>& a, const std::vector<double>& b, const std::vector<double>& f,
             std::vector<double>& x) {
    x.resize(f.size());
    const int rc = vibe_helmholtz_solve(h_.get(), a.data(), b.data(), f.data(), x.data());
    if (rc == VIBE_C_ERR_SINGULAR) throw NumericalError(vibe_helmholtz_last_error());
    if (rc != VIBE_C_OK) throw std::runtime_error(vibe_helmholtz_last_error());
  }
  int iterations() const noexcept { return vibe_helmholtz_iterations(h_.get()); }
  double residual() const noexcept { return vibe_helmholtz_residual(h_.get()); }
  const char* name() const noexcept { return vibe_helmholtz_name(h_.get()); }
  void set_iterative_refinement(bool on, int precision = 3) {
    vibe_helmholtz_set_iterative_refinement(h_.get(), on ? 1 : 0, precision);
  }

 private:
  struct Del {
    void operator()(vibe_helmholtz* h) const { vibe_helmholtz_destroy(h); }
  };
  std::unique_ptr<vibe_helmholtz, Del> h_;
};

// make_helmholtz_solver (helmholtz.cpp:478-494) for a model's grid
inline std::unique_ptr<HelmholtzSolver> make_helmholtz_solver(int kind, const State& s, int max_iter = 200,
                                                              double tol = 1e-8) {
  const vibe_gb300_setup& su = s.setup();
  std::vector<double> zeta(su.nz + 1), zs((size_t)su.nx * su.ny), dzeta(su.nz);
  check(vibe_gb300_get_zeta(s.model(), zeta.data()));
  check(vibe_gb300_get_terrain(s.model(), zs.data()));
  for (int k = 0; k < su.nz; ++k) dzeta[k] = zeta[k + 1] - zeta[k];
  return std::make_unique<HelmholtzSolver>(kind, su.nx, su.ny, su.nz, su.dx, su.dy, su.z_top, dzeta, zs,
                                           max_iter, tol);
}

// da::TangentLinearModel + da::AdjointModel over 12-species FieldT states.
class TangentLinearModel {
 public:
  using Fields = std::vector<std::vector<double>>;
  TangentLinearModel(const State& grid_of, int precision = 0) {
    const vibe_gb300_setup& su = grid_of.setup();
    std::vector<double> zeta(su.nz + 1), zs((size_t)su.nx * su.ny), dzeta(su.nz);
    check(vibe_gb300_get_zeta(grid_of.model(), zeta.data()));
    check(vibe_gb300_get_terrain(grid_of.model(), zs.data()));
    for (int k = 0; k < su.nz; ++k) dzeta[k] = zeta[k + 1] - zeta[k];
    vibe_tlad* t = nullptr;
    if (vibe_tlad_create(su.nx, su.ny, su.nz, su.dx, su.dy, su.z_top, dzeta.data(), zs.data(), precision, &t) !=
        VIBE_C_OK)
      throw std::runtime_error(vibe_tlad_last_error());
    t_.reset(t);
  }
  void set_base(const Fields& xb) { ok(vibe_tlad_set_base(t_.get(), ptrs(xb).data())); }
  // TangentLinearModel::propagate (base state frozen, as the reference)
  void propagate(const Fields& dx0, double dt, int n_steps, Fields& out) {
    out = dx0;
    auto o = mptrs(out);
    ok(vibe_tl_propagate(t_.get(), dt, n_steps, ptrs(dx0).data(), o.data()));
  }
  // AdjointModel::propagate_with_trajectory over the same trajectory
  void adjoint(const Fields& dy, double dt, int n_steps, Fields& out) {
    out = dy;
    auto o = mptrs(out);
    ok(vibe_ad_propagate(t_.get(), dt, n_steps, ptrs(dy).data(), o.data()));
  }

 private:
  static void ok(int rc) {
    if (rc != VIBE_C_OK) throw std::runtime_error(vibe_tlad_last_error());
  }
  static std::vector<const double*> ptrs(const Fields& f) {
    std::vector<const double*> p;
    for (const auto& v : f) p.push_back(v.data());
    return p;
  }
  static std::vector<double*> mptrs(Fields& f) {
    std::vector<double*> p;
    for (auto& v : f) p.push_back(v.data());
    return p;
  }
  struct Del {
    void operator()(vibe_tlad* t) const { vibe_tlad_destroy(t); }
  };
  std::unique_ptr<vibe_tlad, Del> t_;
};

}  // namespace vibe::gb300

#endif
