// vibe-model_gb300/refside/gb300_integrator.hpp
//
// The file a maintainer of the reference adds to its tree to step the
// reference's own dyn::State with the GB300 library: a
// vibe::timeint::Integrator (include/vibe/time/integrator.hpp:62-82) whose
// step() runs the device model of libvibe_gb300.so. It includes the
// reference's headers, so it compiles only inside (or against) the
// reference tree; the library itself never includes it.
//
// Behaviour, following RungeKutta3Integrator::step (runge_kutta.cpp:77-119):
//   * the state's species are copied to the device model before the step
//     and back after it (FieldT storage unchanged, field.hpp:34-184: the
//     library uses the same halo'd layout), one RK3 step with
//     ctx.acoustic_substeps substeps per stage runs on the GPU, and the
//     sponge is part of that step;
//   * a non-finite state throws vibe::NumericalError, as runge_kutta.cpp:103-106
//     (any other library error throws it too, with the library's message);
//   * the boundary callback runs after the step (runge_kutta.cpp:114), the
//     stats count steps and substeps, s.time advances by dt;
//   * a host-side physics::PhysicsDriver cannot run inside a device step:
//     with one set and ctx.physics_on, step() throws (install a device
//     package through vibe_gb300_set_physics instead, as the library's
//     Kessler package does);
//   * max_stable_dt copies the state up and asks the device
//     (vibe_gb300_max_stable_dt, the formula of runge_kutta.cpp:121-140).
// The case description (grid, reference state, numerics, composition flags)
// comes from a vibe_gb300_setup the caller fills from its ModelConfig; the
// reference's State must have that grid's dimensions.
#pragma once

#include <string>

#include "vibe/common/error.hpp"
#include "vibe/dyn/state.hpp"
#include "vibe/time/integrator.hpp"
#include "vibe_gb300.h"

namespace vibe::timeint {

class Gb300Integrator final : public Integrator {
 public:
  Gb300Integrator(const vibe_gb300_setup& s, int precision) : nspecies_(s.moist ? dyn::kNumSpecies : 7) {
    if (vibe_gb300_model_create(&s, precision, &m_) != VIBE_GB300_OK) fail("model create");
  }
  ~Gb300Integrator() override { vibe_gb300_model_destroy(m_); }
  Gb300Integrator(const Gb300Integrator&) = delete;
  Gb300Integrator& operator=(const Gb300Integrator&) = delete;

  void step(dyn::State& s, const StepContext& ctx) override {
    if (physics_ != nullptr && ctx.physics_on)
      throw std::runtime_error("Gb300Integrator: a host PhysicsDriver cannot run inside the device step; "
                               "install a device package with vibe_gb300_set_physics");
    upload(s);
    const int rc = vibe_gb300_step(m_, ctx.dt, ctx.acoustic_substeps, 1);
    if (rc == VIBE_GB300_ENONFINITE) stats_.diverged = true;
    if (rc != VIBE_GB300_OK) fail("step");
    download(s);
    stats_.acoustic_substeps += 3 * (ctx.acoustic_substeps > 1 ? ctx.acoustic_substeps : 1);
    if (boundary_) boundary_(s, ctx);
    stats_.steps += 1;
    s.time = ctx.time + ctx.dt;
  }
  const char* name() const noexcept override { return "gb300_rk3"; }
  const IntegratorStats& stats() const noexcept override { return stats_; }
  void reset_stats() override { stats_ = IntegratorStats{}; }
  Real max_stable_dt(const dyn::State& s) const override {
    upload(s);
    double dt = 0.0;
    if (vibe_gb300_max_stable_dt(m_, &dt) != VIBE_GB300_OK) fail("max_stable_dt");
    return dt;
  }
  vibe_gb300_model* model() const noexcept { return m_; }

 private:
  [[noreturn]] static void fail(const char* what) {
    throw NumericalError(std::string("Gb300Integrator ") + what + ": " + vibe_gb300_last_error());
  }
  void upload(const dyn::State& s) const {
    const double* p[dyn::kNumSpecies];
    for (int q = 0; q < nspecies_; ++q) p[q] = s.field(static_cast<dyn::Species>(q)).storage().data();
    if (vibe_gb300_set_state(m_, p, nspecies_) != VIBE_GB300_OK) fail("set_state");
  }
  void download(dyn::State& s) const {
    double* p[dyn::kNumSpecies];
    for (int q = 0; q < nspecies_; ++q) p[q] = s.field(static_cast<dyn::Species>(q)).storage().data();
    if (vibe_gb300_get_state(m_, p, nspecies_) != VIBE_GB300_OK) fail("get_state");
  }

  vibe_gb300_model* m_ = nullptr;
  int nspecies_;
  IntegratorStats stats_;
};

}  // namespace vibe::timeint
