// tests/cpp/refside_check.cpp -- TEST INFRASTRUCTURE: built by
// tests/test_refside_cpu.py where the reference tree is present.
//
// Links the reference's own compiled sources (src/time/helmholtz.cpp with its
// VerticalTridiagonalSolver, the dyn/grid/config objects) against
// libvibe_gb300.so INSTEAD of the reference's c_kernels.o, together with the
// reference-side adapter vibe-model_gb300/refside/gb300_integrator.hpp.
// A clean link proves the drop-in at the symbol level: every C-kernel call
// of the reference resolves to the GPU library, and the adapter compiles
// against include/vibe/time/integrator.hpp:62-82 with every virtual bound.
// Run on a machine without a GPU, both paths must fail the reference's way:
// the adapter's constructor and the vertical solve (its Thomas call returns
// VIBE_C_ERR_DEVICE) throw vibe::NumericalError.
#include <cstdio>
#include <cstring>
#include <memory>

#include "gb300_integrator.hpp"
#include "vibe/config/config.hpp"
#include "vibe/grid/decomposition.hpp"
#include "vibe/grid/geometry.hpp"
#include "vibe/time/helmholtz.hpp"

int main() {
  using namespace vibe;
  vibe_gb300_setup su;
  vibe_gb300_setup_defaults(&su);
  su.nx = 8;
  su.ny = 6;
  su.nz = 5;
  int thrown = 0;
  try {
    timeint::Gb300Integrator integ(su, VIBE_GB300_FP64);
    timeint::Integrator& base = integ;
    std::printf("adapter created: %s\n", base.name());
  } catch (const NumericalError& e) {
    std::printf("adapter: NumericalError: %s\n", e.what());
    thrown |= 1;
  }
  grid::Geometry geo;
  geo.nx = su.nx;
  geo.ny = su.ny;
  geo.nz = su.nz;
  geo.dx = su.dx;
  geo.dy = su.dy;
  geo.z_top = su.z_top;
  geo.zeta = grid::make_stretched_zeta(su.nz, 1.0, 1.0);
  geo.name = "refside";
  grid::Grid g(geo, grid::Decomposition::make(su.nx, su.ny, su.nz, 1, 1, 4, false, false));
  config::ModelConfig cfg;
  auto solver = timeint::make_helmholtz_solver(timeint::HelmholtzKind::VerticalTridiagonal, g, cfg);
  grid::Field<Real> a(g, grid::Stagger::Cell, "a"), b(g, grid::Stagger::Cell, "b"), f(g, grid::Stagger::Cell, "f"),
      x(g, grid::Stagger::Cell, "x");
  a.fill(1.0);
  b.fill(1.0);
  f.fill(1.0);
  solver->set_coefficients(a, b);
  try {
    solver->solve(a, b, f, x);
    std::printf("vertical solve through libvibe_gb300: x(0,0,0) = %.17g\n", x(0, 0, 0));
  } catch (const NumericalError& e) {
    std::printf("vertical solve: NumericalError: %s\n", e.what());
    thrown |= 2;
  }
  std::printf("thrown=%d\n", thrown);
  return 0;
}
