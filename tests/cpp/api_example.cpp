// tests/cpp/api_example.cpp -- a host program written against the C++
// interfaces of include/vibe_gb300.hpp, the way the reference's own driver
// uses timeint::Integrator (src/driver/driver.cpp:127-138,288): build a
// state, step it with the RK3 integrator and the semi-implicit integrator,
// solve a Helmholtz problem, step a moist state with the Kessler physics
// package installed through Integrator::set_physics, and run the TL/AD
// dot-product test. It writes the fields it produced to the file named by
// argv[1] for the test to compare.
#include <cstdio>
#include <cstring>
#include <vector>

#include "vibe_gb300.hpp"

using namespace vibe::gb300;

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  FILE* out = std::fopen(argv[1], "wb");
  if (!out) return 2;
  auto dump = [&](const std::vector<double>& v) { std::fwrite(v.data(), sizeof(double), v.size(), out); };
  try {
    vibe_gb300_setup su = State::defaults();
    su.nx = 20; su.ny = 16; su.nz = 12; su.dx = 250.0; su.dy = 250.0; su.z_top = 3000.0;
    su.zeta_stretch = 1.08; su.bubble_xc = 2500.0; su.bubble_yc = 2000.0; su.bubble_zc = 1000.0;
    su.bubble_radius_x = 1500.0; su.bubble_radius_z = 1000.0; su.u_background = 5.0; su.shear_u = 0.001;
    State s(su, Precision::FP64);
    Rk3Integrator rk3;
    const double dt = 1.0;  // below max_stable_dt for this case
    for (int n = 0; n < 2; ++n) rk3.step(s, StepContext::make(dt, 4, s.time));
    for (int q = 0; q < 7; ++q) dump(s.field(q));
    std::printf("rk3: %ld steps, %ld substeps, t = %.1f, max_stable_dt = %.6f\n", rk3.stats().steps,
                rk3.stats().acoustic_substeps, s.time, rk3.max_stable_dt(s));

    State si(su, Precision::FP64);
    SemiImplicitIntegrator sint(VIBE_HZ_VERTICAL_TRIDIAGONAL);
    sint.step(si, StepContext::make(2.0, 1, 0.0));
    for (int q = 0; q < 7; ++q) dump(si.field(q));
    std::printf("si: helmholtz iterations %d\n", sint.stats().helmholtz_iterations);

    auto hz = make_helmholtz_solver(VIBE_HZ_MG_BICGSTAB_MIXED, si, 200, 1e-10);
    const size_t n = si.size(VIBE_RHO);
    std::vector<double> a(n, 0.0), b(n, 0.0), f(n, 0.0), x;
    for (int k = 0; k < su.nz; ++k)
      for (int j = 0; j < su.ny; ++j)
        for (int i = 0; i < su.nx; ++i) {
          const size_t c = ((size_t)(k + 4) * (su.ny + 8) + (j + 4)) * (su.nx + 8) + (i + 4);
          a[c] = 1e5 * (1.0 + 0.1 * ((i * 7 + j * 3 + k) % 5));
          b[c] = 1.0;
          f[c] = std::sin(0.3 * i) * std::cos(0.2 * j) + 0.01 * k;
        }
    hz->solve(a, b, f, x);
    dump(x);
    std::printf("helmholtz %s: %d iterations, residual %.3e\n", hz->name(), hz->iterations(), hz->residual());

    vibe_gb300_setup mo = su;
    mo.moist = 1; mo.qv_surface = 0.025; mo.qv_decay_height = 2500.0;
    State wet(mo, Precision::FP64);
    KesslerPhysics kessler;
    kessler.options.exner_offset = 0;
    Rk3Integrator rk3w;
    rk3w.set_physics(kessler.fn(), kessler.user());
    for (int n = 0; n < 2; ++n) rk3w.step(wet, StepContext::make(dt, 4, wet.time));
    for (int q : {VIBE_THETA, VIBE_QV, VIBE_QC, VIBE_QR}) dump(wet.field(q));

    AcousticSubstepper sub;
    std::printf("acoustic cfl %.6f, substeps for dt=4: %d\n", sub.acoustic_cfl(s, 0.25), sub.required_substeps(s, 4.0));

    TangentLinearModel tl(s);
    TangentLinearModel::Fields xb(12), dx(12), dy(12), mdx, mtdy;
    for (int q = 0; q < 12; ++q) {
      xb[q] = s.field(q);
      dx[q].assign(xb[q].size(), 0.0);
      dy[q].assign(xb[q].size(), 0.0);
      for (size_t e = 0; e < dx[q].size(); ++e) {
        dx[q][e] = std::sin(0.37 * (double)e + q);
        dy[q][e] = std::cos(0.11 * (double)e - q);
      }
    }
    tl.set_base(xb);
    tl.propagate(dx, 2.0, 2, mdx);
    tl.adjoint(dy, 2.0, 2, mtdy);
    double lhs = 0.0, rhs = 0.0;
    for (int q = 0; q < 12; ++q)
      for (size_t e = 0; e < dx[q].size(); ++e) {
        lhs += mdx[q][e] * dy[q][e];
        rhs += dx[q][e] * mtdy[q][e];
      }
    std::printf("dot test: %.15e %.15e\n", lhs, rhs);
    const double rel = std::fabs(lhs - rhs) / std::fmax(std::fabs(lhs), std::fabs(rhs));
    std::fclose(out);
    return rel < 1e-10 ? 0 : 3;
  } catch (const std::exception& e) {
    std::fprintf(stderr, "error: %s\n", e.what());
    std::fclose(out);
    return 1;
  }
}
