// oracle/ref/ref_driver.cpp -- TEST INFRASTRUCTURE ONLY.
//
// C entry points (vref_*, declared in oracle/vibe_oracle.h) over the
// reference's own compiled classes: grid::Grid, dyn::ReferenceState,
// dyn::State, dyn::Equations, dyn::Advection, dyn::Damping,
// timeint::AcousticSubstepper and driver::init_warm_bubble. Built by
// oracle/Makefile (target `ref`) into oracle/_ref/ only.
//
// Restated glue (the reference's versions do not compile, see the notes):
//   * vref_rk3_step follows RungeKutta3Integrator::step
//     (src/time/runge_kutta.cpp:77-119). The shipped code calls
//     State::add_scaled(Real, const Tendency&), which does not exist
//     (runge_kutta.cpp:92 vs include/vibe/dyn/state.hpp:137-139); here that
//     update is expanded field by field over the 12 species.
//   * the acoustic substep follows runge_kutta.cpp:65-75 verbatim.
//   * vref_si_step follows SemiImplicitIntegrator::step and assemble_rhs
//     (src/time/semi_implicit.cpp:56-106,167-226), which do not compile
//     (the same State::add_scaled(Real, Tendency) call, :182); the solve is
//     the reference's own HelmholtzSolver from make_helmholtz_solver.
//   * weno_scalars=1 replaces the non-conservative scalar advection of theta
//     and the moisture species (src/dyn/equations.cpp:129-137) with
//     Advection::scalar in WENO5 flux form (src/dyn/advection.cpp:144-187)
//     and re-applies the positivity clip (equations.cpp:139-149).
//   * the composition flags of vo_setup (pgf_perturbation, split_fast,
//     weno_advective, acoustic_mode 0/1/2, hevi_beta, w_rigid) are composed
//     from the reference's own operators (Equations::tendencies,
//     Equations::acoustic_tendencies, Advection::scalar,
//     AcousticSubstepper::step, timeint::thomas_solve): see slow_tendency,
//     acoustic_substep and consistent_hevi_substep below. This is an
//     independent second statement of the flags the plain-C oracle restates.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../vibe_oracle.h"
#include "vibe/common/constants.hpp"
#include "vibe/config/config.hpp"
#include "vibe/driver/initial_conditions.hpp"
#include "vibe/dyn/advection.hpp"
#include "vibe/dyn/diagnostics.hpp"
#include "vibe/dyn/equations.hpp"
#include "vibe/dyn/reference_state.hpp"
#include "vibe/dyn/state.hpp"
#include "vibe/io/field_io.hpp"
#include "vibe/dyn/tendency.hpp"
#include "vibe/grid/decomposition.hpp"
#include "vibe/grid/geometry.hpp"
#include "vibe/time/acoustic_substep.hpp"
#include "vibe/physics/microphysics.hpp"
#include "vibe/time/helmholtz.hpp"
#include "vibe/grid/nest.hpp"
#include "vibe/da/tangent_linear.hpp"

using namespace vibe;

struct vref_model {
  vo_setup setup{};
  config::ModelConfig cfg;
  std::unique_ptr<grid::Grid> grid;
  std::unique_ptr<dyn::ReferenceState> ref;
  std::unique_ptr<dyn::State> state;
  std::unique_ptr<dyn::Equations> eq;
  std::unique_ptr<dyn::Advection> weno;
  std::unique_ptr<dyn::Tendency> slow, scratch;
};

namespace {

const char* advection_name(int a) {
  switch (a) {
    case 4: return "central4";
    case 6: return "central6";
    case 5: return "weno5";
    default: return "central2";
  }
}

const grid::Field<Real>& reffield(const vref_model* m, int which) {
  switch (which) {
    case VO_THETA0: return m->ref->theta0();
    case VO_PI0: return m->ref->pi0();
    case VO_RHO0: return m->ref->rho0();
    case VO_P0: return m->ref->p0();
    default: return m->ref->qv0();
  }
}

// The state the pressure-gradient terms see: with pgf_perturbation = 1 a
// copy whose Exner field holds pi' = pi - pi0 (every other field as given),
// so Equations::tendencies / acoustic_tendencies (equations.cpp:70-110,
// 157-185) difference pi' instead of the total Exner function.
dyn::State pgf_view(const vref_model* m, const dyn::State& s) {
  dyn::State v = s.clone();
  if (m->setup.pgf_perturbation) {
    auto& p = v.pi().storage();
    const auto& p0 = m->ref->pi0().storage();
    for (Size e = 0; e < p.size(); ++e) p[e] = p[e] - p0[e];
  }
  return v;
}

// Slow tendency of the composition the setup selects, built from the
// reference's own operators only:
//   * Equations::tendencies (equations.cpp:60-150) on pgf_view(s); the
//     divergence damping of pi (damping.cpp:43-74, the only writer of the pi
//     tendency there) keeps acting on the total Exner function;
//   * weno_scalars: Advection::scalar in WENO5 flux form (advection.cpp:144-187)
//     for theta and the moisture species, then the positivity clip again
//     (equations.cpp:139-149);
//   * weno_advective: + q div(u). Advection::scalar of a field of ones is
//     exactly -div(u) with the same face winds, spacings and vertical-flux
//     condition (every WENO5 candidate of a constant is the constant, so the
//     face flux is the face wind), so q div(u) = q * (-scalar(1));
//   * split_fast: minus Equations::acoustic_tendencies (equations.cpp:152-209)
//     of the same state for u, v, w and rho.
void slow_tendency(vref_model* m, dyn::State& s, dyn::Tendency& d) {
  const grid::Grid& g = *m->grid;
  const dyn::State v = pgf_view(m, s);
  m->eq->tendencies(v, d);
  if (m->setup.pgf_perturbation && m->setup.divergence_damping > 0.0) {
    m->eq->tendencies(s, *m->scratch);
    d.pi().storage() = m->scratch->pi().storage();
  }
  if (m->setup.weno_scalars) {
    grid::Field<Real> negdiv(g, grid::Stagger::Cell, "negdiv");
    if (m->setup.weno_advective) {
      grid::Field<Real> ones(g, grid::Stagger::Cell, "ones");
      ones.fill(Real(1));
      m->weno->scalar(ones, s.u(), s.v(), s.w(), s.rho(), negdiv);
    }
    const int last = m->setup.moist ? static_cast<int>(dyn::Species::Qg)
                                    : static_cast<int>(dyn::Species::Qv);
    for (int sp = static_cast<int>(dyn::Species::Theta); sp <= last; ++sp) {
      if (sp == static_cast<int>(dyn::Species::Pi)) continue;
      const auto species = static_cast<dyn::Species>(sp);
      const grid::Field<Real>& q = s.field(species);
      grid::Field<Real>& dq = d.field(species);
      m->weno->scalar(q, s.u(), s.v(), s.w(), s.rho(), dq);
      if (!m->setup.weno_advective) continue;
      for (Int k = 0; k < g.nz(); ++k)
        for (Int j = 0; j < g.ny(); ++j)
          for (Int i = 0; i < g.nx(); ++i) dq(i, j, k) += q(i, j, k) * -negdiv(i, j, k);
    }
    for (int sp = static_cast<int>(dyn::Species::Qv); sp <= static_cast<int>(dyn::Species::Qg); ++sp) {
      const auto species = static_cast<dyn::Species>(sp);
      const grid::Field<Real>& q = s.field(species);
      grid::Field<Real>& dq = d.field(species);
      for (Int k = 0; k < g.nz(); ++k)
        for (Int j = 0; j < g.ny(); ++j)
          for (Int i = 0; i < g.nx(); ++i)
            if (q(i, j, k) <= Real(0) && dq(i, j, k) < Real(0)) dq(i, j, k) = Real(0);
    }
  }
  if (m->setup.split_fast) {
    m->eq->acoustic_tendencies(v, *m->scratch);
    const dyn::Species fast[4] = {dyn::Species::U, dyn::Species::V, dyn::Species::W, dyn::Species::Rho};
    for (const auto sp : fast) {
      auto& t = d.field(sp).storage();
      const auto& f = m->scratch->field(sp).storage();
      for (Size e = 0; e < t.size(); ++e) t[e] -= f[e];
    }
  }
}

// RungeKutta3Integrator::acoustic_substep (runge_kutta.cpp:65-75): forward
// rho/pi, then u/v/w from the updated pressure (through pgf_view).
void acoustic_substep(vref_model* m, dyn::State& s, Real dtau) {
  dyn::Tendency& sc = *m->scratch;
  m->eq->acoustic_tendencies(pgf_view(m, s), sc);
  s.rho().add_scaled(dtau, sc.rho());
  s.pi().add_scaled(dtau, sc.pi());
  m->eq->acoustic_tendencies(pgf_view(m, s), sc);
  s.u().add_scaled(dtau, sc.u());
  s.v().add_scaled(dtau, sc.v());
  s.w().add_scaled(dtau, sc.w());
}

// The vertically implicit substep of docs/design/04_time_integration.md
// sec. 2.4 (Crank-Nicolson weight b = hevi_beta on the vertical acoustic
// terms, explicit horizontal terms), assembled from the reference's linear
// acoustic operator alone. With A(u, v, w, x) = Equations::acoustic_tendencies
// of a state with winds (u, v, w) and Exner field x (pi', or total pi when
// pgf_perturbation = 0):
//   W(x)  = A(0, 0, 0, x).w          vertical pressure gradient on w faces
//   R(..) = A(.., .., .., 0).rho     mass divergence, P(..) = A(..).pi its pi rate
//   w~    = w + dtau (1-b) W(x_old)
//   pi*   = pi + dtau [P(u,v,0) + (1-b) P(0,0,w) + b P(0,0,w~)]
//   (I - (dtau b)^2 L) x = pi* - pi0 (or pi*),  L x = P(0, 0, W(x))
//   w_new = w~ + dtau b W(x),  rho_new = rho + dtau [R(u,v,0) + (1-b) R(0,0,w) + b R(0,0,w_new)]
//   pi_new = x + pi0 (or x),   u, v += dtau A(., ., ., x).u/.v
// L is read off the reference operator itself: it couples levels of one
// column only and is tridiagonal, so three probes (x = 1 on the levels
// k = r mod 3) give every column's three diagonals. Each column is solved
// with timeint::thomas_solve (helmholtz.cpp:57-86).
void consistent_hevi_substep(vref_model* m, dyn::State& s, Real dtau) {
  const grid::Grid& g = *m->grid;
  const Int nx = g.nx(), ny = g.ny(), nz = g.nz();
  const Real b = m->setup.hevi_beta, ob = Real(1) - b;
  const bool pert = m->setup.pgf_perturbation != 0;
  const auto& pi0 = m->ref->pi0();
  dyn::State a(g);
  a.set_reference(m->ref.get());
  dyn::Tendency t(g);
  auto zero_winds = [&]() {
    a.u().fill(Real(0));
    a.v().fill(Real(0));
    a.w().fill(Real(0));
  };
  // x_old and W(x_old)
  grid::Field<Real> x(g, grid::Stagger::Cell, "x");
  for (Size e = 0; e < x.storage().size(); ++e)
    x.storage()[e] = s.pi().storage()[e] - (pert ? pi0.storage()[e] : Real(0));
  zero_winds();
  a.pi() = x;
  m->eq->acoustic_tendencies(a, t);
  grid::Field<Real> wt = s.w();
  wt.add_scaled(dtau * ob, t.w());
  // horizontal and vertical mass divergences and their pi rates
  a.pi().fill(Real(0));
  a.u() = s.u();
  a.v() = s.v();
  m->eq->acoustic_tendencies(a, t);
  const grid::Field<Real> rh = t.rho(), ph = t.pi();
  zero_winds();
  a.w() = s.w();
  m->eq->acoustic_tendencies(a, t);
  const grid::Field<Real> rv_old = t.rho(), pv_old = t.pi();
  a.w() = wt;
  m->eq->acoustic_tendencies(a, t);
  const grid::Field<Real> pv_t = t.pi();
  // L = P(0, 0, W(.)) probed per level colour
  std::vector<grid::Field<Real>> probe;
  for (int r = 0; r < 3; ++r) {
    zero_winds();
    a.pi().fill(Real(0));
    for (Int k = r; k < nz; k += 3)
      for (Int j = 0; j < ny; ++j)
        for (Int i = 0; i < nx; ++i) a.pi()(i, j, k) = Real(1);
    m->eq->acoustic_tendencies(a, t);
    a.w() = t.w();
    a.pi().fill(Real(0));
    m->eq->acoustic_tendencies(a, t);
    probe.push_back(t.pi());
  }
  const Real c2 = (dtau * b) * (dtau * b);
  std::vector<Real> ta(static_cast<Size>(nz > 1 ? nz - 1 : 0)), tb(static_cast<Size>(nz)),
      tc(static_cast<Size>(nz > 1 ? nz - 1 : 0)), rhs(static_cast<Size>(nz)), sol;
  for (Int j = 0; j < ny; ++j)
    for (Int i = 0; i < nx; ++i) {
      for (Int k = 0; k < nz; ++k) {
        tb[k] = Real(1) - c2 * probe[k % 3](i, j, k);
        if (k > 0) ta[k - 1] = -c2 * probe[(k - 1) % 3](i, j, k);
        if (k + 1 < nz) tc[k] = -c2 * probe[(k + 1) % 3](i, j, k);
        const Real pstar = s.pi()(i, j, k) + dtau * (ph(i, j, k) + ob * pv_old(i, j, k) + b * pv_t(i, j, k));
        rhs[k] = pstar - (pert ? pi0(i, j, k) : Real(0));
      }
      timeint::thomas_solve(ta, tb, tc, rhs, sol);
      for (Int k = 0; k < nz; ++k) x(i, j, k) = sol[k];
    }
  // w_new = w~ + dtau b W(x); the mass update with it
  zero_winds();
  a.pi() = x;
  m->eq->acoustic_tendencies(a, t);
  const grid::Field<Real> ux = t.u(), vx = t.v();
  grid::Field<Real> wn = wt;
  wn.add_scaled(dtau * b, t.w());
  a.pi().fill(Real(0));
  a.w() = wn;
  m->eq->acoustic_tendencies(a, t);
  for (Int k = 0; k < nz; ++k)
    for (Int j = 0; j < ny; ++j)
      for (Int i = 0; i < nx; ++i) {
        s.rho()(i, j, k) += dtau * (rh(i, j, k) + ob * rv_old(i, j, k) + b * t.rho()(i, j, k));
        s.pi()(i, j, k) = x(i, j, k) + (pert ? pi0(i, j, k) : Real(0));
      }
  s.w() = wn;
  // horizontal momentum, backward with the new pressure
  s.u().add_scaled(dtau, ux);
  s.v().add_scaled(dtau, vx);
}

void hevi_substep(vref_model* m, dyn::State& s, Real dtau) {
  if (m->setup.acoustic_mode == 1) {
    timeint::AcousticOptions opt;
    opt.vertical_implicit = true;
    timeint::AcousticSubstepper sub(*m->grid, opt);
    sub.step(s, dtau, *m->ref);
  } else {
    consistent_hevi_substep(m, s, dtau);
  }
}

}  // namespace

extern "C" {

vref_model* vref_create(const vo_setup* su) {
  auto* m = new vref_model();
  m->setup = *su;
  grid::Geometry geo;
  geo.nx = su->nx;
  geo.ny = su->ny;
  geo.nz = su->nz;
  geo.dx = su->dx;
  geo.dy = su->dy;
  geo.z_top = su->z_top;
  geo.zeta = grid::make_stretched_zeta(su->nz, su->zeta_first, su->zeta_stretch);
  if (su->terrain_kind == 1) {
    geo.zs.assign(static_cast<Size>(su->nx) * static_cast<Size>(su->ny), Real(0));
    for (Int j = 0; j < su->ny; ++j)
      for (Int i = 0; i < su->nx; ++i) {
        const Real x = (static_cast<Real>(i) + Real(0.5)) * su->dx - su->hill_xc;
        const Real y = (static_cast<Real>(j) + Real(0.5)) * su->dy - su->hill_yc;
        geo.zs[static_cast<Size>(j) * su->nx + i] =
            su->hill_h * std::exp(-(x * x + y * y) / (su->hill_a * su->hill_a));
      }
  }
  geo.name = "oracle";
  auto dec = grid::Decomposition::make(su->nx, su->ny, su->nz, 1, 1, VO_HALO, false, false);
  m->grid = std::make_unique<grid::Grid>(geo, dec);
  const grid::Grid& g = *m->grid;

  if (su->ref_kind == 1) {
    std::vector<Real> z, th;
    const int np = static_cast<int>(std::ceil(su->z_top / su->profile_dz)) + 2;
    for (int p = 0; p < np; ++p) {
      const Real zz = static_cast<Real>(p) * su->profile_dz;
      z.push_back(zz);
      th.push_back(su->theta0 * std::exp(su->bv_n * su->bv_n * zz / kGravity));
    }
    m->ref = std::make_unique<dyn::ReferenceState>(
        dyn::ReferenceState::from_profile(g, z, th, su->p_surf));
  } else {
    m->ref = std::make_unique<dyn::ReferenceState>(
        dyn::ReferenceState::isothermal(g, su->theta0, su->p_surf));
  }

  auto& c = m->cfg;
  c.numerics.advection = advection_name(su->advection);
  c.numerics.flux_form = true;
  c.numerics.coriolis = su->coriolis == 0 ? "none" : (su->coriolis == 2 ? "betaplane" : "fplane");
  c.numerics.fplane_latitude = su->latitude;
  c.numerics.sponge_alpha = su->sponge_alpha;
  c.numerics.sponge_start_fraction = su->sponge_start_fraction;
  c.numerics.divergence_damping = su->divergence_damping;
  c.numerics.divergence_order = su->divergence_order;
  c.physics.microphysics = su->moist ? "kessler" : "none";
  m->eq = std::make_unique<dyn::Equations>(g, *m->ref, c);
  m->weno = std::make_unique<dyn::Advection>(g, dyn::AdvectionScheme::WENO5, true);
  m->slow = std::make_unique<dyn::Tendency>(g);
  m->scratch = std::make_unique<dyn::Tendency>(g);

  m->state = std::make_unique<dyn::State>(g);
  m->state->set_reference(m->ref.get());
  driver::IcOptions opt;
  opt.bubble_amplitude = su->bubble_amplitude;
  opt.bubble_radius_x = su->bubble_radius_x;
  opt.bubble_radius_z = su->bubble_radius_z;
  opt.bubble_xc = su->bubble_xc;
  opt.bubble_yc = su->bubble_yc;
  opt.bubble_zc = su->bubble_zc;
  opt.qv_surface = su->qv_surface;
  opt.qv_decay_height = su->qv_decay_height;
  opt.u_background = su->u_background;
  opt.shear_u = su->shear_u;
  driver::init_warm_bubble(g, *m->ref, *m->state, opt);
  return m;
}

void vref_destroy(vref_model* m) { delete m; }

size_t vref_storage_size(const vref_model* m, int species) {
  return m->state->field(static_cast<dyn::Species>(species)).size();
}

void vref_get_field(const vref_model* m, int species, double* out) {
  const auto& f = m->state->field(static_cast<dyn::Species>(species)).storage();
  std::memcpy(out, f.data(), f.size() * sizeof(double));
}

void vref_set_field(vref_model* m, int species, const double* in) {
  auto& f = m->state->field(static_cast<dyn::Species>(species)).storage();
  std::memcpy(f.data(), in, f.size() * sizeof(double));
}

void vref_get_reffield(const vref_model* m, int which, double* out) {
  const auto& f = reffield(m, which).storage();
  std::memcpy(out, f.data(), f.size() * sizeof(double));
}

void vref_get_zeta(const vref_model* m, double* out) {
  const auto& z = m->grid->geom().zeta;
  std::memcpy(out, z.data(), z.size() * sizeof(double));
}

void vref_get_terrain(const vref_model* m, double* out) {
  const grid::Grid& g = *m->grid;
  for (Int j = 0; j < g.ny(); ++j)
    for (Int i = 0; i < g.nx(); ++i) out[static_cast<Size>(j) * g.nx() + i] = g.terrain(i, j);
}

void vref_get_sponge(const vref_model* m, double* out) {
  const auto& sp = m->eq->damping().sponge_profile();
  std::memcpy(out, sp.data(), sp.size() * sizeof(double));
}

int vref_rk3_step(vref_model* m, double dt, int n_sub_in) {
  dyn::State& s = *m->state;
  const int n_sub = std::max(n_sub_in, 1);
  const dyn::State s0 = s.clone();
  const Real dt_stage[3] = {dt / Real(3), dt / Real(2), dt};
  for (int stage = 0; stage < 3; ++stage) {
    slow_tendency(m, s, *m->slow);
    s = s0;
    for (int sp = 0; sp < dyn::kNumSpecies; ++sp) {
      const auto species = static_cast<dyn::Species>(sp);
      s.field(species).add_scaled(dt_stage[stage], m->slow->field(species));
    }
    const Real dtau_stage = dt_stage[stage] / static_cast<Real>(n_sub);
    for (int n = 0; n < n_sub; ++n) {
      if (m->setup.acoustic_mode == 0)
        acoustic_substep(m, s, dtau_stage);
      else
        hevi_substep(m, s, dtau_stage);
    }
    if (s.has_nonfinite()) return 1;
  }
  m->eq->damping().apply_sponge(s, *m->ref, dt);
  if (m->setup.w_rigid) {
    const grid::Grid& g = *m->grid;
    for (Int j = 0; j < g.ny(); ++j)
      for (Int i = 0; i < g.nx(); ++i) {
        s.w()(i, j, 0) = Real(0);
        s.w()(i, j, g.nz()) = Real(0);
      }
  }
  s.step += 1;
  return 0;
}

void vref_slow_tendency(vref_model* m, double* const* out) {
  slow_tendency(m, *m->state, *m->slow);
  for (int sp = 0; sp < dyn::kNumSpecies; ++sp) {
    const auto& f = m->slow->field(static_cast<dyn::Species>(sp)).storage();
    std::memcpy(out[sp], f.data(), f.size() * sizeof(double));
  }
}

void vref_acoustic_substep(vref_model* m, double dtau) { acoustic_substep(m, *m->state, dtau); }

void vref_hevi_substep(vref_model* m, double dtau) { hevi_substep(m, *m->state, dtau); }

void vref_sponge(vref_model* m, double dt) {
  m->eq->damping().apply_sponge(*m->state, *m->ref, dt);
}

namespace {
grid::Field<Real> cell_field(const grid::Grid& g, const double* p, const char* name) {
  grid::Field<Real> f(g, grid::Stagger::Cell, name);
  if (p != nullptr) std::memcpy(f.storage().data(), p, f.storage().size() * sizeof(double));
  return f;
}
int solve_with(vref_model* m, int kind, int max_iter, double tol, int refine, const grid::Field<Real>& a,
               const grid::Field<Real>& b, const grid::Field<Real>& f, grid::Field<Real>& x, int* iterations,
               double* residual) {
  config::ModelConfig cfg = m->cfg;
  cfg.numerics.helmholtz_max_iter = max_iter;
  cfg.numerics.helmholtz_tol = tol;
  auto solver = timeint::make_helmholtz_solver(static_cast<timeint::HelmholtzKind>(kind), *m->grid, cfg);
  solver->set_iterative_refinement(refine != 0, gpu::Precision::FP64);
  solver->set_coefficients(a, b);
  try {
    solver->solve(a, b, f, x);
  } catch (const std::exception&) {
    return 1;
  }
  if (iterations) *iterations = solver->iterations();
  if (residual) *residual = solver->residual();
  return 0;
}
}  // namespace

void vref_helmholtz_apply_norm(vref_model* m, const double* a, const double* b, const double* f,
                               const double* x, double* out) {
  const grid::Grid& g = *m->grid;
  *out = timeint::helmholtz_residual_l2(g, cell_field(g, a, "a"), cell_field(g, b, "b"), cell_field(g, f, "f"),
                                        cell_field(g, x, "x"));
}

int vref_helmholtz_solve(vref_model* m, int kind, int max_iter, double tol, int refine, const double* a,
                         const double* b, const double* f, double* x, int* iterations, double* residual) {
  const grid::Grid& g = *m->grid;
  grid::Field<Real> fx = cell_field(g, nullptr, "x");
  const int rc = solve_with(m, kind, max_iter, tol, refine, cell_field(g, a, "a"), cell_field(g, b, "b"),
                            cell_field(g, f, "f"), fx, iterations, residual);
  std::memcpy(x, fx.storage().data(), fx.storage().size() * sizeof(double));
  return rc;
}

void vref_multigrid_restrict(vref_model* m, const double* fine, double* coarse) {
  const grid::Grid& g = *m->grid;
  grid::Field<Real> c = cell_field(g, nullptr, "c");
  timeint::multigrid_restrict(cell_field(g, fine, "f"), c);
  std::memcpy(coarse, c.storage().data(), c.storage().size() * sizeof(double));
}

void vref_multigrid_prolong(vref_model* m, const double* coarse, double* fine) {
  const grid::Grid& g = *m->grid;
  grid::Field<Real> f = cell_field(g, nullptr, "f");
  timeint::multigrid_prolong(cell_field(g, coarse, "c"), f);
  std::memcpy(fine, f.storage().data(), f.storage().size() * sizeof(double));
}

int vref_si_step(vref_model* m, double dt, int kind, int max_iter, double tol, int* iterations,
                 double* residual, double* pi_new, double* rhs_out, double* a_out) {
  const grid::Grid& g = *m->grid;
  const dyn::ReferenceState& ref = *m->ref;
  dyn::State& s = *m->state;
  dyn::Tendency& n = *m->slow;
  slow_tendency(m, s, n);
  const Int nx = g.nx(), ny = g.ny(), nz = g.nz();
  const Real half_dt = Real(0.5) * dt;
  grid::Field<Real> acoef = cell_field(g, nullptr, "a_coef"), bcoef = cell_field(g, nullptr, "b_coef");
  grid::Field<Real> rhs = cell_field(g, nullptr, "rhs"), x = cell_field(g, nullptr, "pi_new");
  for (Int k = 0; k < nz; ++k)
    for (Int j = 0; j < ny; ++j)
      for (Int i = 0; i < nx; ++i) {
        acoef(i, j, k) = half_dt * half_dt * (kRd / kCv) * ref.pi0()(i, j, k) * kCp * ref.theta0()(i, j, k);
        bcoef(i, j, k) = Real(1);
      }
  for (Int k = 0; k < nz; ++k)
    for (Int j = 0; j < ny; ++j)
      for (Int i = 0; i < nx; ++i) {
        const Real dx = g.dx_at(i), dy = g.dy_at(j);
        const Real scale = g.geom().z_top - g.terrain(i, j);
        const Real dz = std::max(g.dzeta(k) * scale, Real(1));
        const auto& r0 = ref.rho0();
        auto flux_div = [&](const grid::Field<Real>& u, const grid::Field<Real>& v, const grid::Field<Real>& w) {
          const Real fx = u(i + 1, j, k) * Real(0.5) * (r0(i, j, k) + r0(std::min(i + 1, nx - 1), j, k)) -
                          u(i, j, k) * Real(0.5) * (r0(std::max(i - 1, Int(0)), j, k) + r0(i, j, k));
          const Real fy = v(i, j + 1, k) * Real(0.5) * (r0(i, j, k) + r0(i, std::min(j + 1, ny - 1), k)) -
                          v(i, j, k) * Real(0.5) * (r0(i, std::max(j - 1, Int(0)), k) + r0(i, j, k));
          const Real fz = w(i, j, k + 1) * Real(0.5) * (r0(i, j, k) + r0(i, j, std::min(k + 1, nz - 1))) -
                          w(i, j, k) * Real(0.5) * (r0(i, j, std::max(k - 1, Int(0))) + r0(i, j, k));
          return fx / dx + fy / dy + fz / dz;
        };
        const Real G = flux_div(s.u(), s.v(), s.w()) + half_dt * flux_div(n.u(), n.v(), n.w());
        const Real c = (kRd / kCv) * (ref.pi0()(i, j, k) / std::max(ref.rho0()(i, j, k), Real(1e-8)));
        const Real a0 = acoef(i, j, k);
        const auto& pi = s.pi();
        const Real div_a_grad =
            (a0 * (pi(std::min(i + 1, nx - 1), j, k) - pi(i, j, k)) -
             a0 * (pi(i, j, k) - pi(std::max(i - 1, Int(0)), j, k))) / (dx * dx) +
            (a0 * (pi(i, std::min(j + 1, ny - 1), k) - pi(i, j, k)) -
             a0 * (pi(i, j, k) - pi(i, std::max(j - 1, Int(0)), k))) / (dy * dy);
        rhs(i, j, k) = pi(i, j, k) - dt * c * G + div_a_grad;
      }
  const int rc = solve_with(m, kind, max_iter, tol, 1, acoef, bcoef, rhs, x, iterations, residual);
  if (pi_new) std::memcpy(pi_new, x.storage().data(), x.storage().size() * sizeof(double));
  if (rhs_out) std::memcpy(rhs_out, rhs.storage().data(), rhs.storage().size() * sizeof(double));
  if (a_out) std::memcpy(a_out, acoef.storage().data(), acoef.storage().size() * sizeof(double));
  if (rc) return 2;
  s.theta().add_scaled(dt, n.theta());
  s.qv().add_scaled(dt, n.qv());
  s.rho().add_scaled(dt, n.rho());
  for (int sp = static_cast<int>(dyn::Species::Qc); sp <= static_cast<int>(dyn::Species::Qg); ++sp) {
    const auto species = static_cast<dyn::Species>(sp);
    s.field(species).add_scaled(dt, n.field(species));
  }
  m->eq->damping().apply_sponge(s, ref, dt);
  return s.has_nonfinite() ? 1 : 0;
}


namespace {
grid::Grid plain_grid(int nx, int ny, int nz) {
  grid::Geometry geo;
  geo.nx = nx;
  geo.ny = ny;
  geo.nz = nz;
  geo.dx = 1.0;
  geo.dy = 1.0;
  geo.z_top = 1.0;
  geo.zeta = grid::make_stretched_zeta(nz, 1.0, 1.0);
  geo.name = "nest";
  return grid::Grid(geo, grid::Decomposition::make(nx, ny, nz, 1, 1, VO_HALO, false, false));
}
grid::Stagger stagger_of(int s) {
  return s == 1 ? grid::Stagger::FaceX : s == 2 ? grid::Stagger::FaceY : s == 3 ? grid::Stagger::FaceZ
                                                                               : grid::Stagger::Cell;
}
std::vector<grid::Field<Real>> fields_of(const grid::Grid& g, int nvars, const int* stagger, const double* const* p) {
  std::vector<grid::Field<Real>> fs;
  for (int v = 0; v < nvars; ++v) {
    fs.emplace_back(g, stagger_of(stagger[v]), "f");
    std::memcpy(fs.back().storage().data(), p[v], fs.back().storage().size() * sizeof(double));
  }
  return fs;
}
void copy_out(std::vector<grid::Field<Real>>& fs, double* const* p) {
  for (size_t v = 0; v < fs.size(); ++v)
    std::memcpy(p[v], fs[v].storage().data(), fs[v].storage().size() * sizeof(double));
}
std::vector<grid::Field<Real>*> ptrs(std::vector<grid::Field<Real>>& fs) {
  std::vector<grid::Field<Real>*> out;
  for (auto& f : fs) out.push_back(&f);
  return out;
}
grid::NestPlacement placement_of(const vo_nest_placement* p) {
  grid::NestPlacement q;
  q.i0 = p->i0;
  q.j0 = p->j0;
  q.k0 = p->k0;
  q.iext = p->iext;
  q.jext = p->jext;
  q.ratio = p->ratio;
  q.boundary_zone = p->boundary_zone;
  return q;
}
}  // namespace

void vref_davies_profile(int n_zone, double alpha_max, double* out) {
  const auto a = grid::davies_profile(n_zone, alpha_max);
  std::memcpy(out, a.data(), a.size() * sizeof(double));
}

void vref_nest_interpolate_from_parent(const vo_nest_placement* p, int nvars, const int* stagger, int pnx, int pny,
                                       int pnz, const double* const* parent, int cnx, int cny, int cnz,
                                       double* const* child) {
  grid::Grid pg = plain_grid(pnx, pny, pnz), cg = plain_grid(cnx, cny, cnz);
  grid::Nest nest(cg, pg, placement_of(p));
  auto pf = fields_of(pg, nvars, stagger, parent);
  auto cf = fields_of(cg, nvars, stagger, child);
  auto pp = ptrs(pf);
  auto cp = ptrs(cf);
  nest.interpolate_from_parent(pp, cp);
  copy_out(cf, child);
}

void vref_nest_restrict_to_parent(const vo_nest_placement* p, int nvars, const int* stagger, int cnx, int cny,
                                  int cnz, const double* const* child, int pnx, int pny, int pnz,
                                  double* const* parent) {
  grid::Grid pg = plain_grid(pnx, pny, pnz), cg = plain_grid(cnx, cny, cnz);
  grid::Nest nest(cg, pg, placement_of(p));
  auto pf = fields_of(pg, nvars, stagger, parent);
  auto cf = fields_of(cg, nvars, stagger, child);
  auto pp = ptrs(pf);
  auto cp = ptrs(cf);
  nest.restrict_to_parent(cp, pp);
  copy_out(pf, parent);
}

void vref_nest_apply_lateral_boundary(const vo_nest_placement* p, int nvars, const int* stagger, int cnx, int cny,
                                      int cnz, double* const* child, const double* const* parent_interp) {
  grid::Grid cg = plain_grid(cnx, cny, cnz);
  grid::Nest nest(cg, cg, placement_of(p));
  auto cf = fields_of(cg, nvars, stagger, child);
  auto pf = fields_of(cg, nvars, stagger, parent_interp);
  auto cp = ptrs(cf);
  auto pp = ptrs(pf);
  nest.apply_lateral_boundary(cp, pp);
  copy_out(cf, child);
}


namespace {
void load_state(dyn::State& st, const double* const* p) {
  for (int sp = 0; sp < dyn::kNumSpecies; ++sp) {
    auto& f = st.field(static_cast<dyn::Species>(sp)).storage();
    std::memcpy(f.data(), p[sp], f.size() * sizeof(double));
  }
}
void store_state(const dyn::State& st, double* const* p) {
  for (int sp = 0; sp < dyn::kNumSpecies; ++sp) {
    const auto& f = st.field(static_cast<dyn::Species>(sp)).storage();
    std::memcpy(p[sp], f.data(), f.size() * sizeof(double));
  }
}
void store_tend(const dyn::Tendency& t, double* const* p) {
  for (int sp = 0; sp < dyn::kNumSpecies; ++sp) {
    const auto& f = t.field(static_cast<dyn::Species>(sp)).storage();
    std::memcpy(p[sp], f.data(), f.size() * sizeof(double));
  }
}
}  // namespace

void vref_tl_step(vref_model* m, const double* const* xb, const double* const* dx, double dt, double* const* out) {
  const grid::Grid& g = *m->grid;
  config::DaConfig da;
  da::TangentLinearModel tl(g, *m->ref, m->cfg, da);
  dyn::State sxb(g), sdx(g), sout(g);
  load_state(sxb, xb);
  load_state(sdx, dx);
  tl.step(sxb, sdx, dt, sout);
  store_state(sout, out);
}

void vref_ad_step(vref_model* m, const double* const* xb, const double* const* bar_out, double dt,
                  double* const* bar_in) {
  const grid::Grid& g = *m->grid;
  config::DaConfig da;
  da::AdjointModel ad(g, *m->ref, m->cfg, da);
  dyn::State sxb(g), sbo(g), sbi(g);
  load_state(sxb, xb);
  load_state(sbo, bar_out);
  ad.step_adjoint(sxb, sbo, dt, sbi);
  store_state(sbi, bar_in);
}

void vref_tl_propagate(vref_model* m, const double* const* xb, const double* const* dx0, double dt, int n_steps,
                       double* const* out) {
  const grid::Grid& g = *m->grid;
  config::DaConfig da;
  da::TangentLinearModel tl(g, *m->ref, m->cfg, da);
  dyn::State sxb(g), sdx(g), sout(g);
  load_state(sxb, xb);
  load_state(sdx, dx0);
  tl.propagate(sxb, sdx, dt, n_steps, sout);
  store_state(sout, out);
}

void vref_ad_propagate(vref_model* m, const double* const* xb, const double* const* dy, double dt, int n_steps,
                       double* const* out) {
  const grid::Grid& g = *m->grid;
  config::DaConfig da;
  da::TangentLinearModel tl(g, *m->ref, m->cfg, da);
  da::AdjointModel ad(g, *m->ref, m->cfg, da);
  dyn::State sxb(g), sdy(g), sout(g), scratch(g);
  load_state(sxb, xb);
  load_state(sdy, dy);
  tl.record_trajectory(sxb, dt, n_steps);
  ad.propagate_with_trajectory(tl.trajectory(), sdy, sout);
  store_state(sout, out);
}


void vref_cfl(vref_model* m, double dt, double dtau, double* adv_cfl, double* max_sound_speed,
              double* acoustic_cfl) {
  const dyn::State& s = *m->state;
  if (adv_cfl) *adv_cfl = m->eq->advection().cfl_number(s, dt);
  if (max_sound_speed) *max_sound_speed = m->eq->max_sound_speed(s);
  if (acoustic_cfl) {
    timeint::AcousticOptions opt;
    timeint::AcousticSubstepper sub(*m->grid, opt);
    *acoustic_cfl = sub.acoustic_cfl(s, dtau);
  }
}

// RungeKutta3Integrator::max_stable_dt (runge_kutta.cpp:121-140) restated: the
// translation unit does not compile (see vref_rk3_step)
double vref_max_stable_dt(vref_model* m) {
  const grid::Grid& g = *m->grid;
  const dyn::State& s = *m->state;
  const Real adv_cfl = m->eq->advection().cfl_number(s, Real(1));
  const Real cs = m->eq->max_sound_speed(s);
  Real acoustic_rate = Real(0);
  for (Int k = 0; k < g.nz(); ++k)
    for (Int j = 0; j < g.ny(); ++j)
      for (Int i = 0; i < g.nx(); ++i) {
        const Real scale = g.geom().z_top - g.terrain(i, j);
        const Real dz = std::max(g.dzeta(k) * scale, Real(1));
        acoustic_rate = std::max(acoustic_rate, cs * (Real(1) / g.dx_at(i) + Real(1) / g.dy_at(j) + Real(1) / dz));
      }
  const Real dt_adv = (adv_cfl > Real(0)) ? Real(0.8) / adv_cfl : Real(1e9);
  const Real dt_ac = (acoustic_rate > Real(0)) ? Real(2) / acoustic_rate : Real(1e9);
  return std::min(dt_adv, dt_ac);
}


// io::write_restart / io::read_restart (src/io/field_io.cpp:207-250): the
// .vibebin restart file of the model's state (header time = state time).
int vref_write_restart(vref_model* m, const char* path, double time, int step) {
  try {
    m->state->time = time;
    io::RestartInfo info;
    info.time = time;
    info.step = step;
    io::write_restart(path, *m->state, info);
  } catch (...) {
    return 1;
  }
  return 0;
}

int vref_read_restart(vref_model* m, const char* path, double* time, int* step) {
  try {
    const io::RestartInfo info = io::read_restart(path, *m->state);
    if (time) *time = info.time;
    if (step) *step = info.step;
  } catch (...) {
    return 1;
  }
  return 0;
}


// dyn::energy_budget (src/dyn/diagnostics.cpp:255-277)
void vref_energy_budget(vref_model* m, double* out6) {
  const dyn::EnergyBudget e = dyn::energy_budget(*m->state, *m->ref);
  out6[0] = e.kinetic;
  out6[1] = e.internal;
  out6[2] = e.potential;
  out6[3] = e.latent;
  out6[4] = e.total;
  out6[5] = e.mass;
}

// KesslerMicrophysics::step_column (src/physics/microphysics_kessler.cpp:269-331)
// on a column built like state_to_column leaves it (dz from
// PhysicsColumn::diagnose_layer_depth; qi, qs, qg zero). PhysicsDriver itself
// does not build in the reference tree (pbl_myj.cpp / pbl_ysu.cpp declare
// diagnose_height with another exception specifier, surface_layer.cpp names
// an option PhysicsOptions does not have), so the column step is pinned here
// and state_to_column is restated in the oracle.
double vref_kessler_column(const vo_kessler* k, int n, double dt, const double* z, const double* p,
                           const double* rho, double* theta, double* qv, double* qc, double* qr) {
  physics::PhysicsOptions opt;
  opt.kessler_qc0 = k->qc0;
  opt.kessler_k1 = k->k1;
  opt.kessler_k2 = k->k2;
  opt.kessler_evap_coef = k->evap_coef;
  opt.kessler_rain_a = k->rain_a;
  opt.kessler_rain_b = k->rain_b;
  opt.positive_definite = k->positive_definite != 0;
  physics::KesslerMicrophysics mp(opt);
  physics::PhysicsColumn col;
  col.resize(n);
  for (int s = 0; s < n; ++s) {
    col.z[s] = z[s];
    col.p[s] = p[s];
    col.rho[s] = rho[s];
    col.theta[s] = theta[s];
    col.qv[s] = qv[s];
    col.qc[s] = qc[s];
    col.qr[s] = qr[s];
  }
  col.diagnose_layer_depth();
  physics::PhysicsDiagnostics diag;
  const double precip = mp.step_column(col, dt, diag);
  for (int s = 0; s < n; ++s) {
    theta[s] = col.theta[s];
    qv[s] = col.qv[s];
    qc[s] = col.qc[s];
    qr[s] = col.qr[s];
  }
  return precip;
}

}  // extern "C"
