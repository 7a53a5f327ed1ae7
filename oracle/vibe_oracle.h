/* oracle/vibe_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU oracle for the VIBE-Model dynamics step. Two implementations share this
 * interface:
 *   - vo_*   : oracle/vibe_oracle.c, a plain-C restatement of the reference's
 *              serial FP64 algorithm (each function cites the reference
 *              file:line it follows). Builds anywhere with gcc.
 *   - vref_* : oracle/ref/ref_driver.cpp, linked against the reference's own
 *              sources compiled unchanged (oracle/_ref/libvibe_ref.so).
 *              Only buildable where the reference tree is present.
 * Only tests, the smoke check and bench.py's CPU-baseline leg may use either.
 *
 * Data layout = the reference's grid::FieldT storage (field.hpp:6-11,77-81):
 *   offset(i,j,k) = ((k+h)*nsy + (j+h))*nsx + (i+h), halo h = 4,
 *   nsx = nx+2h (+1 for u), nsy = ny+2h (+1 for v), nsz = nz+2h (+1 for w).
 * Species order = dyn::Species (state.hpp:53-55):
 *   u v w rho theta pi qv qc qr qi qs qg.
 */
#ifndef VIBE_ORACLE_H
#define VIBE_ORACLE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VO_NSPECIES 12
#define VO_HALO 4

enum vo_species { VO_U = 0, VO_V, VO_W, VO_RHO, VO_THETA, VO_PI, VO_QV,
                  VO_QC, VO_QR, VO_QI, VO_QS, VO_QG };

/* Reference-state fields (reference_state.hpp): theta0, pi0, rho0, p0, qv0. */
enum vo_reffield { VO_THETA0 = 0, VO_PI0, VO_RHO0, VO_P0, VO_QV0 };

/* Case description shared by the oracle, the reference-linked driver and the
 * GPU library's set-up code (same field meaning in all three). */
typedef struct vo_setup {
  int nx, ny, nz;
  double dx, dy, z_top;
  /* vertical levels: geometry.cpp:39-60 make_stretched_zeta(nz, first, stretch) */
  double zeta_first, zeta_stretch;
  /* terrain: 0 flat, 1 Gaussian hill h*exp(-r^2/a^2) centred at (hx, hy) */
  int terrain_kind;
  double hill_h, hill_a, hill_xc, hill_yc;
  /* reference state: 0 = ReferenceState::isothermal(theta0, p_surf)
   *                  1 = ReferenceState::from_profile of theta0*exp(N^2 z/g)
   *                      sampled every profile_dz metres up to z_top + profile_dz */
  int ref_kind;
  double theta0, p_surf, bv_n, profile_dz;
  /* warm bubble (initial_conditions.cpp:136-159) + IcOptions defaults */
  double bubble_amplitude, bubble_radius_x, bubble_radius_z;
  double bubble_xc, bubble_yc, bubble_zc;
  double qv_surface, qv_decay_height;
  double u_background, shear_u;
  /* numerics (config.hpp:55-68) */
  int advection;        /* 2, 4, 6 central; 5 = weno5 (falls to 2nd order in
                           scalar_nonconservative, advection.cpp:106-120) */
  int weno_scalars;     /* 1: theta/q use Advection::scalar WENO5 flux form */
  int moist;            /* microphysics != "none" */
  int coriolis;         /* 0 none, 1 f-plane, 2 beta-plane */
  double latitude;
  double sponge_alpha, sponge_start_fraction;
  double divergence_damping;
  int divergence_order;
  /* --- compositions the reference does not provide: the port restates them
   * in C, the reference-linked driver composes them from the reference's
   * own operators (oracle/ref/ref_driver.cpp) ---
   * pgf_perturbation: 0 = pressure-gradient terms act on the total Exner
   *   function, as src/dyn/equations.cpp:79,88,101,164,173,183 compute;
   *   1 = they act on pi' = pi - pi0, the form the reference documents
   *   (include/vibe/dyn/equations.hpp:9-16, docs/design/04_time_integration.md
   *   sec. 2.2). Only 1 keeps a resting atmosphere at rest.
   * acoustic_mode: 0 = explicit forward-backward substep
   *   (runge_kutta.cpp:65-75); 1 = the reference's HEVI substep
   *   (acoustic_substep.cpp:139-149, dimensionally inconsistent, kernel-level
   *   use only); 2 = vertically implicit (Crank-Nicolson weight hevi_beta)
   *   substep written consistently with the explicit operator.
   */
  int pgf_perturbation;
  int acoustic_mode;
  double hevi_beta;
  /* split_fast: 0 = the slow tendency keeps the pressure-gradient and the
   *   linear mass-divergence terms that the acoustic substeps integrate again
   *   (runge_kutta.cpp:88-100 as written: fast terms counted twice, explicit
   *   at the full stage step); 1 = those terms (acoustic_tendencies of the
   *   stage input state, equations.cpp:152-200) are removed from the slow
   *   tendency of u, v, w and rho, so the substeps integrate them once
   *   (docs/design/04_time_integration.md sec. 2.1-2.2). */
  int split_fast;
  /* weno_advective: 1 = the WENO5 flux-form scalar tendency
   *   (advection.cpp:144-187: -div(u q), no density weight) gets + q div(u)
   *   with the same face winds and spacings, giving the advective form
   *   dq/dt = -u.grad(q) that equations.cpp:8-11 documents; a constant field
   *   then has zero tendency even where the flow is divergent. */
  int weno_advective;
  /* w_rigid: 1 = rigid ground and lid: after every RK3 step (after the
   *   sponge) w is set to zero on the k = 0 and k = nz faces. 0 = the
   *   reference, whose tendencies move every w face (equations.cpp:91-110
   *   over k in [0, nz]), so a buoyant or unbalanced column pushes mass
   *   through the ground. */
  int w_rigid;
} vo_setup;

/* Fill *s with the Config-1 warm-bubble case on an nx x ny x nz grid. */
void vo_setup_defaults(vo_setup *s);

/* ---- plain-C restatement (oracle/vibe_oracle.c) ---- */
typedef struct vo_model vo_model;
vo_model *vo_create(const vo_setup *s);
void vo_destroy(vo_model *m);
size_t vo_storage_size(const vo_model *m, int species);
void vo_get_field(const vo_model *m, int species, double *out);
void vo_set_field(vo_model *m, int species, const double *in);
void vo_get_reffield(const vo_model *m, int which, double *out);
void vo_get_zeta(const vo_model *m, double *out);      /* nz+1 */
void vo_get_terrain(const vo_model *m, double *out);   /* nx*ny */
void vo_get_sponge(const vo_model *m, double *out);    /* nz */
int  vo_rk3_step(vo_model *m, double dt, int n_sub);   /* 0 ok, 1 non-finite */
void vo_slow_tendency(vo_model *m, double *const *out);/* 12 storage arrays */
void vo_acoustic_substep(vo_model *m, double dtau);
void vo_hevi_substep(vo_model *m, double dtau);
void vo_sponge(vo_model *m, double dt);

/* Helmholtz family on the model's grid (src/time/helmholtz.cpp:126-495).
 * a, b, f, x, y are cell FieldT storage arrays (vo_storage_size(m, VO_RHO)
 * doubles, halo 4). apply: y = -div(a grad x) + b x (helmholtz.cpp:173-201);
 * residual_l2: ||A x - f||_2 over the interior (:214-229). kind as
 * HelmholtzKind (helmholtz.hpp:57): 0 vertical_tridiagonal, 1
 * krylov_multigrid (the factory wraps it in the iterative-refinement solver,
 * :486-488), 2 krylov_jacobi. Returns 0, or 1 where the reference throws
 * (singular column). */
enum vo_helmholtz_kind { VO_HZ_VERTICAL = 0, VO_HZ_KRYLOV_MG = 1, VO_HZ_KRYLOV_JACOBI = 2 };
void vo_helmholtz_apply(const vo_model *m, const double *a, const double *b, const double *x, double *y);
double vo_helmholtz_residual_l2(const vo_model *m, const double *a, const double *b, const double *f,
                                const double *x);
int vo_helmholtz_solve(const vo_model *m, int kind, int max_iter, double tol, int refine,
                       const double *a, const double *b, const double *f, double *x, int *iterations,
                       double *residual);
/* multigrid_restrict / multigrid_prolong (helmholtz.cpp:130-164): same-size
 * cell fields (the reference's coarse field lives on the fine grid). */
void vo_multigrid_restrict(const vo_model *m, const double *fine, double *coarse);
void vo_multigrid_prolong(const vo_model *m, const double *coarse, double *fine);
/* One SemiImplicitIntegrator::step (semi_implicit.cpp:167-226, O-SI) with
 * the Helmholtz solver of `kind`. pi_new (nullable) receives the solver's
 * solution; rhs and a_coef (nullable) the assembled right-hand side and a.
 * Returns 0, 1 on a non-finite state, 2 on a singular column. */
int vo_si_step(vo_model *m, double dt, int kind, int max_iter, double tol, int *iterations, double *residual,
               double *pi_new, double *rhs, double *a_coef);

/* Nest transfers (src/grid/nest.cpp:34-124) on FieldT storage arrays: nvars
 * fields of the parent grid (pnx, pny, pnz) and of the child grid (cnx, cny,
 * cnz); stagger[v] (0 cell, 1 x-face, 2 y-face, 3 z-face) sets each field's
 * storage size. davies_profile: n_zone weights (nest.cpp:34-44). */
typedef struct { int i0, j0, k0, iext, jext, ratio, boundary_zone; } vo_nest_placement;
void vo_davies_profile(int n_zone, double alpha_max, double *out);
void vo_nest_interpolate_from_parent(const vo_nest_placement *p, int nvars, const int *stagger, int pnx, int pny,
                                     int pnz, const double *const *parent, int cnx, int cny, int cnz,
                                     double *const *child);
void vo_nest_restrict_to_parent(const vo_nest_placement *p, int nvars, const int *stagger, int cnx, int cny,
                                int cnz, const double *const *child, int pnx, int pny, int pnz,
                                double *const *parent);
void vo_nest_apply_lateral_boundary(const vo_nest_placement *p, int nvars, const int *stagger, int cnx, int cny,
                                    int cnz, double *const *child, const double *const *parent_interp);

/* Tangent-linear / adjoint of the simplified collocated RK3
 * (src/da/tangent_linear.cpp:72-603) on the model's grid. xb, dx, d, ...:
 * 12 FieldT storage arrays (species order). tendency_tl writes d (zeroed
 * first); tendency_ad ACCUMULATES into bar_dx (tangent_linear.cpp:412: the
 * caller zeroes it). tl_step = rk3_tl, ad_step = rk3_ad (:567-603). */
void vo_tl_tendency(const vo_model *m, const double *const *xb, const double *const *dx, double *const *d);
void vo_ad_tendency(const vo_model *m, const double *const *xb, const double *const *bar_d, double *const *bar_dx);
void vo_tl_step(const vo_model *m, const double *const *xb, const double *const *dx, double dt, double *const *out);
/* the nonlinear collocated RK3 whose TL is vo_tl_step (nl_rk3 of the
 * reference's tests/unit/test_tl_ad.cpp:100-199); theta_b from xb */
void vo_nl_step(const vo_model *m, const double *const *xb, const double *const *x, double dt, double *const *out);
void vo_nl_tendency(const vo_model *m, const double *const *xb, const double *const *x, double *const *d);
/* .vibebin restart file of the state (io::write_restart / read_restart,
 * src/io/field_io.cpp:207-250, format src/io/binary_writer.cpp:1-20);
 * 0 on success. */
int vo_write_restart(const vo_model *m, const char *path, double time, int step);
/* dyn::energy_budget (src/dyn/diagnostics.cpp:255-277): {kinetic, internal,
 * potential, latent, total, mass} */
void vo_energy_budget(const vo_model *m, double *out6);
int vo_read_restart(vo_model *m, const char *path, double *time, int *step);

void vo_ad_step(const vo_model *m, const double *const *xb, const double *const *bar_out, double dt,
                double *const *bar_in);

/* Time-step diagnostics: Advection::cfl_number (advection.cpp:325-340),
 * Equations::max_sound_speed (equations.cpp:238-249), AcousticSubstepper::
 * acoustic_cfl (acoustic_substep.cpp:151-168) and RungeKutta3Integrator::
 * max_stable_dt (runge_kutta.cpp:121-140). */
void vo_cfl(const vo_model *m, double dt, double dtau, double *adv_cfl, double *max_sound_speed,
            double *acoustic_cfl);
double vo_max_stable_dt(const vo_model *m);

/* C-ABI kernels restated (src/common/c_kernels.c). vo_tridiagonal_solve
 * follows the documented contract (c_kernels.h:38-55) with the textbook
 * recurrence of thomas_solve (helmholtz.cpp:57-86): the shipped
 * c_kernels.c:18-60 does not solve the system it documents. */
int vo_tridiagonal_solve(const double *a, const double *b, const double *c,
                         const double *d, int n, double *x, double *ws);
void vo_weno5_reconstruct(double qm2, double qm1, double q0, double q1,
                          double q2, double *q_left, double *q_right);
double vo_bilinear(const double *f, int halo, int nsx, int nsy, int nz,
                   double xi, double yj, int k);
double vo_cfl_scan(const double *u, const double *v, const double *w,
                   const double *dzeta, const double *zs, int nx, int ny,
                   int nz, double dx, double dy, double z_top, double dt,
                   double *max_wind_out, double *min_dz_out);
double vo_neumaier_sum(const double *x, size_t n);
void vo_advect_scalar_flux(const double *q, const double *rho, const double *u,
                           const double *v, const double *w, const double *dzeta,
                           const double *zs, int nx, int ny, int nz, double dx,
                           double dy, double z_top, double *dqdt);

/* Kessler warm-rain microphysics (src/physics/microphysics_kessler.cpp) and
 * its coupling through PhysicsDriver's microphysics step
 * (physics_driver.cpp:95-128 state_to_column, :271-288 tendencies) and
 * RungeKutta3Integrator::slow_tendency (runge_kutta.cpp:46-63). The option
 * defaults are PhysicsOptions' (physics_types.hpp:417-430). exner_offset = 1
 * builds the column pressure from pi0 + pi as state_to_column does (the
 * state's pi being the total Exner function, this doubles it); 0 uses pi. */
typedef struct {
  double qc0, k1, k2, evap_coef, rain_a, rain_b;
  int positive_definite, exner_offset;
} vo_kessler;
void vo_kessler_defaults(vo_kessler *k);
/* KesslerMicrophysics::step_column on one column of n levels (k = 0 at the
 * bottom): z (level heights), p, rho given; theta, qv, qc, qr updated in
 * place (qi, qs, qg zero). Returns the surface precipitation rate. */
double vo_kessler_column(const vo_kessler *k, int n, double dt, const double *z, const double *p,
                         const double *rho, double *theta, double *qv, double *qc, double *qr);
/* The PhysicsTendency the microphysics step adds to the slow tendency for
 * the model's current state: out[0..3] = theta, qv, qc, qr rates (cell
 * FieldT storage, zero outside the interior). */
void vo_kessler_tendency(const vo_model *m, const vo_kessler *k, double dt, double *const *out);
/* Couple the scheme into vo_rk3_step (NULL: off). */
void vo_set_physics_kessler(vo_model *m, const vo_kessler *k);

/* ---- reference-linked driver (oracle/ref/ref_driver.cpp) ---- */
typedef struct vref_model vref_model;
vref_model *vref_create(const vo_setup *s);
int vref_write_restart(vref_model *m, const char *path, double time, int step);
void vref_energy_budget(vref_model *m, double *out6);
int vref_read_restart(vref_model *m, const char *path, double *time, int *step);
void vref_destroy(vref_model *m);
/* KesslerMicrophysics::step_column of the compiled reference on the same
 * column as vo_kessler_column. */
double vref_kessler_column(const vo_kessler *k, int n, double dt, const double *z, const double *p,
                           const double *rho, double *theta, double *qv, double *qc, double *qr);
size_t vref_storage_size(const vref_model *m, int species);
void vref_get_field(const vref_model *m, int species, double *out);
void vref_set_field(vref_model *m, int species, const double *in);
void vref_get_reffield(const vref_model *m, int which, double *out);
void vref_get_zeta(const vref_model *m, double *out);
void vref_get_terrain(const vref_model *m, double *out);
void vref_get_sponge(const vref_model *m, double *out);
int  vref_rk3_step(vref_model *m, double dt, int n_sub);
void vref_slow_tendency(vref_model *m, double *const *out);
void vref_acoustic_substep(vref_model *m, double dtau);
void vref_hevi_substep(vref_model *m, double dtau);
void vref_sponge(vref_model *m, double dt);
void vref_helmholtz_apply_norm(vref_model *m, const double *a, const double *b, const double *f,
                               const double *x, double *out);
int vref_helmholtz_solve(vref_model *m, int kind, int max_iter, double tol, int refine, const double *a,
                         const double *b, const double *f, double *x, int *iterations, double *residual);
void vref_multigrid_restrict(vref_model *m, const double *fine, double *coarse);
void vref_multigrid_prolong(vref_model *m, const double *coarse, double *fine);
int vref_si_step(vref_model *m, double dt, int kind, int max_iter, double tol, int *iterations,
                 double *residual, double *pi_new, double *rhs, double *a_coef);
/* tendency_tl/_ad are file-local in the reference (tangent_linear.cpp:295,
 * 414); they are pinned through the public step and propagate calls. */
void vref_tl_step(vref_model *m, const double *const *xb, const double *const *dx, double dt, double *const *out);
void vref_ad_step(vref_model *m, const double *const *xb, const double *const *bar_out, double dt,
                  double *const *bar_in);
/* TangentLinearModel::propagate (frozen xb) and AdjointModel::
 * propagate_with_trajectory over the trajectory it records */
void vref_tl_propagate(vref_model *m, const double *const *xb, const double *const *dx0, double dt, int n_steps,
                       double *const *out);
void vref_ad_propagate(vref_model *m, const double *const *xb, const double *const *dy, double dt, int n_steps,
                       double *const *out);
void vref_cfl(vref_model *m, double dt, double dtau, double *adv_cfl, double *max_sound_speed,
              double *acoustic_cfl);
double vref_max_stable_dt(vref_model *m);
void vref_davies_profile(int n_zone, double alpha_max, double *out);
void vref_nest_interpolate_from_parent(const vo_nest_placement *p, int nvars, const int *stagger, int pnx, int pny,
                                       int pnz, const double *const *parent, int cnx, int cny, int cnz,
                                       double *const *child);
void vref_nest_restrict_to_parent(const vo_nest_placement *p, int nvars, const int *stagger, int cnx, int cny,
                                  int cnz, const double *const *child, int pnx, int pny, int pnz,
                                  double *const *parent);
void vref_nest_apply_lateral_boundary(const vo_nest_placement *p, int nvars, const int *stagger, int cnx, int cny,
                                      int cnz, double *const *child, const double *const *parent_interp);

#ifdef __cplusplus
}
#endif

#endif
