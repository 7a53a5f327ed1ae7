/* include/vibe_gb300.h
 *
 * C ABI of the GB300 dynamics step: the device-resident counterpart of the
 * reference's C++ stepper interfaces. Each entry point names the reference
 * interface it replaces:
 *   vibe_gb300_model_create     RungeKutta3Integrator ctor (include/vibe/time/
 *                               runge_kutta.hpp:53-56) + Grid/ReferenceState/
 *                               State set-up (geometry.hpp:89-161,
 *                               reference_state.hpp:36-49, state.hpp:98-103)
 *                               + driver::init_warm_bubble
 *                               (initial_conditions.hpp:84-85)
 *   vibe_gb300_step             Integrator::step(State&, const StepContext&)
 *                               (include/vibe/time/integrator.hpp:65), n times
 *   vibe_gb300_slow_tendency    Equations::tendencies (equations.hpp:67)
 *   vibe_gb300_acoustic_substep RungeKutta3Integrator::acoustic_substep
 *                               (runge_kutta.hpp:62-63)
 *   vibe_gb300_hevi_substep     AcousticSubstepper::step (acoustic_substep.hpp:59)
 *   vibe_gb300_sponge           Damping::apply_sponge (damping.hpp:36)
 *   vibe_gb300_get/set_field    FieldT::storage() of a State species
 *                               (field.hpp:73-74), same halo'd layout
 * Errors: every int-returning call returns 0 on success and a negative
 * VIBE_GB300_E* code otherwise (the reference throws NumericalError /
 * VIBE_CHECK failures instead); vibe_gb300_last_error() gives the message.
 * Threading: one model is not thread-safe (as the reference's integrators);
 * separate models may be used from separate threads. All device work of a
 * model runs on its own CUDA stream.
 */
#ifndef VIBE_GB300_H
#define VIBE_GB300_H

#include <stddef.h>

#include "vibe_c_kernels.h"

#ifdef __cplusplus
extern "C" {
#endif

#define VIBE_GB300_OK 0
#define VIBE_GB300_EBADARG (-1)
#define VIBE_GB300_EDEVICE (-2)
#define VIBE_GB300_ENONFINITE (-3) /* RK3 non-finite check, runge_kutta.cpp:103-106 */
#define VIBE_GB300_ESINGULAR (-4)  /* Thomas pivot < 1e-300, helmholtz.cpp:78-80 */
#define VIBE_GB300_EUNSUPPORTED (-5)

#define VIBE_GB300_FP64 0  /* all arithmetic FP64 */
#define VIBE_GB300_MIXED 1 /* FP64 state, FP32 tendencies and substeps */
#define VIBE_GB300_FP64_EXACT 2 /* FP64 without FMA contraction: the reference's bits */

/* Species order of dyn::Species (include/vibe/dyn/state.hpp:53-55). */
enum vibe_gb300_species {
  VIBE_U = 0, VIBE_V, VIBE_W, VIBE_RHO, VIBE_THETA, VIBE_PI, VIBE_QV,
  VIBE_QC, VIBE_QR, VIBE_QI, VIBE_QS, VIBE_QG, VIBE_NSPECIES
};

/* Case and numerics description. Field meaning as in config.hpp:26-68,
 * IcOptions (initial_conditions.hpp:49-74) and ReferenceState. The last
 * five fields select compositions the reference does not provide: the
 * reference as written integrates the fast terms twice (once in the slow
 * tendency, once in the substeps) and takes the pressure gradient of the
 * total Exner function, and diverges within a few steps; pgf_perturbation,
 * split_fast and weno_advective give the stable composition, acoustic_mode
 * 2 a dimensionally consistent Crank-Nicolson HEVI with off-centring
 * hevi_beta. Plain C struct, no defaults: fill with
 * vibe_gb300_setup_defaults() first. */
typedef struct vibe_gb300_setup {
  int nx, ny, nz;
  double dx, dy, z_top;
  double zeta_first, zeta_stretch;  /* make_stretched_zeta(nz, first, stretch) */
  int terrain_kind;                 /* 0 flat, 1 Gaussian hill */
  double hill_h, hill_a, hill_xc, hill_yc;
  int ref_kind;                     /* 0 isothermal(theta0), 1 theta0*exp(N^2 z/g) profile */
  double theta0, p_surf, bv_n, profile_dz;
  double bubble_amplitude, bubble_radius_x, bubble_radius_z;
  double bubble_xc, bubble_yc, bubble_zc;
  double qv_surface, qv_decay_height;
  double u_background, shear_u;
  int advection;                    /* 2, 4, 6 central; 5 weno5 */
  int weno_scalars;                 /* theta/q by WENO5 flux form */
  int moist;
  int coriolis;                     /* 0 none, 1 f-plane, 2 beta-plane */
  double latitude;
  double sponge_alpha, sponge_start_fraction;
  double divergence_damping;
  int divergence_order;
  int pgf_perturbation;             /* pressure gradient on pi - pi0 */
  int acoustic_mode;                /* 0 explicit FB, 1 reference HEVI, 2 consistent HEVI */
  double hevi_beta;
  int split_fast;                   /* fast terms integrated only by the substeps */
  int weno_advective;               /* WENO5 flux form + q div(u) */
  int w_rigid;                      /* 1: w = 0 on the ground and lid faces after every step */
} vibe_gb300_setup;

typedef struct vibe_gb300_model vibe_gb300_model;

void vibe_gb300_setup_defaults(vibe_gb300_setup *s);

/* Builds grid metrics, reference state and the warm-bubble initial state on
 * the host (same formulas as the reference), uploads them and allocates all
 * device buffers. precision: VIBE_GB300_FP64 or VIBE_GB300_MIXED (the mixed
 * path needs flat terrain, a horizontally uniform reference state,
 * pgf_perturbation = 1 and split_fast = 1). */
int vibe_gb300_model_create(const vibe_gb300_setup *s, int precision,
                            vibe_gb300_model **out);
void vibe_gb300_model_destroy(vibe_gb300_model *m);

/* Number of doubles in the FieldT storage of a species (halo 4). */
size_t vibe_gb300_storage_size(const vibe_gb300_model *m, int species);
/* Copy a species between the device state and a host array in FieldT
 * storage layout. get writes zeros into halo points other than the east/
 * north ghost line the step reads (the serial reference never fills them). */
int vibe_gb300_get_field(vibe_gb300_model *m, int species, double *host);
int vibe_gb300_set_field(vibe_gb300_model *m, int species, const double *host);
/* Reference-state field (0 theta0, 1 pi0, 2 rho0, 3 p0, 4 qv0), zeta
 * (nz+1), terrain (nx*ny) and sponge profile (nz) as built on the host. */
int vibe_gb300_get_reffield(const vibe_gb300_model *m, int which, double *host);
int vibe_gb300_get_zeta(const vibe_gb300_model *m, double *host);
int vibe_gb300_get_terrain(const vibe_gb300_model *m, double *host);
int vibe_gb300_get_sponge(const vibe_gb300_model *m, double *host);

/* n_steps RK3 steps of length dt with n_sub acoustic substeps per stage.
 * Blocks until done; returns VIBE_GB300_ENONFINITE if a stage produced a
 * non-finite value. */
int vibe_gb300_step(vibe_gb300_model *m, double dt, int n_sub, int n_steps);
/* Enqueue only (no host synchronisation); vibe_gb300_sync returns the
 * status of everything enqueued since the previous sync. */
int vibe_gb300_step_async(vibe_gb300_model *m, double dt, int n_sub, int n_steps);
int vibe_gb300_sync(vibe_gb300_model *m);

/* Time-step diagnostics of the current state (FP64, exact maxima):
 * adv_cfl = Advection::cfl_number(s, dt) (advection.cpp:325-340),
 * max_sound_speed = Equations::max_sound_speed(s) (equations.cpp:238-249),
 * acoustic_cfl = AcousticSubstepper::acoustic_cfl(s, dtau)
 * (acoustic_substep.cpp:151-168). Outputs nullable. */
int vibe_gb300_cfl(vibe_gb300_model *m, double dt, double dtau, double *adv_cfl, double *max_sound_speed,
                   double *acoustic_cfl);
/* RungeKutta3Integrator::max_stable_dt (runge_kutta.cpp:121-140). */
int vibe_gb300_max_stable_dt(vibe_gb300_model *m, double *dt_out);

/* Mixed path: replay each step as a CUDA graph (default on; the first step
 * after a dt/n_sub change runs eagerly, the next ones capture and replay;
 * off while kernel timing is on). */
int vibe_gb300_set_graph(vibe_gb300_model *m, int enable);

/* Groups: several mixed-precision models (acoustic_mode 2, equal nz and
 * numerics flags, any nx/ny; members of an ensemble, or the parents, or the
 * nests of a nested set) advanced together with one launch per kernel for
 * all of them (a work-list over every domain's blocks) and each step
 * replayed as a CUDA graph. The models keep their state; the group does not
 * own them (destroy the group first). group_step blocks until done and
 * returns the first failure of any member (VIBE_GB300_ENONFINITE, ...). */
typedef struct vibe_gb300_group vibe_gb300_group;
int vibe_gb300_group_create(vibe_gb300_model *const *models, int n, vibe_gb300_group **out);
void vibe_gb300_group_destroy(vibe_gb300_group *g);
int vibe_gb300_group_step(vibe_gb300_group *g, double dt, int n_sub, int n_steps);
int vibe_gb300_group_launches_per_step(const vibe_gb300_group *g);
vibe_stream_t vibe_gb300_group_stream(vibe_gb300_group *g);

/* Nested sets (two-way nests with time sub-cycling, O-NEST): the parents
 * step with dt as one group, then every nest gets its parent's state
 * interpolated into a boundary buffer (Nest::interpolate_from_parent,
 * nest.cpp:58-84, with interp_pl[c]), the nests take r = ratio sub-steps of
 * dt/r as one group, each followed by the Davies relaxation towards that
 * buffer (apply_lateral_boundary, nest.cpp:107-124), and finally each nest
 * is restricted onto its parent (restrict_to_parent, nest.cpp:86-105, with
 * restrict_pl[c]). The reference's interpolation takes the nest offset in
 * child points and its restriction in parent points, hence two placements.
 * Fields transferred: u v w rho theta pi qv (+ the moisture species when
 * moist). Models are not owned. */
struct vibe_nest_placement;
typedef struct vibe_gb300_nested vibe_gb300_nested;
int vibe_gb300_nested_create(vibe_gb300_model *const *parents, int n_parents, vibe_gb300_model *const *children,
                             int n_children, const int *parent_of, const struct vibe_nest_placement *interp_pl,
                             const struct vibe_nest_placement *restrict_pl, vibe_gb300_nested **out);
void vibe_gb300_nested_destroy(vibe_gb300_nested *n);
/* One parent step is one CUDA graph on the set's stream (captured once per
 * pair of state parities). nested_step = nested_launch (enqueue, returns at
 * once) + nested_wait (synchronise, then report a non-finite state or a
 * device wait that gave up). */
int vibe_gb300_nested_step(vibe_gb300_nested *n, double dt, int n_sub, int n_steps);
int vibe_gb300_nested_launch(vibe_gb300_nested *n, double dt, int n_sub, int n_steps);
int vibe_gb300_nested_wait(vibe_gb300_nested *n);
/* kernel launches of one parent step (after the first launch) */
int vibe_gb300_nested_launches_per_step(const vibe_gb300_nested *n);
vibe_stream_t vibe_gb300_nested_stream(vibe_gb300_nested *n);

/* Assimilation windows (Config-5 style): the TL/AD model of a vibe_tlad
 * object (include/vibe_tlad.h, same grid) linearised about this model's own
 * trajectory over n_steps steps of dt (n_sub acoustic substeps), the TL/AD
 * taking tl_substeps steps of dt/tl_substeps per model step (its explicit
 * acoustics need the shorter step). The state at model step n is the
 * linearisation point of TL/AD step n (TangentLinearModel::propagate with a
 * recorded trajectory, tangent_linear.cpp:679-716; AdjointModel::
 * propagate_with_trajectory, :749-765). States are copied to device
 * checkpoints every `every` steps; the adjoint recomputes each segment from
 * its checkpoint (CheckpointStrategy::Recompute, tangent_linear.hpp:56-61).
 * every = 0 chooses by free device memory: every step stored when the whole
 * trajectory fits (StoreAll), else checkpoints every ceil(sqrt(n_steps/2))
 * steps with recomputation; window_stats reports the choice.
 * Both sweeps start from the model's current state and leave it there.
 * Perturbations: 12 FieldT host arrays (species order), halos pass through.
 * window_stats: device time of the last sweep, checkpoint and segment memory.
 * t = NULL selects the tangent-linear and adjoint of the model's own step
 * instead (vibe_gb300_step_tl / _ad below: the configured slow tendency, its
 * acoustic substeps and the sponge, runge_kutta.cpp:77-119), linearised about
 * the model's trajectory, one TL/AD step per model step (tl_substeps must be
 * 1); its segments hold each step's three stage inputs, recomputed from the
 * checkpoints.
 * window_plan: the automatic choice of `every` (every = 0) as a pure
 * function: store every step when n_steps + seg_states states fit in 80 % of
 * free_bytes, else every = ceil(sqrt(n_steps / seg_states)) if the
 * checkpoints and one segment (seg_states states per step) fit, else
 * VIBE_GB300_EDEVICE. seg_states: 2 with a vibe_tlad object (double-buffered
 * segments), 3 for the model's own step. */
struct vibe_tlad;
typedef struct vibe_gb300_window vibe_gb300_window;
int vibe_gb300_window_plan(size_t free_bytes, size_t state_bytes, int n_steps, int seg_states, int *every);
int vibe_gb300_window_create(vibe_gb300_model *m, struct vibe_tlad *t, double dt, int n_sub, int n_steps, int every,
                             int tl_substeps, vibe_gb300_window **out);
void vibe_gb300_window_destroy(vibe_gb300_window *w);
int vibe_gb300_window_tl(vibe_gb300_window *w, const double *const *dx0, double *const *dx_out);
int vibe_gb300_window_ad(vibe_gb300_window *w, const double *const *dy, double *const *dx0_adjoint);
int vibe_gb300_window_stats(const vibe_gb300_window *w, double *last_ms, size_t *checkpoint_bytes,
                            size_t *segment_bytes);

/* Tangent-linear and adjoint of the model's own slow tendency and step,
 * linearised about the model's current state (which they leave as it is);
 * no counterpart in the reference, whose TL/AD (tangent_linear.cpp:295-603)
 * is of a collocated step without acoustic substeps. The step is the one
 * vibe_gb300_step takes (runge_kutta.cpp:77-119 with the configured
 * composition): x1 = A^n (x0 + dt/3 R(x0)), x2 = A^n (x0 + dt/2 R(x1)),
 * x3 = A^n (x0 + dt R(x2)), then the sponge and the rigid ground/lid; R the
 * slow tendency (Equations::tendencies, equations.cpp:60-150, with the WENO5
 * or central scalar scheme), A one acoustic substep (explicit or consistent
 * HEVI). The TL of R differentiates the WENO5 weights and the
 * Lax-Friedrichs switch exactly (the positivity clip contributes zero where
 * it holds); the adjoint is its exact transpose. FP64 models compute in FP64;
 * mixed models in FP32 (the slow tendency's TL/AD and the model's own FP32
 * substeps and their adjoints), with FP64 storage.
 * Arrays: 12 FieldT host arrays (species order). tendency_tl writes the
 * tendency's staggered boxes (zero elsewhere); tendency_ad takes the bar of
 * those boxes and returns the bar of every input point (the boxes with the
 * ghost column and row); step_tl / step_ad keep the points no step writes
 * from their input. Not supported (VIBE_GB300_EUNSUPPORTED): a physics
 * package, acoustic_mode 1 (the reference HEVI), fourth-order divergence
 * damping. */
int vibe_gb300_tendency_tl(vibe_gb300_model *m, const double *const *dx, double *const *out);
int vibe_gb300_tendency_ad(vibe_gb300_model *m, const double *const *bar_r, double *const *bar_x);
int vibe_gb300_step_tl(vibe_gb300_model *m, double dt, int n_sub, const double *const *dx, double *const *out);
int vibe_gb300_step_ad(vibe_gb300_model *m, double dt, int n_sub, const double *const *dy, double *const *out);

/* Kernel-level entry points (FP64 path only for the tendency). */
int vibe_gb300_slow_tendency(vibe_gb300_model *m, double *const *host_out);
int vibe_gb300_acoustic_substep(vibe_gb300_model *m, double dtau);

/* Tangent-linear and adjoint of the explicit forward-backward substep
 * (RungeKutta3Integrator::acoustic_substep, runge_kutta.cpp:65-75, with
 * Equations::acoustic_tendencies, equations.cpp:152-209, taking the pressure
 * gradient of pi itself so that the substep is linear in the perturbation):
 * n_sub substeps of dtau about the model's reference state, in FP64 for
 * either precision. in / out: FieldT storage of the perturbations of u, v, w,
 * rho and pi, in that order (out may alias in). The adjoint runs the
 * transposed phases in reverse. Points outside each field's staggered box
 * pass through unchanged. */
int vibe_gb300_acoustic_tl(vibe_gb300_model *m, double dtau, int n_sub, const double *const *in, double *const *out);
int vibe_gb300_acoustic_ad(vibe_gb300_model *m, double dtau, int n_sub, const double *const *in, double *const *out);
/* The same pair for the dimensionally consistent HEVI substep (the
 * vertically implicit Crank-Nicolson substep with the model's hevi_beta and
 * the horizontal u/v backward update), also linear about the reference state
 * with the gradient of pi itself; the adjoint transposes the column system.
 * As the model's own substep does, it sets the ghost column i = nx and row
 * j = ny of w, rho and pi to zero. */
int vibe_gb300_hevi_tl(vibe_gb300_model *m, double dtau, int n_sub, const double *const *in, double *const *out);
/* FP32 forms for mixed models: the model's own FP32 forward-backward substep
 * (per-level reference tables) on perturbations of u, v, w, rho' = rho - rho0
 * and pi' = pi - pi0 (FieldT storage in and out, as above), and its adjoint. */
int vibe_gb300_acoustic_tl_f32(vibe_gb300_model *m, double dtau, int n_sub, const double *const *in,
                               double *const *out);
int vibe_gb300_acoustic_ad_f32(vibe_gb300_model *m, double dtau, int n_sub, const double *const *in,
                               double *const *out);
/* The FP32 pair for the mixed model's own consistent HEVI substep (column
 * kernel + u/v update, hevi_beta of the model); the adjoint transposes the
 * column system through its LU factors. */
int vibe_gb300_hevi_tl_f32(vibe_gb300_model *m, double dtau, int n_sub, const double *const *in, double *const *out);
int vibe_gb300_hevi_ad_f32(vibe_gb300_model *m, double dtau, int n_sub, const double *const *in, double *const *out);
int vibe_gb300_hevi_ad(vibe_gb300_model *m, double dtau, int n_sub, const double *const *in, double *const *out);
int vibe_gb300_hevi_substep(vibe_gb300_model *m, double dtau);
/* Autotuner of the mixed step: times, on this model's grid, the launch shapes
 * of the same update -- the HEVI column kernel variant (0 register ring,
 * 1 cp.async ring, 2/3 two columns per thread, 4 two columns per thread fed
 * by TMA boxes, 5 the same with the w/rho' corrections of the implicit
 * sweep applied by the next reader of those fields, which cuts the
 * backward sweep's traffic to pi' alone -- the built-in choice; -1 = the
 * built-in choice) and
 * the stage kernel's levels per block -- and keeps the fastest for every
 * single model of this grid in the process (groups keep the built-in column
 * kernel). Variants differ only by FP32 rounding (FMA contraction, vertical
 * fluxes recomputed at level-chunk starts). The model's state is left as it
 * was. Returns the choice, its time per step and the built-in one's. */
typedef struct {
  int stage_levels;
  int column_kernel;
  double ms_per_step;
  double default_ms_per_step;
  int candidates;
} vibe_gb300_tuning;
int vibe_gb300_autotune(vibe_gb300_model *m, double dt, int n_sub, vibe_gb300_tuning *out);
/* Pin a tuning (stage_levels 0 = built-in, column_kernel -1 = built-in) for
 * this model's grid, e.g. one found by an earlier autotune run; the other
 * fields of t are ignored. */
int vibe_gb300_set_tuning(vibe_gb300_model *m, const vibe_gb300_tuning *t);

/* ---- physics coupling (Integrator::set_physics, integrator.hpp:74;
 * RungeKutta3Integrator::slow_tendency, runge_kutta.cpp:46-63) ----
 * A physics package is a function that the step calls once per RK stage,
 * while the stage's launches are enqueued, with the stage's input state and
 * zeroed tendency accumulators; it enqueues its work on `stream` (work on
 * that stream is captured into the step's CUDA graph, so the function must
 * not synchronise) and returns 0, or nonzero to fail the step. The step then
 * adds the accumulated local rates of theta, qv..qg, u and v to the slow
 * tendency (d += pt) before the stage update, as the reference does with its
 * PhysicsTendency. Device layout of every field: element (i, j, k) at
 * (k*(ny+1) + j)*pitch + i. */
typedef struct {
  int precision;          /* VIBE_GB300_FP64 (double fields) or VIBE_GB300_MIXED (float fields) */
  int stage;              /* RK stage 0, 1, 2 */
  double dt;              /* the step's dt (what PhysicsDriver::step receives) */
  int nx, ny, nz, pitch;
  int moist;              /* 1: qc..qg are prognostic (setup.moist) */
  /* stage input per species (device). FP64: the totals. MIXED: u, v, w and
   * the moisture species as totals, rho, theta, pi as departures from the
   * reference state below. */
  const void *state[12];
  /* zeroed device accumulators (local rates) for u, v, theta, qv..qg; the
   * other species' entries are NULL */
  void *tend[12];
  const double *ref_theta, *ref_pi, *ref_rho; /* device, reference state (device layout, FP64) */
  const double *zeta_mid;                     /* device, nz: normalised height of the level centres */
  const double *terrain;                      /* device, nx*ny row-major: terrain height */
  const double *depth;                        /* device, nx*ny: z_top - terrain height */
  void *stream;                               /* cudaStream_t */
  /* in/out: bit q set = the package may write tend[q]. It comes in with all
   * nine accumulators; a package that writes fewer clears the others' bits,
   * and only those accumulators are zeroed before its next call and added to
   * the tendency (the rest stay zero). */
  unsigned written;
} vibe_gb300_physics_args;
typedef int (*vibe_gb300_physics_fn)(void *user, vibe_gb300_physics_args *args);
/* Install (fn != NULL) or remove the package; drops the step graphs. Groups
 * and nested sets step their members without physics: creating one from a
 * model with a package installed fails (VIBE_GB300_EUNSUPPORTED), and a
 * package installed on a member afterwards does not enter the group's steps. */
int vibe_gb300_set_physics(vibe_gb300_model *m, vibe_gb300_physics_fn fn, void *user);
/* The installed package's tendency for the current state (one call as at
 * stage 0 with this dt), downloaded as FieldT storage: out[0..8] = u, v,
 * theta, qv, qc, qr, qi, qs, qg (entries may be NULL). */
int vibe_gb300_physics_tendency(vibe_gb300_model *m, double dt, double *const *out);

/* Built-in package: Kessler warm rain (KesslerMicrophysics::step_column,
 * src/physics/microphysics_kessler.cpp:269-331) as PhysicsDriver's
 * microphysics step applies it (state_to_column, physics_driver.cpp:95-128;
 * tendencies (after - before)/dt, :271-288), radiation, surface, boundary
 * layer, cumulus and subgrid momentum off. One thread per column; FP64
 * arithmetic for FP64 models, FP32 for mixed ones. Needs moisture species
 * (setup.moist = 1). user = const vibe_gb300_kessler* (kept by the caller). */
typedef struct {
  double qc0, k1, k2, evap_coef, rain_a, rain_b; /* PhysicsOptions::kessler_* (physics_types.hpp:424-429) */
  int positive_definite;                         /* PhysicsOptions::positive_definite */
  /* 1: column pressure from ref_pi + pi, as state_to_column builds it (the
   * state's pi is the total Exner function there, so this doubles it);
   * 0: from pi alone */
  int exner_offset;
} vibe_gb300_kessler;
void vibe_gb300_kessler_defaults(vibe_gb300_kessler *k);
int vibe_gb300_physics_kessler(void *user, vibe_gb300_physics_args *args);
/* One step with host input and output (FieldT storage, pinned host memory
 * for full speed), asynchronous and pipelined across calls: the call
 * enqueues the input's host -> device copies on a copy stream, the step on
 * the model's stream and the result's device -> host copies on a second copy
 * stream, with two device staging buffers each way, so that step n's
 * download and step n+2's upload overlap step n+1. host_in[q] / host_out[q]
 * may be NULL (species not uploaded / not read); n_in, n_out <= 12. The host
 * buffers must stay untouched until vibe_gb300_sync (which also reports
 * errors) returns. vibe_gb300_io_join makes the model's stream wait for all
 * copies (a CUDA event recorded on it afterwards covers the whole pipeline). */
int vibe_gb300_step_io(vibe_gb300_model *m, const double *const *host_in, int n_in, double *const *host_out,
                       int n_out, double dt, int n_sub);
int vibe_gb300_io_join(vibe_gb300_model *m);
/* Global energy and mass budget of the current state in FP64 (dyn::
 * energy_budget, src/dyn/diagnostics.cpp:255-277): out6 = {kinetic,
 * internal, potential, latent, total, mass} in J and kg, summed on the
 * device with compensated (Neumaier) FP64 accumulation, deterministic. */
int vibe_gb300_energy_budget(vibe_gb300_model *m, double *out6);
/* Restart files of the device state in the reference's .vibebin format
 * (io::write_restart / read_restart, src/io/field_io.cpp:207-250; layout
 * src/io/binary_writer.cpp:1-20): the 12 species over their stagger's
 * points plus "__restart_info__" = [time, step]; files are interchangeable
 * with the reference's. Reading keeps the points the file does not hold
 * (halo, ghost lines, absent species) and refreshes the FP32 working copy. */
int vibe_gb300_write_restart(vibe_gb300_model *m, const char *path, double time, int step);
int vibe_gb300_read_restart(vibe_gb300_model *m, const char *path, double *time, int *step);
/* Device-side copy of the prognostic state: op 0 saves the current state
 * (all species, model layout) into a snapshot held by the model, op 1 puts
 * it back (and refreshes the FP32 working copy). Asynchronous on the model's
 * stream; no host memory is touched. Used for restarts of a run from a
 * checkpoint and for trajectory checkpoints. */
int vibe_gb300_snapshot(vibe_gb300_model *m, int op);
int vibe_gb300_sponge(vibe_gb300_model *m, double dt);

/* One semi-implicit step, replacing SemiImplicitIntegrator::step
 * (src/time/semi_implicit.cpp:167-226) as the reference's code computes it
 * (FP64 precisions only): slow tendency R; Helmholtz problem of
 * assemble_rhs (:56-106: a = (dt/2)^2 (Rd/cv) pi0 cp theta0, b = 1); solve
 * with the solver helmholtz_kind of include/vibe_helmholtz.h (the
 * reference's default is krylov_multigrid, max_iter 200, tol 1e-8);
 * theta, qv, rho and the moisture species += dt R; sponge; non-finite check.
 * The shipped step writes the solved pressure only into a copy of the state
 * that it then drops, so u, v, w and pi change only through the sponge.
 * iterations, residual: the solver's statistics (nullable); pi_new
 * (nullable): the solution, host FieldT cell storage. */
int vibe_gb300_si_step(vibe_gb300_model *m, double dt, int helmholtz_kind, int max_iter, double tol,
                       int *iterations, double *residual, double *pi_new);
/* Statistics of the last semi-implicit step's solve (IntegratorStats::
 * helmholtz_iterations / helmholtz_residual, integrator.hpp:53-59) and its
 * device time in ms (coefficient set-up + solve, CUDA events). */
int vibe_gb300_si_stats(const vibe_gb300_model *m, int *iterations, double *residual, double *solve_ms);

/* Bulk forms of set/get_field over species 0..nspecies-1 (NULL entries are
 * skipped). Asynchronous on the model stream: host arrays must stay valid
 * until vibe_gb300_sync(); pinned host memory makes the copies overlap. */
int vibe_gb300_set_state(vibe_gb300_model *m, const double *const *host, int nspecies);
int vibe_gb300_get_state(vibe_gb300_model *m, double *const *host, int nspecies);

/* Optional timing of kernel classes with CUDA events on the model stream
 * (0 = RK stage kernels, 1 = acoustic substep column/mass kernels,
 * 2 = finish/sponge/checks, 3 = horizontal momentum of the HEVI substep).
 * kernel_times returns the accumulated milliseconds and event-pair counts
 * since timing was enabled. */
int vibe_gb300_set_kernel_timing(vibe_gb300_model *m, int enable);
int vibe_gb300_kernel_times(vibe_gb300_model *m, double *ms, long *count, int nclass);

/* Device pointer of a species in the device layout
 * idx = (k*(ny+1) + j)*pitch + i, and that pitch. */
int vibe_gb300_device_field(vibe_gb300_model *m, int species, double **ptr, int *pitch);
vibe_stream_t vibe_gb300_stream(vibe_gb300_model *m);
/* Number of kernels this model launches per step for (dt, n_sub). */
int vibe_gb300_launches_per_step(const vibe_gb300_model *m, int n_sub);

const char *vibe_gb300_last_error(void);

#ifdef __cplusplus
}
#endif

#endif
