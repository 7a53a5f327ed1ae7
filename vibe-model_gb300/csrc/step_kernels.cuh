// vibe-model_gb300/csrc/step_kernels.cuh -- launchers of the step kernels.
#pragma once
#include <vector>

#include "vibe_internal.cuh"

namespace vgb {

// ---- FP64 path (step_fp64.cu) ----
void fp64_slow_tendency(const Dims& d, const Metric& m, const Flags& fl, double* const* st, double* const* tend,
                        double* lap_scratch, double* face_scratch, cudaStream_t stream);
void fp64_stage_update(const Dims& d, double* const* s0, double* const* tend, double a, double* const* out,
                       cudaStream_t stream);
void fp64_fb_substep(const Dims& d, const Metric& m, const Flags& fl, double* const* st, double dtau,
                     cudaStream_t stream);
void fp64_fb_substep_ad(const Dims& d, const Metric& m, double* const* bar, double dtau, cudaStream_t stream);
void fp64_hevi_substep_ad(const Dims& d, const Metric& m, const Flags& fl, double* const* bar, double* bdh,
                          double* scratch, double dtau, unsigned* err, cudaStream_t stream);
void fp64_ref_hevi_substep(const Dims& d, const Metric& m, double* const* st, double dtau, const double* ta,
                           const double* tb, const double* tc, double* scratch, unsigned* err, cudaStream_t stream);
void fp64_cons_hevi_substep(const Dims& d, const Metric& m, const Flags& fl, double* const* st, double* const* tmp,
                            double* scratch, double dtau, unsigned* err, cudaStream_t stream);
void fp64_sponge(const Dims& d, const Metric& m, double* const* st, int kmin, double dt, cudaStream_t stream);
void fp64_nonfinite(const Dims& d, double* const* st, unsigned* err, cudaStream_t stream);

// ---- bit-exact FP64 path (step_fp64.cu built with --fmad=false) ----
void fp64_slow_tendency_exact(const Dims& d, const Metric& m, const Flags& fl, double* const* st, double* const* tend,
                        double* lap_scratch, double* face_scratch, cudaStream_t stream);
void fp64_stage_update_exact(const Dims& d, double* const* s0, double* const* tend, double a, double* const* out,
                       cudaStream_t stream);
void fp64_fb_substep_exact(const Dims& d, const Metric& m, const Flags& fl, double* const* st, double dtau,
                     cudaStream_t stream);
void fp64_fb_substep_ad_exact(const Dims& d, const Metric& m, double* const* bar, double dtau, cudaStream_t stream);
void fp64_hevi_substep_ad_exact(const Dims& d, const Metric& m, const Flags& fl, double* const* bar, double* bdh,
                                double* scratch, double dtau, unsigned* err, cudaStream_t stream);
void fp64_ref_hevi_substep_exact(const Dims& d, const Metric& m, double* const* st, double dtau, const double* ta,
                           const double* tb, const double* tc, double* scratch, unsigned* err, cudaStream_t stream);
void fp64_cons_hevi_substep_exact(const Dims& d, const Metric& m, const Flags& fl, double* const* st, double* const* tmp,
                            double* scratch, double dtau, unsigned* err, cudaStream_t stream);
void fp64_sponge_exact(const Dims& d, const Metric& m, double* const* st, int kmin, double dt, cudaStream_t stream);
void fp64_nonfinite_exact(const Dims& d, double* const* st, unsigned* err, cudaStream_t stream);

// ---- semi-implicit step (si_step.cu, no FMA contraction) ----
// a, b, f: nx*ny*nz (Helmholtz solver layout); st, tend: model layout
void si_assemble(const Dims& d, const Metric& met, double* const* st, double* const* tend, double dt, double* a,
                 double* b, double* f, cudaStream_t s);
void si_cells_add_scaled(const Dims& d, double* x, const double* y, double a, cudaStream_t s);
void si_to_cells(const Dims& d, const double* in, double* out, cudaStream_t s);

// ---- time-step diagnostics (diag.cu): out[0..3] = advective CFL at dt,
// max sound speed, acoustic CFL at dtau, max(1/dx + 1/dy + 1/dz), as IEEE bits ----
void diag_cfl(const Dims& d, const Metric& met, double* const* st, double dt, double dtau, unsigned long long* out,
              cudaStream_t s);

// ---- nest transfers on model-layout fields (nest.cu): op 0 interpolate,
// 1 restrict, 2 Davies blend (see include/vibe_nest.h) ----
}  // namespace vgb
struct vibe_nest_placement;
namespace vgb {
// Launch choices of the mixed step per grid (stage levels per block, 0 =
// built-in choice; column kernel 0 register ring, 1 cp.async ring, 2/3 two
// columns per thread, -1 = built-in), as the autotuner sets them.
struct MixedTune {
  int stage_levels = 0;
  int column = -1;
};
void mixed_set_tune(const Dims& d, const MixedTune& t);
int mixed_stage_levels(const Dims& d);

// zone_only (op 0): interpolate only the points of the Davies zone, the
// only ones op 2 reads (for a boundary buffer)
int nest_model_layout(int op, const vibe_nest_placement* p, int nvars, int pnx, int pny, int pnz,
                      const double* const* parent, size_t p_pitch, size_t p_plane, int cnx, int cny, int cnz,
                      const double* const* child_in, double* const* out, size_t c_pitch, size_t c_plane,
                      cudaStream_t s, bool zone_only = false);

// ---- mixed path (step_mixed.cu): FP64 state, FP32 working state ----
// Horizontally uniform reference state on flat terrain: every coefficient
// is a function of k only and lives in these FP32 tables (device).
struct Tab {
  const float* r0c;    // nz   rho0(k)
  const float* rfz;    // nz+1 0.5*(rho0(max(k-1,0)) + rho0(min(k,nz-1)))
  const float* t0c;    // nz   theta0(k)
  const float* tfz;    // nz+1 0.5*(theta0(max(k-1,0)) + theta0(min(k,nz-1)))
  const float* kap;    // nz   (Rd/cv) * pi0 / max(rho0, 1e-8)
  const float* idzc;   // nz   1/max(dzeta(k)*z_top, 1)        (mass divergence)
  const float* idzw;   // nz+1 1/max(dzeta(min(k,nz-1))*z_top, 1) (w pressure gradient)
  const float* idza;   // nz   1/(dzeta(k)*z_top)               (advection)
  const float* th0inv; // nz   1/max(theta0(k), 1)
  const float* t0d;    // 6*nz theta0(clamp(k+m)) - theta0(k), m = -3..2 (WENO shift)
  const float* spw;    // nz+1 sponge weight 1/(1+dt*alpha(min(k,nz-1))) for the current dt
  const double* spwd;  // nz+1 the same weight in FP64 (damping.cpp:94)
  const double* spdt;  // nz+1 dt*alpha(min(k,nz-1)) in FP64 (damping.cpp:98)
  const double* r0d;   // nz   rho0 (FP64)
  const double* t0dd;  // nz   theta0 (FP64)
  const double* p0d;   // nz   pi0 (FP64)
  float dx_inv, dy_inv, f0, beta, dy;
};

struct WS {          // FP32 working state (perturbation form)
  float* f[NSPECIES]; // u v w rho' theta' pi' qv qc..qg
};

// rout: when given, the tendency R is also written there (FP32)
int mixed_stage(const Dims& d, const Tab& t, const Flags& fl, const WS& win, const WS& w0, const WS& wout,
                const WS* rout, double dt_stage, unsigned* err, cudaStream_t stream);
void mixed_fb_substep(const Dims& d, const Tab& t, const Flags& fl, const WS& win, const WS& wout, float dtau,
                      cudaStream_t stream);
int mixed_hevi_substep(const Dims& d, const Tab& t, const Flags& fl, const WS& win, const WS& wout, float dtau,
                       const float* lu /* 3*nz: a, cprime, inv_denom */, unsigned* err, cudaStream_t stream);
// returns nonzero when a TMA descriptor cannot be made
int mixed_hevi_column(const Dims& d, const Tab& t, const Flags& fl, const WS& win, const WS& wout, float dtau,
                      const float* lu, bool apply_uv, unsigned* err, cudaStream_t stream);
void mixed_uv_backward(const Dims& d, const Tab& t, const WS& win, const WS& wout, float dtau, cudaStream_t stream);
// whether the column kernel chosen for this grid defers its w/rho'
// corrections to the reader (then the last substep of a stage is finished
// by mixed_uv_fix instead of mixed_uv_backward, and mixed_finish gets defer)
bool mixed_hevi_defers(const Dims& d);
// u/v backward update and the deferred w/rho' corrections, in place
void mixed_uv_fix(const Dims& d, const Tab& t, const Flags& fl, const WS& s, float dtau, cudaStream_t stream);
// adjoint of mixed_fb_substep, in place on bars of (u, v, w, rho', pi')
void mixed_fb_substep_ad(const Dims& d, const Tab& t, const WS& bar, float dtau, cudaStream_t stream);
// adjoint of mixed_hevi_substep (lu: the column factors for dtau), in place;
// bdh: nfield floats, scratch: nx*ny*(4nz+2) floats
void mixed_hevi_substep_ad(const Dims& d, const Tab& t, const Flags& fl, const WS& bar, const float* lu, float* bdh,
                           float* scratch, float dtau, cudaStream_t stream);
// uv_dtau != 0: also applies the last substep's u/v backward update (the
// in-place mixed_uv_backward launch is then left out)
void mixed_finish(const Dims& d, const Tab& t, const Flags& fl, const WS& wfin, const WS& wst, const WS& w0,
                  const WS* rin, double dt, double* const* s0, double* const* s1, unsigned* err,
                  cudaStream_t stream, float uv_dtau = 0.f, bool defer = false);
// ---- several domains per launch (work-list), mixed path, HEVI mode ----
struct MixedDomain {
  Dims d;
  Tab t;
  const float* lu;  // 3 stages x 3*nz LU factors (configured for the step's dt, n_sub)
  float* const* W0;
  float* const* WSt0;
  float* const* WSt1;
  float* const* WA;
  float* const* WB;
  float* const* WR;
  double* const* S0;  // state read by the step
  double* const* S1;  // state written by the step
};
struct MixedBatch;
// the launches of one full step of every domain (all with nz equal, the
// same flags, acoustic_mode 2); nullptr on failure
MixedBatch* mixed_batch_build(const std::vector<MixedDomain>& doms, const Flags& fl, double dt, int n_sub,
                              unsigned* err);
void mixed_batch_enqueue(const MixedBatch* b, cudaStream_t s);
int mixed_batch_launches(const MixedBatch* b);
void mixed_batch_destroy(MixedBatch* b);

void mixed_unpack_f32(const Dims& d, int nsx, int nsy, int nsz, int ni, int nj, int nk, const float* src, double* dst,
                      cudaStream_t stream);
void mixed_to_working(const Dims& d, const Tab& t, double* const* s, const WS& w, cudaStream_t stream);
// the same conversion on the columns of the box [ia, ia + ni) x [ja, ja + nj)
// (clipped to the grid)
void mixed_to_working_region(const Dims& d, const Tab& t, double* const* s, const WS& w, int ia, int ja, int ni,
                             int nj, cudaStream_t stream);
// a nest's Davies relaxation of its FP64 state s toward the boundary buffer
// bnd (first nvars fields, the weights davies[0..nzone)) fused with the FP32
// working copy of the points it changes; -1 on bad arguments
int mixed_nest_relax(const Dims& d, const Tab& t, double* const* s, const double* const* bnd, int nvars,
                     const double* davies, int nzone, const WS& w, cudaStream_t stream);

// ---- tangent-linear and adjoint of the slow tendency (step_tlad.cu) ----
// base, pert, out, bar_*: 12 fields each, model layout (plane * (nz+1)
// doubles); face: 9 * plane * (nz+1) doubles; cell_scr: plane * (nz+1).
// f32: FP32 arithmetic (mixed models), else FP64.
// out = J(base) pert, every point of every field written (0 off the boxes)
void tend_tl(const Dims& d, const Metric& m, const Flags& fl, double* const* base, double* const* pert,
             double* const* out, double* face, bool f32, cudaStream_t s);
// bar_in += J(base)^T bar_out (atomic adds)
void tend_ad(const Dims& d, const Metric& m, const Flags& fl, double* const* base, double* const* bar_out,
             double* const* bar_in, double* face, double* cell_scr, bool f32, cudaStream_t s);
// whole-array helpers: out = x0 + a r; acc += a x; conversions
void lin_axpy(size_t n, const double* x0, const double* r, double a, double* out, cudaStream_t s);
void lin_scale_add(size_t n, const double* x, double a, double* acc, cudaStream_t s);
void lin_to_f32(size_t n, const double* x, float* y, cudaStream_t s);
void lin_to_f64(size_t n, const float* x, double* y, cudaStream_t s);
// FP32 working state (perturbation form) -> FP64 total fields (species with a
// null working pointer are left as they are)
void working_to_f64(const Dims& d, const Tab& t, const WS& w, double* const* out, cudaStream_t s);

}  // namespace vgb
