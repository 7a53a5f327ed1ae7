/* include/vibe_tlad.h
 *
 * Tangent-linear and adjoint model on the GPU, replacing the reference's
 * da::TangentLinearModel / da::AdjointModel (include/vibe/da/
 * tangent_linear.hpp:80-150, src/da/tangent_linear.cpp:72-603): the TL of a
 * collocated, 2nd-order, interior-points RK3 linearised about a base state
 * xb held fixed over each step, and its exact transpose.
 *   vibe_tlad_create / set_base   TangentLinearModel / AdjointModel ctor and
 *                                 the linearisation point xb
 *   vibe_tl_step                  TangentLinearModel::step (rk3_tl)
 *   vibe_tl_propagate             TangentLinearModel::propagate (xb frozen
 *                                 over all n_steps, as the reference does)
 *   vibe_ad_step                  AdjointModel::step_adjoint (rk3_ad)
 *   vibe_ad_propagate             AdjointModel::propagate_with_trajectory over
 *                                 the trajectory propagate records (n_steps
 *                                 copies of xb)
 *   vibe_tl_tendency / vibe_ad_tendency   tendency_tl / tendency_ad (the latter
 *                                 accumulates into bar_dx, as the reference)
 * States are the 12 species (dyn::Species order) in FieldT storage, host
 * pointers; halo points pass through unchanged. dt is explicit: the
 * reference's propagate_with_trajectory takes dt from the trajectory's time
 * stamps and falls back to 1 for a single step.
 * precision 0: FP64; 1: FP32 arithmetic with FP64 storage and stage sums.
 * Returns VIBE_C_OK, VIBE_C_ERR_BAD_ARG or VIBE_C_ERR_DEVICE.
 */
#ifndef VIBE_GB300_TLAD_H
#define VIBE_GB300_TLAD_H

#include "vibe_c_kernels.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct vibe_tlad vibe_tlad;

/* grid: sizes, spacings, dzeta (nz, host), terrain zs (nx*ny, host) or NULL */
int vibe_tlad_create(int nx, int ny, int nz, double dx, double dy, double z_top, const double *dzeta,
                     const double *zs, int precision, vibe_tlad **out);
void vibe_tlad_destroy(vibe_tlad *t);
int vibe_tlad_set_base(vibe_tlad *t, const double *const *xb);

int vibe_tl_tendency(vibe_tlad *t, const double *const *dx, double *const *d);
int vibe_ad_tendency(vibe_tlad *t, const double *const *bar_d, double *const *bar_dx);
int vibe_tl_step(vibe_tlad *t, double dt, const double *const *dx, double *const *dx_out);
int vibe_tl_propagate(vibe_tlad *t, double dt, int n_steps, const double *const *dx0, double *const *dx_out);
int vibe_ad_step(vibe_tlad *t, double dt, const double *const *dx_next, double *const *dx_prev);
int vibe_ad_propagate(vibe_tlad *t, double dt, int n_steps, const double *const *dy, double *const *dx0_adjoint);
/* The nonlinear collocated RK3 whose tangent-linear model is the one above
 * (nl_rk3 / nl_tendency of the reference's TL/AD test, tests/unit/
 * test_tl_ad.cpp:100-199; the buoyancy uses the set base's theta): the
 * model of the finite-difference check of the TL (check_tangent,
 * tangent_linear.cpp:832-880). */
int vibe_nl_propagate(vibe_tlad *t, double dt, int n_steps, const double *const *x0, double *const *x_out);
/* its tendency N(x): vibe_tl_tendency is the exact derivative of N at the base */
int vibe_nl_tendency(vibe_tlad *t, const double *const *x, double *const *d);

/* Message of the last failure seen by this thread ("" if none). */
const char *vibe_tlad_last_error(void);

#ifdef __cplusplus
}
#endif

#endif
