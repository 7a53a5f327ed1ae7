/* include/vibe_helmholtz.h
 *
 * GB300 Helmholtz solvers: the device counterpart of the reference's
 * timeint::HelmholtzSolver family (include/vibe/time/helmholtz.hpp:57-122,
 * src/time/helmholtz.cpp:126-495). The operator is the reference's
 *     y = -div(a grad x) + b x          (apply_operator, helmholtz.cpp:173-201)
 * on cell-centred fields with arithmetic face means of a, clamped
 * neighbours (zero flux through every boundary) and
 * dz = max(dzeta(k) * (z_top - zs(i,j)), 1).
 *
 * Entry points and the reference interface each replaces:
 *   vibe_helmholtz_create        make_helmholtz_solver(kind, grid, cfg)
 *                                (helmholtz.cpp:478-494); grid = sizes,
 *                                spacings, dzeta and terrain
 *   vibe_helmholtz_set_coefficients  HelmholtzSolver::set_coefficients
 *   vibe_helmholtz_solve         HelmholtzSolver::solve(a, b, f, x)
 *   vibe_helmholtz_iterations / _residual / _name   iterations(), residual(),
 *                                name()
 *   vibe_helmholtz_set_iterative_refinement   set_iterative_refinement
 *   vibe_helmholtz_residual_l2   helmholtz_residual_l2 (helmholtz.cpp:211-227)
 * Host-pointer calls take the reference's FieldT cell storage (halo 4,
 * ((k+4)(ny+8) + (j+4))(nx+8) + (i+4)); the _dev calls take device arrays
 * of nx*ny*nz doubles, i fastest, no halo, and a stream.
 *
 * Kinds 0-2 are the reference's solvers, FP64, same iteration: 0 the
 * column tridiagonal (with a Thomas that solves its system, where the
 * reference's C Thomas does not), 1 krylov_multigrid (inside the factory's
 * iterative-refinement wrapper, max 3 refinements), 2 krylov_jacobi. The
 * reference's Jacobi-BiCGSTAB updates x with the unpreconditioned s and
 * diverges whenever the Jacobi scaling is far from 1 (the semi-implicit
 * step's operator); kinds 1 and 2 reproduce that.
 * Kinds 3-4 are this library's solvers: right-preconditioned BiCGSTAB with
 * a geometric multigrid V-cycle (vertical line Gauss-Seidel smoother,
 * horizontal coarsening), inside an FP64 iterative-refinement loop on the
 * exact operator; kind 3 runs the inner solve in FP64, kind 4 in FP32.
 * Both stop at ||f - A x||_2 / ||f||_2 < tol.
 */
#ifndef VIBE_GB300_HELMHOLTZ_H
#define VIBE_GB300_HELMHOLTZ_H

#include "vibe_c_kernels.h"

#ifdef __cplusplus
extern "C" {
#endif

enum vibe_helmholtz_kind {
  VIBE_HZ_VERTICAL_TRIDIAGONAL = 0,
  VIBE_HZ_KRYLOV_MULTIGRID = 1,
  VIBE_HZ_KRYLOV_JACOBI = 2,
  VIBE_HZ_MG_BICGSTAB_FP64 = 3,
  VIBE_HZ_MG_BICGSTAB_MIXED = 4
};

typedef struct vibe_helmholtz vibe_helmholtz;

/* dzeta: nz values (host); zs: nx*ny terrain heights (host, j-major) or
 * NULL for flat. max_iter, tol: cfg.numerics.helmholtz_max_iter / _tol
 * (reference defaults 200, 1e-8). Returns VIBE_C_OK, VIBE_C_ERR_BAD_ARG or
 * VIBE_C_ERR_DEVICE. */
int vibe_helmholtz_create(int kind, int nx, int ny, int nz, double dx, double dy, double z_top,
                          const double *dzeta, const double *zs, int max_iter, double tol,
                          vibe_helmholtz **out);
void vibe_helmholtz_destroy(vibe_helmholtz *h);

/* a, b: host FieldT cell storage. */
int vibe_helmholtz_set_coefficients(vibe_helmholtz *h, const double *a, const double *b);
/* Solve with coefficients a, b (host FieldT storage; NULL a and b keep the
 * ones set last), right-hand side f, solution x (host FieldT storage; the
 * halo of x is written with zeros, as Field::fill(0) leaves it). Returns
 * VIBE_C_OK, VIBE_C_ERR_SINGULAR (column pivot < 1e-300), VIBE_C_ERR_BAD_ARG
 * or VIBE_C_ERR_DEVICE; iterations and residual as the reference reports
 * them (NaN residual included). */
int vibe_helmholtz_solve(vibe_helmholtz *h, const double *a, const double *b, const double *f, double *x);
/* Device forms: f, x (and a, b) are nx*ny*nz device doubles, i fastest. */
int vibe_helmholtz_set_coefficients_dev(vibe_helmholtz *h, const double *a, const double *b,
                                        vibe_stream_t stream);
int vibe_helmholtz_solve_dev(vibe_helmholtz *h, const double *f, double *x, vibe_stream_t stream);
/* y = A x (device arrays), with the coefficients set last. */
int vibe_helmholtz_apply_dev(vibe_helmholtz *h, const double *x, double *y, vibe_stream_t stream);

int vibe_helmholtz_iterations(const vibe_helmholtz *h);
double vibe_helmholtz_residual(const vibe_helmholtz *h);
const char *vibe_helmholtz_name(const vibe_helmholtz *h);
/* Kind 1 only (the reference's RefinementSolver); precision is accepted
 * for interface parity (gpu::Precision, 0..3) and ignored there. */
int vibe_helmholtz_set_iterative_refinement(vibe_helmholtz *h, int on, int precision);
/* Multigrid levels used by kinds 3-4 (1 = smoother only). */
int vibe_helmholtz_levels(const vibe_helmholtz *h);
/* ||A x - f||_2 over the cells (host FieldT storage), with the coefficients
 * set last; the reference computes it the same way (helmholtz.cpp:211-227). */
double vibe_helmholtz_residual_l2(vibe_helmholtz *h, const double *f, const double *x);
/* Message of the last failure seen by this thread ("" if none). */
const char *vibe_helmholtz_last_error(void);

#ifdef __cplusplus
}
#endif

#endif
