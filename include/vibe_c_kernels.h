/* include/vibe_c_kernels.h
 *
 * Drop-in replacement for the reference's C11 hot-kernel ABI
 * (include/vibe/common/c_kernels.h:29-117): same symbol names, argument
 * meaning, NULL handling and return codes, so a caller linked against the
 * reference's libvibe links against libvibe_gb300.so unchanged. The work runs
 * on the GPU (sm_103a): the host-pointer entry points stage their arrays
 * through device memory on an internal stream; the *_dev entry points take
 * device pointers and a stream and never copy.
 *
 * Conventions kept from c_kernels.h:13-19: scalars double (float in the
 * *_f32 twins, h:15-16); errors are
 * return codes, never errno; no global state visible to the caller.
 * Differences, each deliberate:
 *   - vibe_tridiagonal_solve_f64 solves the system its contract documents
 *     (c_kernels.h:38-55). The shipped c_kernels.c:18-60 does not: on the
 *     reference's own test matrix diag(1,-4,1) it leaves a residual of 9e-2.
 *   - device failures return VIBE_C_ERR_DEVICE (new code 3); void/double
 *     functions report them through vibe_c_last_error().
 * No allocation per call and reentrancy (c_kernels.h:17-18): every host
 * thread owns, per device, a stream and staging buffers (pinned host,
 * device) that grow on demand and are reused; a host-pointer call packs its
 * inputs into the pinned buffer, makes one host-to-device copy, runs, makes
 * one copy back and waits for its own stream only. After a thread's first
 * calls of a given size its calls allocate nothing (vibe_c_allocations()
 * counts every allocation this layer makes). A host-pointer call costs a
 * launch and two copies (tens of microseconds), so callers with many small
 * systems use the batched or _dev forms. The caller's ws is accepted as the
 * reference requires and left unused: the device workspace is the thread's.
 */
#ifndef VIBE_GB300_C_KERNELS_H
#define VIBE_GB300_C_KERNELS_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VIBE_C_OK 0
#define VIBE_C_ERR_SINGULAR 1
#define VIBE_C_ERR_BAD_ARG 2
#define VIBE_C_ERR_DEVICE 3

typedef struct CUstream_st *vibe_stream_t; /* == cudaStream_t */

/* Replaces c_kernels.h:54-55 (vibe_tridiagonal_solve_f64). Solves
 * a[k] x[k-1] + b[k] x[k] + c[k] x[k+1] = d[k], k = 0..n-1; a, c have n-1
 * entries (a[k-1] is row k's sub-diagonal) and may be NULL (= 0). ws (n) is
 * caller workspace, as in the reference; its contents on return are
 * unspecified. Returns VIBE_C_OK, VIBE_C_ERR_SINGULAR on a zero pivot,
 * VIBE_C_ERR_BAD_ARG, or VIBE_C_ERR_DEVICE; x is written only on VIBE_C_OK
 * (as the reference, which returns before it writes x). */
int vibe_tridiagonal_solve_f64(const double *a, const double *b, const double *c,
                               const double *d, int n, double *x, double *ws);

/* Replaces c_kernels.h:65-66. WENO5 left/right face reconstruction
 * (d = 0.1/0.6/0.3, eps = 1e-6). Silently returns when an output is NULL. */
void vibe_weno5_reconstruct_f64(double qm2, double qm1, double q0, double q1,
                                double q2, double *q_left, double *q_right);

/* Replaces c_kernels.h:77-78. Bilinear sample of a halo'd FieldT-layout
 * array at fractional cell index (xi, yj), level k, clamped to the interior
 * in the reference's order (up to 0, then down to n-1: a grid without
 * interior points reads its last halo point). Returns 0 for NULL f or
 * nz <= 0; NaN (vibe_c_last_error() says why) for halo < 0 or a plane
 * narrower than halo + 1, where the reference reads outside the plane. */
double vibe_bilinear_f64(const double *f, int halo, int nsx, int nsy, int nz,
                         double xi, double yj, int k);

/* Replaces c_kernels.h:89-92. Max over cells of
 * dt*(|u|/dx + |v|/dy + |w|/max(dzeta[k]*(z_top - zs), 1)); also the max wind
 * speed and the min dz (0 when none). zs may be NULL (flat). Returns 0 when
 * u, v, w or dzeta is NULL (outputs untouched), and 0 with both outputs 0 on
 * a grid with nx, ny or nz <= 0 (no cells). */
double vibe_cfl_scan_f64(const double *u, const double *v, const double *w,
                         const double *dzeta, const double *zs, int nx, int ny,
                         int nz, double dx, double dy, double z_top, double dt,
                         double *max_wind_out, double *min_dz_out);

/* Replaces c_kernels.h:101. Compensated (Neumaier) sum of n doubles. The
 * device reduction compensates per thread, per warp and across blocks, so the
 * result carries the same O(eps) error bound as the serial loop (not the same
 * bits). Returns 0 for NULL x. */
double vibe_neumaier_sum_f64(const double *x, size_t n);

/* Replaces c_kernels.h:113-117. Second-order flux-form advection on
 * collocated, halo-free, i-fastest arrays, periodic in x and y, zero vertical
 * flux on the first and last level. Silently returns on NULL arguments and on
 * a grid with nx, ny or nz <= 0 (dqdt untouched). */
void vibe_advect_scalar_flux_f64(const double *q, const double *rho,
                                 const double *u, const double *v, const double *w,
                                 const double *dzeta, const double *zs, int nx,
                                 int ny, int nz, double dx, double dy,
                                 double z_top, double *dqdt);

/* ---- device-pointer and batched forms (no reference counterpart; the same
 * arithmetic as the host entry points above) ---- */

/* n_sys independent systems of size n, each stored contiguously
 * (system s uses a + s*(n-1), b + s*n, ...). One thread per system for
 * n <= 128; above, one warp per system (each lane eliminates a chunk of rows,
 * the chunks' end unknowns are joined by a 2x2 block-tridiagonal solve),
 * whose results agree with the single sweep to rounding. A system whose chunk
 * pivots or interface blocks are zero or tiny (b[r0] = 0 at a chunk start,
 * non-dominant diagonals) is solved again with the single sweep, so the error
 * contract stays the reference's: VIBE_C_ERR_SINGULAR only on an exactly zero
 * sweep pivot (c_kernels.c:26,34,40).
 * status (device, n_sys ints) receives the per-system return code; may be
 * NULL. Returns VIBE_C_OK or VIBE_C_ERR_BAD_ARG/VIBE_C_ERR_DEVICE (launch).
 * Scratch (n*n_sys doubles, 3x for n > 128) comes from a buffer owned by
 * the calling host thread: after its first calls of a size it allocates
 * nothing, and calls of one thread on different streams are ordered through
 * it (the later waits for the earlier), so they never share it while one
 * runs. Under stream capture the scratch is a stream-ordered allocation of
 * the graph instead. */
int vibe_tridiagonal_solve_batched_f64_dev(const double *a, const double *b,
                                           const double *c, const double *d,
                                           int n, int n_sys, double *x,
                                           int *status, vibe_stream_t stream);
/* Allocation-free form of vibe_tridiagonal_solve_batched_f64_dev; it has no
 * counterpart in the reference. For callers that may not allocate device
 * memory (a host model whose own allocator owns the device memory, or a
 * time-critical loop where cudaMalloc/cudaFree would synchronise the device):
 * the per-system workspace lives in a fixed device array of 2^18 doubles
 * (2 MiB, held on every GPU that loads the library until exit), so
 * n * n_sys must not exceed 262144 (larger requests return
 * VIBE_C_ERR_BAD_ARG; vibe_c_last_error() says why). Inputs and outputs are
 * device pointers as in the _dev form. The first call on each device
 * resolves the array's device address (cudaGetSymbolAddress) and keeps it for
 * the life of the process; make that first call before any stream capture,
 * and do not call this form on a device after cudaDeviceReset of it. It runs
 * the one-thread-per-system sweep for every n, so for n > 128 it agrees with
 * the _dev form to rounding (and reports VIBE_C_ERR_SINGULAR on the sweep's
 * exact-zero pivot only). All calls share the one array:
 * calls whose kernels can overlap on the GPU (different streams, no
 * ordering between them) race on it. */
int vibe_tridiagonal_solve_batched_f64_dev_noalloc(const double *a, const double *b,
                                                   const double *c, const double *d,
                                                   int n, int n_sys, double *x,
                                                   int *status, vibe_stream_t stream);
/* Host-pointer batched form; returns the first non-zero per-system code and
 * writes x only for the systems that solved. */
int vibe_tridiagonal_solve_batched_f64(const double *a, const double *b,
                                       const double *c, const double *d, int n,
                                       int n_sys, double *x);
/* Batched WENO5: q holds 5*n values (stencils q[5e..5e+4]). */
int vibe_weno5_reconstruct_batched_f64_dev(const double *q, size_t n,
                                           double *q_left, double *q_right,
                                           vibe_stream_t stream);
/* The CFL scan and the flux advection on device pointers: VIBE_C_ERR_BAD_ARG
 * for a negative dimension; a grid with a zero dimension gives (0, 0, 0) in
 * out3 and leaves dqdt untouched. n = 0 sums to 0. */
int vibe_cfl_scan_f64_dev(const double *u, const double *v, const double *w,
                          const double *dzeta, const double *zs, int nx, int ny,
                          int nz, double dx, double dy, double z_top, double dt,
                          double *out3 /* device: cfl, max_wind, min_dz */,
                          vibe_stream_t stream);
int vibe_neumaier_sum_f64_dev(const double *x, size_t n, double *out /* device */,
                              vibe_stream_t stream);
int vibe_advect_scalar_flux_f64_dev(const double *q, const double *rho,
                                    const double *u, const double *v,
                                    const double *w, const double *dzeta,
                                    const double *zs, int nx, int ny, int nz,
                                    double dx, double dy, double z_top,
                                    double *dqdt, vibe_stream_t stream);

/* ---- FP32 twins: the *_f32 names c_kernels.h:15-16 reserves for the
 * single-precision build (the reference declares none). Same contracts as
 * the FP64 functions above, arithmetic and storage in float. ---- */
int vibe_tridiagonal_solve_f32(const float *a, const float *b, const float *c,
                               const float *d, int n, float *x, float *ws);
void vibe_weno5_reconstruct_f32(float qm2, float qm1, float q0, float q1,
                                float q2, float *q_left, float *q_right);
float vibe_bilinear_f32(const float *f, int halo, int nsx, int nsy, int nz,
                        float xi, float yj, int k);
float vibe_cfl_scan_f32(const float *u, const float *v, const float *w,
                        const float *dzeta, const float *zs, int nx, int ny,
                        int nz, float dx, float dy, float z_top, float dt,
                        float *max_wind_out, float *min_dz_out);
float vibe_neumaier_sum_f32(const float *x, size_t n);
void vibe_advect_scalar_flux_f32(const float *q, const float *rho,
                                 const float *u, const float *v, const float *w,
                                 const float *dzeta, const float *zs, int nx,
                                 int ny, int nz, float dx, float dy,
                                 float z_top, float *dqdt);
int vibe_tridiagonal_solve_batched_f32(const float *a, const float *b,
                                       const float *c, const float *d, int n,
                                       int n_sys, float *x);
int vibe_tridiagonal_solve_batched_f32_dev(const float *a, const float *b,
                                           const float *c, const float *d,
                                           int n, int n_sys, float *x,
                                           int *status, vibe_stream_t stream);
int vibe_weno5_reconstruct_batched_f32_dev(const float *q, size_t n,
                                           float *q_left, float *q_right,
                                           vibe_stream_t stream);
int vibe_cfl_scan_f32_dev(const float *u, const float *v, const float *w,
                          const float *dzeta, const float *zs, int nx, int ny,
                          int nz, float dx, float dy, float z_top, float dt,
                          float *out3, vibe_stream_t stream);
int vibe_neumaier_sum_f32_dev(const float *x, size_t n, float *out,
                              vibe_stream_t stream);
int vibe_advect_scalar_flux_f32_dev(const float *q, const float *rho,
                                    const float *u, const float *v,
                                    const float *w, const float *dzeta,
                                    const float *zs, int nx, int ny, int nz,
                                    float dx, float dy, float z_top,
                                    float *dqdt, vibe_stream_t stream);

/* ---- tangent-linear and adjoint of the flux advection (no reference
 * counterpart; for the incremental 4D-Var built on this ABI) ----
 * TL: d_dqdt = the derivative of vibe_advect_scalar_flux_f64's dqdt at
 * (q, rho, u, v, w) applied to (dq, drho, du, dv, dw): every face flux
 * vel*Rbar*Qbar differentiated in all three factors, and the density
 * divisor where rho > 1e-12 (the 1e-12 floor is constant). AD: its
 * transpose applied to bar_dqdt, ADDED to bar_q, bar_rho, bar_u, bar_v,
 * bar_w (as the reference's adjoint kernels accumulate, tangent_linear.cpp:
 * 426-546). Arrays as in the forward function; returns VIBE_C_OK,
 * VIBE_C_ERR_BAD_ARG or VIBE_C_ERR_DEVICE. */
int vibe_advect_scalar_flux_tl_f64(const double *q, const double *rho, const double *u, const double *v,
                                   const double *w, const double *dq, const double *drho, const double *du,
                                   const double *dv, const double *dw, const double *dzeta, const double *zs, int nx,
                                   int ny, int nz, double dx, double dy, double z_top, double *d_dqdt);
int vibe_advect_scalar_flux_ad_f64(const double *q, const double *rho, const double *u, const double *v,
                                   const double *w, const double *bar_dqdt, const double *dzeta, const double *zs,
                                   int nx, int ny, int nz, double dx, double dy, double z_top, double *bar_q,
                                   double *bar_rho, double *bar_u, double *bar_v, double *bar_w);
int vibe_advect_scalar_flux_tl_f64_dev(const double *q, const double *rho, const double *u, const double *v,
                                       const double *w, const double *dq, const double *drho, const double *du,
                                       const double *dv, const double *dw, const double *dzeta, const double *zs,
                                       int nx, int ny, int nz, double dx, double dy, double z_top, double *d_dqdt,
                                       vibe_stream_t stream);
int vibe_advect_scalar_flux_ad_f64_dev(const double *q, const double *rho, const double *u, const double *v,
                                       const double *w, const double *bar_dqdt, const double *dzeta, const double *zs,
                                       int nx, int ny, int nz, double dx, double dy, double z_top, double *bar_q,
                                       double *bar_rho, double *bar_u, double *bar_v, double *bar_w,
                                       vibe_stream_t stream);
int vibe_advect_scalar_flux_tl_f32(const float *q, const float *rho, const float *u, const float *v, const float *w,
                                   const float *dq, const float *drho, const float *du, const float *dv,
                                   const float *dw, const float *dzeta, const float *zs, int nx, int ny, int nz,
                                   float dx, float dy, float z_top, float *d_dqdt);
int vibe_advect_scalar_flux_ad_f32(const float *q, const float *rho, const float *u, const float *v, const float *w,
                                   const float *bar_dqdt, const float *dzeta, const float *zs, int nx, int ny, int nz,
                                   float dx, float dy, float z_top, float *bar_q, float *bar_rho, float *bar_u,
                                   float *bar_v, float *bar_w);

/* Message of the last device failure seen by this thread ("" if none). */
const char *vibe_c_last_error(void);

/* Number of device and pinned-host allocations (cudaMalloc, cudaMallocHost)
 * the C-ABI layer has made in this process, over all threads and devices; it
 * stops growing once every calling thread's buffers fit its calls. No
 * reference counterpart: it makes the no-allocation convention of
 * c_kernels.h:17 checkable. */
unsigned long long vibe_c_allocations(void);

#ifdef __cplusplus
}
#endif

#endif
