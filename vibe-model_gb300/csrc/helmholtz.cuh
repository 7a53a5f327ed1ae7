// vibe-model_gb300/csrc/helmholtz.cuh
//
// Device side of the Helmholtz solvers (include/vibe_helmholtz.h).
// Layout: cell fields of nx*ny*nz values, idx = (k*ny + j)*nx + i.
#pragma once
#include <cuda_runtime.h>

#include "vibe_internal.cuh"

namespace vgb {

struct HGeo {
  int nx, ny, nz;
  double dx, dy;
  const double* dzeta;  // nz
  const double* scale;  // nx*ny: z_top - zs(i,j)
  __host__ __device__ size_t n() const { return (size_t)nx * ny * nz; }
};

// ---- FP64 kernels with the reference's operation order (compiled without
// FMA contraction: helmholtz_ref.cu) ----
void hz_apply_ref(const HGeo& g, const double* a, const double* b, const double* x, double* y, cudaStream_t s);
// r = f - A x
void hz_residual_ref(const HGeo& g, const double* a, const double* b, const double* f, const double* x, double* r,
                     cudaStream_t s);
void hz_jacobi_prec(const HGeo& g, const double* a, const double* b, double* prec, cudaStream_t s);
// column tridiagonal solve of VerticalTridiagonalSolver; cp, dp: n scratch
void hz_vertical_solve(const HGeo& g, const double* a, const double* b, const double* f, double* x, double* cp,
                       double* dp, unsigned* err, cudaStream_t s);

// ---- deterministic FP64 reductions: sum over n of x*y (y may equal x) into
// out[slot]; partials: >= kRedBlocks doubles per slot ----
constexpr int kRedBlocks = 456;  // 3 x 152 SMs
void dot64(const double* x, const double* y, size_t n, double* partials, double* out, cudaStream_t s);

// elementwise FP64 vector ops of the reference's Jacobi BiCGSTAB
// (helmholtz.cpp:318-361); scalars by value
void vop_sub(const double* f, const double* v, double* r, size_t n, cudaStream_t s);                 // r = f - v
void vop_mul(const double* p, const double* r, double* o, size_t n, cudaStream_t s);                 // o = p*r
void vop_pupdate(const double* rh, double* p, const double* v, double beta, double omega, size_t n,
                 cudaStream_t s);                                                                    // p = rh + beta*(p - omega*v)
void vop_axpy_to(const double* r, const double* v, double alpha, double* s_, size_t n, cudaStream_t s); // s = r - alpha*v
void vop_xadd1(double* x, const double* p, double alpha, size_t n, cudaStream_t s);                  // x += alpha*p
void vop_xadd2(double* x, const double* p, const double* s_, double alpha, double omega, size_t n,
               cudaStream_t s);                                                                      // x += alpha*p + omega*s
void vop_add(double* x, const double* d, size_t n, cudaStream_t s);                                  // x += d

// ---- multigrid-preconditioned BiCGSTAB (helmholtz_mg.cu), T = float/double ----
template <typename T>
struct MgSolver;
template <typename T>
MgSolver<T>* mg_create(const HGeo& g, int max_levels);
template <typename T>
void mg_destroy(MgSolver<T>* m);
template <typename T>
int mg_levels(const MgSolver<T>* m);
// builds every level's couplings and column factors from the FP64 a, b
template <typename T>
int mg_set_coefficients(MgSolver<T>* m, const double* a, const double* b, cudaStream_t s);
// approximately solves A d = r64 / scale (FP64 in, FP64 out scaled back):
// BiCGSTAB in T to relative tolerance rtol or max_iter iterations.
// r_norm2: (r64, r64) when the caller has it, else negative (computed here).
// Returns the iterations done (negative on breakdown).
template <typename T>
int mg_solve(MgSolver<T>* m, const double* r64, double* d64, double rtol, int max_iter, cudaStream_t s,
             double r_norm2 = -1.0);

}  // namespace vgb
