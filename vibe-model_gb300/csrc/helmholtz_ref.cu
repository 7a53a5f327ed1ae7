// vibe-model_gb300/csrc/helmholtz_ref.cu
//
// FP64 kernels of the reference's Helmholtz solvers, in the reference's
// operation order. Built with --fmad=false (no FMA contraction), so the
// operator, the Jacobi scaling and the column solve give the bits of the
// reference's serial loops; only reductions differ in summation order.
#include "helmholtz.cuh"

namespace vgb {
namespace {

constexpr int kT = 256;

__device__ __forceinline__ size_t hix(const HGeo& g, int i, int j, int k) {
  return ((size_t)k * g.ny + j) * (size_t)g.nx + i;
}

// apply_operator, helmholtz.cpp:173-201: y = -fx - fy - fz + b x with
// ae = (a + a.clamp_at(i+1))/2 ... and dz = max(dzeta(k)(z_top - zs), 1)
template <bool kResidual>
__global__ void k_apply_ref(HGeo g, const double* __restrict__ a, const double* __restrict__ b,
                            const double* __restrict__ x, const double* __restrict__ f, double* __restrict__ y) {
  const size_t n = g.n();
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(c % g.nx);
    const size_t cj = c / g.nx;
    const int j = (int)(cj % g.ny), k = (int)(cj / g.ny);
    const double dx = g.dx, dy = g.dy;
    const double dz = dmax(g.dzeta[k] * g.scale[(size_t)j * g.nx + i], 1.0);
    const size_t ie = hix(g, imin(i + 1, g.nx - 1), j, k), iw = hix(g, imax(i - 1, 0), j, k);
    const size_t in = hix(g, i, imin(j + 1, g.ny - 1), k), is = hix(g, i, imax(j - 1, 0), k);
    const size_t it = hix(g, i, j, imin(k + 1, g.nz - 1)), ib = hix(g, i, j, imax(k - 1, 0));
    const double ac = a[c];
    const double ae = 0.5 * (ac + a[ie]);
    const double aw = 0.5 * (ac + a[iw]);
    const double an = 0.5 * (ac + a[in]);
    const double as = 0.5 * (ac + a[is]);
    const double at = 0.5 * (ac + a[it]);
    const double ab = 0.5 * (ac + a[ib]);
    const double xc = x[c];
    const double fx = (ae * (x[ie] - xc) - aw * (xc - x[iw])) / (dx * dx);
    const double fy = (an * (x[in] - xc) - as * (xc - x[is])) / (dy * dy);
    const double fz = (at * (x[it] - xc) - ab * (xc - x[ib])) / (dz * dz);
    const double ax = -fx - fy - fz + b[c] * xc;
    y[c] = kResidual ? f[c] - ax : ax;
  }
}

// KrylovJacobiSolver's preconditioner, helmholtz.cpp:304-314
__global__ void k_jacobi_prec(HGeo g, const double* __restrict__ a, const double* __restrict__ b,
                              double* __restrict__ prec) {
  const size_t n = g.n();
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(c % g.nx);
    const size_t cj = c / g.nx;
    const int j = (int)(cj % g.ny), k = (int)(cj / g.ny);
    const double dx = g.dx, dy = g.dy;
    const double dz = dmax(g.dzeta[k] * g.scale[(size_t)j * g.nx + i], 1.0);
    const double ac = a[c];
    const double diag = 2.0 * ac / (dx * dx) + 2.0 * ac / (dy * dy) + 2.0 * ac / (dz * dz) + b[c];
    prec[c] = 1.0 / dmax(diag, 1e-30);
  }
}

// VerticalTridiagonalSolver::solve, helmholtz.cpp:241-274: one thread per
// column; the system of each column is solved with the recurrence of
// thomas_solve (helmholtz.cpp:71-85) as the documented C contract demands
__global__ void k_vertical(HGeo g, const double* __restrict__ a, const double* __restrict__ b,
                           const double* __restrict__ f, double* __restrict__ x, double* __restrict__ ws,
                           unsigned* err) {
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= g.nx * g.ny) return;
  const int nz = g.nz;
  const size_t pl = (size_t)g.nx * g.ny;
  const double scale = g.scale[col];
  auto coefs = [&](int k, double& sa, double& sb, double& sc) {
    const double dz = dmax(g.dzeta[k] * scale, 1.0);
    const size_t c = (size_t)k * pl + col;
    const double ac = a[c];
    const double az = 0.5 * (ac + a[(size_t)imin(k + 1, nz - 1) * pl + col]);
    const double azm = 0.5 * (ac + a[(size_t)imax(k - 1, 0) * pl + col]);
    sb = (az + azm) / (dz * dz) + b[c];
    sa = -azm / (dz * dz);
    sc = -az / (dz * dz);
  };
  double sa, sb, sc;
  coefs(0, sa, sb, sc);
  if (nz == 1) {
    if (sb == 0.0) { atomicOr(err, (unsigned)kErrSingular); return; }
    x[col] = f[col] / sb;
    return;
  }
  double denom = sb;
  if (denom == 0.0) { atomicOr(err, (unsigned)kErrSingular); return; }
  double wprev = sc / denom, xprev = f[col] / denom;
  ws[col] = wprev;
  x[col] = xprev;
  for (int k = 1; k < nz; ++k) {
    coefs(k, sa, sb, sc);
    const size_t c = (size_t)k * pl + col;
    denom = sb - sa * wprev;
    if (denom == 0.0) { atomicOr(err, (unsigned)kErrSingular); return; }
    xprev = (f[c] - sa * xprev) / denom;
    x[c] = xprev;
    if (k < nz - 1) {
      wprev = sc / denom;
      ws[c] = wprev;
    }
  }
  double xn = xprev;
  for (int k = nz - 1; k-- > 0;) {
    const size_t c = (size_t)k * pl + col;
    xn = x[c] - ws[c] * xn;
    x[c] = xn;
  }
}

// two-level deterministic dot product
__global__ void k_dot_part(const double* __restrict__ x, const double* __restrict__ y, size_t n, double* part) {
  __shared__ double sh[kT];
  double s = 0.0;
  for (size_t q = blockIdx.x * (size_t)kT + threadIdx.x; q < n; q += (size_t)gridDim.x * kT) s += x[q] * y[q];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = kT / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void k_dot_final(const double* __restrict__ part, int nb, double* out) {
  __shared__ double sh[kT];
  double s = 0.0;
  for (int q = threadIdx.x; q < nb; q += kT) s += part[q];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = kT / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sh[0];
}

#define VOP_LOOP for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x)
__global__ void k_sub(const double* f, const double* v, double* r, size_t n) { VOP_LOOP r[q] = f[q] - v[q]; }
__global__ void k_mul(const double* p, const double* r, double* o, size_t n) { VOP_LOOP o[q] = p[q] * r[q]; }
__global__ void k_pupd(const double* rh, double* p, const double* v, double beta, double omega, size_t n) {
  VOP_LOOP p[q] = rh[q] + beta * (p[q] - omega * v[q]);
}
__global__ void k_axpy_to(const double* r, const double* v, double alpha, double* s, size_t n) {
  VOP_LOOP s[q] = r[q] - alpha * v[q];
}
__global__ void k_xadd1(double* x, const double* p, double alpha, size_t n) { VOP_LOOP x[q] += alpha * p[q]; }
__global__ void k_xadd2(double* x, const double* p, const double* s, double alpha, double omega, size_t n) {
  VOP_LOOP x[q] += alpha * p[q] + omega * s[q];
}
__global__ void k_add(double* x, const double* d, size_t n) { VOP_LOOP x[q] += d[q]; }
#undef VOP_LOOP

int grid_for(size_t n) {
  const size_t b = (n + kT - 1) / kT;
  return (int)(b < 4096 ? (b > 0 ? b : 1) : 4096);
}

}  // namespace

void hz_apply_ref(const HGeo& g, const double* a, const double* b, const double* x, double* y, cudaStream_t s) {
  k_apply_ref<false><<<grid_for(g.n()), kT, 0, s>>>(g, a, b, x, nullptr, y);
}
void hz_residual_ref(const HGeo& g, const double* a, const double* b, const double* f, const double* x, double* r,
                     cudaStream_t s) {
  k_apply_ref<true><<<grid_for(g.n()), kT, 0, s>>>(g, a, b, x, f, r);
}
void hz_jacobi_prec(const HGeo& g, const double* a, const double* b, double* prec, cudaStream_t s) {
  k_jacobi_prec<<<grid_for(g.n()), kT, 0, s>>>(g, a, b, prec);
}
void hz_vertical_solve(const HGeo& g, const double* a, const double* b, const double* f, double* x, double* cp,
                       double* dp, unsigned* err, cudaStream_t s) {
  (void)dp;
  const int cols = g.nx * g.ny;
  k_vertical<<<(cols + 127) / 128, 128, 0, s>>>(g, a, b, f, x, cp, err);
}
void dot64(const double* x, const double* y, size_t n, double* partials, double* out, cudaStream_t s) {
  int nb = (int)((n + kT - 1) / kT);
  nb = nb < kRedBlocks ? (nb > 0 ? nb : 1) : kRedBlocks;
  k_dot_part<<<nb, kT, 0, s>>>(x, y, n, partials);
  k_dot_final<<<1, kT, 0, s>>>(partials, nb, out);
}
void vop_sub(const double* f, const double* v, double* r, size_t n, cudaStream_t s) {
  k_sub<<<grid_for(n), kT, 0, s>>>(f, v, r, n);
}
void vop_mul(const double* p, const double* r, double* o, size_t n, cudaStream_t s) {
  k_mul<<<grid_for(n), kT, 0, s>>>(p, r, o, n);
}
void vop_pupdate(const double* rh, double* p, const double* v, double beta, double omega, size_t n, cudaStream_t s) {
  k_pupd<<<grid_for(n), kT, 0, s>>>(rh, p, v, beta, omega, n);
}
void vop_axpy_to(const double* r, const double* v, double alpha, double* s_, size_t n, cudaStream_t s) {
  k_axpy_to<<<grid_for(n), kT, 0, s>>>(r, v, alpha, s_, n);
}
void vop_xadd1(double* x, const double* p, double alpha, size_t n, cudaStream_t s) {
  k_xadd1<<<grid_for(n), kT, 0, s>>>(x, p, alpha, n);
}
void vop_xadd2(double* x, const double* p, const double* s_, double alpha, double omega, size_t n, cudaStream_t s) {
  k_xadd2<<<grid_for(n), kT, 0, s>>>(x, p, s_, alpha, omega, n);
}
void vop_add(double* x, const double* d, size_t n, cudaStream_t s) { k_add<<<grid_for(n), kT, 0, s>>>(x, d, n); }

}  // namespace vgb
