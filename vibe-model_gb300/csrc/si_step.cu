// vibe-model_gb300/csrc/si_step.cu
//
// Pointwise kernels of the semi-implicit step (O-SI), built without FMA
// contraction so they give the bits of the reference's serial loops:
//   * assembly of the Helmholtz problem, SemiImplicitIntegrator::
//     assemble_rhs (src/time/semi_implicit.cpp:56-106):
//       a = (dt/2)^2 (Rd/cv) pi0 cp theta0,  b = 1,
//       f = pi - dt c G + div_h(a0 grad pi),  c = (Rd/cv) pi0 / max(rho0, 1e-8),
//       G = div(rho0 u^n) + (dt/2) div(rho0 N_u)  (unclamped i+1/j+1/k+1 face
//       reads, clamped rho0), written in the Helmholtz solver's layout;
//   * the explicit update x += dt R of theta, qv, rho and the moisture species
//     (semi_implicit.cpp:194-200; FieldT::add_scaled, field.hpp:108-111).
#include "helmholtz.cuh"
#include "step_kernels.cuh"

namespace vgb {
namespace {

__global__ void k_si_assemble(Dims d, Metric met, const double* __restrict__ u, const double* __restrict__ v,
                              const double* __restrict__ w, const double* __restrict__ pi,
                              const double* __restrict__ nu, const double* __restrict__ nv,
                              const double* __restrict__ nw, double dt, double* __restrict__ a,
                              double* __restrict__ b, double* __restrict__ f) {
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const size_t n = (size_t)nx * ny * nz;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(q % nx);
    const size_t qj = q / nx;
    const int j = (int)(qj % ny), k = (int)(qj / ny);
    const double half_dt = 0.5 * dt;
    const size_t c = d.idx(i, j, k);
    const double a0 = half_dt * half_dt * (kRd / kCv) * met.pi0[c] * kCp * met.th0[c];
    a[q] = a0;
    b[q] = 1.0;
    const double dx = met.dx, dy = met.dy;
    const double dz = dmax(met.dzeta[k] * met.scale[(size_t)j * nx + i], 1.0);
    const double* r0 = met.rho0;
    const double rc = r0[c];
    const double rE = r0[d.idx(imin(i + 1, nx - 1), j, k)], rW = r0[d.idx(imax(i - 1, 0), j, k)];
    const double rN = r0[d.idx(i, imin(j + 1, ny - 1), k)], rS = r0[d.idx(i, imax(j - 1, 0), k)];
    const double rT = r0[d.idx(i, j, imin(k + 1, nz - 1))], rB = r0[d.idx(i, j, imax(k - 1, 0))];
    const size_t ce = d.idx(i + 1, j, k), cn = d.idx(i, j + 1, k), ct = d.idx(i, j, k + 1);
    auto flux_div = [&](const double* U, const double* V, const double* W) {
      const double fx = U[ce] * 0.5 * (rc + rE) - U[c] * 0.5 * (rW + rc);
      const double fy = V[cn] * 0.5 * (rc + rN) - V[c] * 0.5 * (rS + rc);
      const double fz = W[ct] * 0.5 * (rc + rT) - W[c] * 0.5 * (rB + rc);
      return fx / dx + fy / dy + fz / dz;
    };
    const double G = flux_div(u, v, w) + half_dt * flux_div(nu, nv, nw);
    const double cc = (kRd / kCv) * (met.pi0[c] / dmax(rc, 1e-8));
    const double pc = pi[c];
    const double div_a_grad =
        (a0 * (pi[d.idx(imin(i + 1, nx - 1), j, k)] - pc) - a0 * (pc - pi[d.idx(imax(i - 1, 0), j, k)])) / (dx * dx) +
        (a0 * (pi[d.idx(i, imin(j + 1, ny - 1), k)] - pc) - a0 * (pc - pi[d.idx(i, imax(j - 1, 0), k)])) / (dy * dy);
    f[q] = pc - dt * cc * G + div_a_grad;
  }
}

// x += a y over the cells (the halo and ghost line of a tendency are zero)
__global__ void k_cells_add_scaled(Dims d, double* __restrict__ x, const double* __restrict__ y, double a) {
  const size_t n = (size_t)d.nx * d.ny * d.nz;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(q % d.nx);
    const size_t qj = q / d.nx;
    const size_t c = d.idx(i, (int)(qj % d.ny), (int)(qj / d.ny));
    x[c] += a * y[c];
  }
}

// device layout of the solver (nx*ny*nz) -> model cell layout
__global__ void k_to_cells(Dims d, const double* __restrict__ in, double* __restrict__ out) {
  const size_t n = (size_t)d.nx * d.ny * d.nz;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(q % d.nx);
    const size_t qj = q / d.nx;
    out[d.idx(i, (int)(qj % d.ny), (int)(qj / d.ny))] = in[q];
  }
}

int blocks_for(size_t n) {
  const size_t b = (n + 255) / 256;
  return (int)(b < 4096 ? (b > 0 ? b : 1) : 4096);
}

}  // namespace

void si_assemble(const Dims& d, const Metric& met, double* const* st, double* const* tend, double dt, double* a,
                 double* b, double* f, cudaStream_t s) {
  k_si_assemble<<<blocks_for((size_t)d.nx * d.ny * d.nz), 256, 0, s>>>(d, met, st[U], st[V], st[W], st[PI], tend[U],
                                                                        tend[V], tend[W], dt, a, b, f);
}
void si_cells_add_scaled(const Dims& d, double* x, const double* y, double a, cudaStream_t s) {
  k_cells_add_scaled<<<blocks_for((size_t)d.nx * d.ny * d.nz), 256, 0, s>>>(d, x, y, a);
}
void si_to_cells(const Dims& d, const double* in, double* out, cudaStream_t s) {
  k_to_cells<<<blocks_for((size_t)d.nx * d.ny * d.nz), 256, 0, s>>>(d, in, out);
}

}  // namespace vgb
