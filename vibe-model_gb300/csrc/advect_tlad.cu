// vibe-model_gb300/csrc/advect_tlad.cu
//
// Tangent-linear and adjoint of the C-ABI flux advection
// (vibe_advect_scalar_flux_f64, the reference's c_kernels.c:209-286):
//   dqdt = -div(F) / max(rho, 1e-12),
//   F on a face = vel * (rho_a + rho_b)/2 * (q_a + q_b)/2 between its cells
//   a and b, periodic in x and y, vertical faces only for cells with
//   0 < k < nz-1 (the others have zero vertical flux), dz = max(dzeta(k) *
//   (z_top - zs), 1).
// The TL differentiates every face flux (dF = dvel R Q + vel dR Q + vel R dQ)
// and the density divisor (where rho > 1e-12). The adjoint is a gather: each
// point collects, from the six faces it touches, bar_F = (h(b) - h(a))/dx
// with h = bar_dqdt / max(rho, 1e-12) (vertically each cell only where its
// vertical fluxes exist), so every output is written by one thread and no
// atomics are needed. The adjoint accumulates into its outputs.
#include <cmath>
#include <string>

#include "cabi_host.cuh"
#include "vibe_c_kernels.h"
#include "vibe_internal.cuh"

namespace {

struct Grid3 {
  int nx, ny, nz;
  size_t nxy;
  __device__ size_t at(int i, int j, int k) const { return (size_t)k * nxy + (size_t)j * nx + (size_t)i; }
  __device__ int wrapx(int i) const { return (i + nx) % nx; }
  __device__ int wrapy(int j) const { return (j + ny) % ny; }
};

template <typename T>
__device__ __forceinline__ T dz_of(const T* dzeta, const T* zs, T z_top, const Grid3& g, int i, int j, int k) {
  const T scale = zs ? (z_top - zs[(size_t)j * g.nx + i]) : z_top;
  T dz = dzeta[k] * scale;
  return dz < (T)1 ? (T)1 : dz;
}

template <typename T>
__global__ void k_flux_tl(const T* __restrict__ q, const T* __restrict__ rho, const T* __restrict__ u,
                          const T* __restrict__ v, const T* __restrict__ w, const T* __restrict__ dq,
                          const T* __restrict__ drho, const T* __restrict__ du, const T* __restrict__ dv,
                          const T* __restrict__ dw, const T* __restrict__ dzeta, const T* __restrict__ zs, Grid3 g,
                          T dx, T dy, T z_top, T* __restrict__ out) {
  const size_t n = g.nxy * g.nz;
  const T hf = (T)0.5;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(c / g.nxy), j = (int)((c / g.nx) % g.ny), i = (int)(c % g.nx);
    // flux through a face with velocity index fv between cells a, b, and its TL
    auto flux = [&](size_t fv, size_t a, size_t b, const T* vel, const T* dvel, T& F, T& dF) {
      const T R = hf * (rho[a] + rho[b]), Q = hf * (q[a] + q[b]);
      const T dR = hf * (drho[a] + drho[b]), dQ = hf * (dq[a] + dq[b]);
      F = vel[fv] * R * Q;
      dF = dvel[fv] * R * Q + vel[fv] * dR * Q + vel[fv] * R * dQ;
    };
    const size_t e = g.at(g.wrapx(i + 1), j, k), wv = g.at(g.wrapx(i - 1), j, k);
    const size_t nn = g.at(i, g.wrapy(j + 1), k), ss = g.at(i, g.wrapy(j - 1), k);
    T fE, dfE, fW, dfW, fN, dfN, fS, dfS, fT = 0, dfT = 0, fB = 0, dfB = 0;
    flux(e, c, e, u, du, fE, dfE);
    flux(c, wv, c, u, du, fW, dfW);
    flux(nn, c, nn, v, dv, fN, dfN);
    flux(c, ss, c, v, dv, fS, dfS);
    if (k > 0 && k + 1 < g.nz) {
      flux(c + g.nxy, c, c + g.nxy, w, dw, fT, dfT);
      flux(c, c - g.nxy, c, w, dw, fB, dfB);
    }
    const T dz = dz_of(dzeta, zs, z_top, g, i, j, k);
    const T div = (fE - fW) / dx + (fN - fS) / dy + (fT - fB) / dz;
    const T ddiv = (dfE - dfW) / dx + (dfN - dfS) / dy + (dfT - dfB) / dz;
    const bool pos = rho[c] > (T)1e-12;
    const T rr = pos ? rho[c] : (T)1e-12;
    T r = -ddiv / rr;
    if (pos) r += div * drho[c] / (rr * rr);
    out[c] = r;
  }
}

template <typename T>
__global__ void k_flux_ad(const T* __restrict__ q, const T* __restrict__ rho, const T* __restrict__ u,
                          const T* __restrict__ v, const T* __restrict__ w, const T* __restrict__ bd,
                          const T* __restrict__ dzeta, const T* __restrict__ zs, Grid3 g, T dx, T dy, T z_top,
                          T* __restrict__ bq, T* __restrict__ brho, T* __restrict__ bu, T* __restrict__ bv,
                          T* __restrict__ bw) {
  const size_t n = g.nxy * g.nz;
  const T hf = (T)0.5;
  auto h = [&](size_t c) { return bd[c] / (rho[c] > (T)1e-12 ? rho[c] : (T)1e-12); };
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < n; p += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(p / g.nxy), j = (int)((p / g.nx) % g.ny), i = (int)(p % g.nx);
    T sq = 0, srho = 0;
    // one face between cells a and b with velocity vel[fv] and adjoint bar_F:
    // contributions to q[p], rho[p] (p is a or b); returns R*Q for the velocity
    auto face = [&](size_t fv, size_t a, size_t b, const T* vel, T barF) {
      const T R = hf * (rho[a] + rho[b]), Q = hf * (q[a] + q[b]);
      const T s = barF * vel[fv];
      sq += s * R * hf;
      srho += s * hf * Q;
      return R * Q;
    };
    const size_t west = g.at(g.wrapx(i - 1), j, k), east = g.at(g.wrapx(i + 1), j, k);
    const size_t south = g.at(i, g.wrapy(j - 1), k), north = g.at(i, g.wrapy(j + 1), k);
    // x faces: west (at u[p]) between west and p; east (at u[east]) between p and east
    const T rqW = face(p, west, p, u, (h(p) - h(west)) / dx);
    face(east, p, east, u, (h(east) - h(p)) / dx);
    const T rqS = face(p, south, p, v, (h(p) - h(south)) / dy);
    face(north, p, north, v, (h(north) - h(p)) / dy);
    T rqB = 0, barB = 0;
    auto interior = [&](int kk) { return kk > 0 && kk + 1 < g.nz; };
    if (k >= 1) {  // face between k-1 and k, at w[p]
      const size_t below = p - g.nxy;
      if (interior(k - 1)) barB -= h(below) / dz_of(dzeta, zs, z_top, g, i, j, k - 1);
      if (interior(k)) barB += h(p) / dz_of(dzeta, zs, z_top, g, i, j, k);
      rqB = face(p, below, p, w, barB);
    }
    if (k + 1 <= g.nz - 1) {  // face between k and k+1, at w[p + nxy]
      const size_t above = p + g.nxy;
      T barT = 0;
      if (interior(k)) barT -= h(p) / dz_of(dzeta, zs, z_top, g, i, j, k);
      if (interior(k + 1)) barT += h(above) / dz_of(dzeta, zs, z_top, g, i, j, k + 1);
      face(above, p, above, w, barT);
    }
    // density divisor of the own cell
    if (rho[p] > (T)1e-12) {
      T fE, fW, fN, fS, fT = 0, fB = 0;
      auto F = [&](size_t fv, size_t a, size_t b, const T* vel) {
        return vel[fv] * (hf * (rho[a] + rho[b])) * (hf * (q[a] + q[b]));
      };
      fE = F(east, p, east, u);
      fW = F(p, west, p, u);
      fN = F(north, p, north, v);
      fS = F(p, south, p, v);
      if (interior(k)) {
        fT = F(p + g.nxy, p, p + g.nxy, w);
        fB = F(p, p - g.nxy, p, w);
      }
      const T div = (fE - fW) / dx + (fN - fS) / dy + (fT - fB) / dz_of(dzeta, zs, z_top, g, i, j, k);
      srho += bd[p] * div / (rho[p] * rho[p]);
    }
    bq[p] += sq;
    brho[p] += srho;
    bu[p] += ((h(p) - h(west)) / dx) * rqW;
    bv[p] += ((h(p) - h(south)) / dy) * rqS;
    bw[p] += barB * rqB;
  }
}

// device failures go to the thread's C-ABI error message (vibe_c_last_error)
bool ok(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return true;
  vgb_cabi::set_error(what, e);
  return false;
}

int blocks_for(size_t n) { return (int)((n + 255) / 256 < 65535 ? (n + 255) / 256 : 65535); }

template <typename T>
int tl_dev(const T* q, const T* rho, const T* u, const T* v, const T* w, const T* dq, const T* drho, const T* du,
           const T* dv, const T* dw, const T* dzeta, const T* zs, int nx, int ny, int nz, T dx, T dy, T z_top, T* out,
           cudaStream_t s) {
  if (!q || !rho || !u || !v || !w || !dq || !drho || !du || !dv || !dw || !dzeta || !out || nx < 1 || ny < 1 ||
      nz < 1)
    return VIBE_C_ERR_BAD_ARG;
  const Grid3 g{nx, ny, nz, (size_t)nx * ny};
  k_flux_tl<T><<<blocks_for(g.nxy * nz), 256, 0, s>>>(q, rho, u, v, w, dq, drho, du, dv, dw, dzeta, zs, g, dx, dy,
                                                      z_top, out);
  return ok(cudaGetLastError(), "flux TL launch") ? VIBE_C_OK : VIBE_C_ERR_DEVICE;
}

template <typename T>
int ad_dev(const T* q, const T* rho, const T* u, const T* v, const T* w, const T* bd, const T* dzeta, const T* zs,
           int nx, int ny, int nz, T dx, T dy, T z_top, T* bq, T* brho, T* bu, T* bv, T* bw, cudaStream_t s) {
  if (!q || !rho || !u || !v || !w || !bd || !dzeta || !bq || !brho || !bu || !bv || !bw || nx < 1 || ny < 1 || nz < 1)
    return VIBE_C_ERR_BAD_ARG;
  const Grid3 g{nx, ny, nz, (size_t)nx * ny};
  k_flux_ad<T><<<blocks_for(g.nxy * nz), 256, 0, s>>>(q, rho, u, v, w, bd, dzeta, zs, g, dx, dy, z_top, bq, brho, bu,
                                                      bv, bw);
  return ok(cudaGetLastError(), "flux AD launch") ? VIBE_C_OK : VIBE_C_ERR_DEVICE;
}

// host forms: every array staged through the calling thread's buffers in
// one copy each way (cabi_host.cuh), no allocation once they fit
template <typename T>
int tl_host(const T* q, const T* rho, const T* u, const T* v, const T* w, const T* dq, const T* drho, const T* du,
            const T* dv, const T* dw, const T* dzeta, const T* zs, int nx, int ny, int nz, T dx, T dy, T z_top,
            T* out) {
  if (!q || !rho || !u || !v || !w || !dq || !drho || !du || !dv || !dw || !dzeta || !out || nx < 1 || ny < 1 ||
      nz < 1)
    return VIBE_C_ERR_BAD_ARG;
  using vgb_cabi::HostCall;
  const size_t n = (size_t)nx * ny * nz, e = sizeof(T);
  HostCall hc;
  const T* ins[10] = {q, rho, u, v, w, dq, drho, du, dv, dw};
  int id[10];
  for (int t = 0; t < 10; ++t) id[t] = hc.add(ins[t], n * e, HostCall::kIn);
  const int iz = hc.add(dzeta, (size_t)nz * e, HostCall::kIn);
  const int izs = hc.add(zs, zs ? (size_t)nx * ny * e : 0, HostCall::kIn);
  const int io = hc.add(out, n * e, HostCall::kOut);
  int rc = hc.commit() ? VIBE_C_OK : VIBE_C_ERR_DEVICE;
  if (rc == VIBE_C_OK)
    rc = tl_dev<T>(hc.dev<T>(id[0]), hc.dev<T>(id[1]), hc.dev<T>(id[2]), hc.dev<T>(id[3]), hc.dev<T>(id[4]),
                   hc.dev<T>(id[5]), hc.dev<T>(id[6]), hc.dev<T>(id[7]), hc.dev<T>(id[8]), hc.dev<T>(id[9]),
                   hc.dev<T>(iz), hc.dev<T>(izs), nx, ny, nz, dx, dy, z_top, hc.dev<T>(io), hc.stream());
  if (!hc.finish() && rc == VIBE_C_OK) rc = VIBE_C_ERR_DEVICE;
  return rc;
}

template <typename T>
int ad_host(const T* q, const T* rho, const T* u, const T* v, const T* w, const T* bd, const T* dzeta, const T* zs,
            int nx, int ny, int nz, T dx, T dy, T z_top, T* bq, T* brho, T* bu, T* bv, T* bw) {
  if (!q || !rho || !u || !v || !w || !bd || !dzeta || !bq || !brho || !bu || !bv || !bw || nx < 1 || ny < 1 || nz < 1)
    return VIBE_C_ERR_BAD_ARG;
  using vgb_cabi::HostCall;
  const size_t n = (size_t)nx * ny * nz, e = sizeof(T);
  HostCall hc;
  const T* ins[6] = {q, rho, u, v, w, bd};
  int id[6];
  for (int t = 0; t < 6; ++t) id[t] = hc.add(ins[t], n * e, HostCall::kIn);
  const int iz = hc.add(dzeta, (size_t)nz * e, HostCall::kIn);
  const int izs = hc.add(zs, zs ? (size_t)nx * ny * e : 0, HostCall::kIn);
  // the outputs accumulate: their current values travel to the device and back
  T* outs[5] = {bq, brho, bu, bv, bw};
  int io[5];
  for (int t = 0; t < 5; ++t) io[t] = hc.add(outs[t], n * e, HostCall::kInOut);
  int rc = hc.commit() ? VIBE_C_OK : VIBE_C_ERR_DEVICE;
  if (rc == VIBE_C_OK)
    rc = ad_dev<T>(hc.dev<T>(id[0]), hc.dev<T>(id[1]), hc.dev<T>(id[2]), hc.dev<T>(id[3]), hc.dev<T>(id[4]),
                   hc.dev<T>(id[5]), hc.dev<T>(iz), hc.dev<T>(izs), nx, ny, nz, dx, dy, z_top, hc.dev<T>(io[0]),
                   hc.dev<T>(io[1]), hc.dev<T>(io[2]), hc.dev<T>(io[3]), hc.dev<T>(io[4]), hc.stream());
  if (!hc.finish() && rc == VIBE_C_OK) rc = VIBE_C_ERR_DEVICE;
  return rc;
}

}  // namespace

extern "C" {

int vibe_advect_scalar_flux_tl_f64(const double* q, const double* rho, const double* u, const double* v,
                                   const double* w, const double* dq, const double* drho, const double* du,
                                   const double* dv, const double* dw, const double* dzeta, const double* zs, int nx,
                                   int ny, int nz, double dx, double dy, double z_top, double* d_dqdt) {
  return tl_host<double>(q, rho, u, v, w, dq, drho, du, dv, dw, dzeta, zs, nx, ny, nz, dx, dy, z_top, d_dqdt);
}

int vibe_advect_scalar_flux_ad_f64(const double* q, const double* rho, const double* u, const double* v,
                                   const double* w, const double* bar_dqdt, const double* dzeta, const double* zs,
                                   int nx, int ny, int nz, double dx, double dy, double z_top, double* bar_q,
                                   double* bar_rho, double* bar_u, double* bar_v, double* bar_w) {
  return ad_host<double>(q, rho, u, v, w, bar_dqdt, dzeta, zs, nx, ny, nz, dx, dy, z_top, bar_q, bar_rho, bar_u, bar_v,
                         bar_w);
}

int vibe_advect_scalar_flux_tl_f64_dev(const double* q, const double* rho, const double* u, const double* v,
                                       const double* w, const double* dq, const double* drho, const double* du,
                                       const double* dv, const double* dw, const double* dzeta, const double* zs,
                                       int nx, int ny, int nz, double dx, double dy, double z_top, double* d_dqdt,
                                       vibe_stream_t stream) {
  return tl_dev<double>(q, rho, u, v, w, dq, drho, du, dv, dw, dzeta, zs, nx, ny, nz, dx, dy, z_top, d_dqdt,
                        (cudaStream_t)stream);
}

int vibe_advect_scalar_flux_ad_f64_dev(const double* q, const double* rho, const double* u, const double* v,
                                       const double* w, const double* bar_dqdt, const double* dzeta, const double* zs,
                                       int nx, int ny, int nz, double dx, double dy, double z_top, double* bar_q,
                                       double* bar_rho, double* bar_u, double* bar_v, double* bar_w,
                                       vibe_stream_t stream) {
  return ad_dev<double>(q, rho, u, v, w, bar_dqdt, dzeta, zs, nx, ny, nz, dx, dy, z_top, bar_q, bar_rho, bar_u, bar_v,
                        bar_w, (cudaStream_t)stream);
}

int vibe_advect_scalar_flux_tl_f32(const float* q, const float* rho, const float* u, const float* v, const float* w,
                                   const float* dq, const float* drho, const float* du, const float* dv,
                                   const float* dw, const float* dzeta, const float* zs, int nx, int ny, int nz,
                                   float dx, float dy, float z_top, float* d_dqdt) {
  return tl_host<float>(q, rho, u, v, w, dq, drho, du, dv, dw, dzeta, zs, nx, ny, nz, dx, dy, z_top, d_dqdt);
}

int vibe_advect_scalar_flux_ad_f32(const float* q, const float* rho, const float* u, const float* v, const float* w,
                                   const float* bar_dqdt, const float* dzeta, const float* zs, int nx, int ny, int nz,
                                   float dx, float dy, float z_top, float* bar_q, float* bar_rho, float* bar_u,
                                   float* bar_v, float* bar_w) {
  return ad_host<float>(q, rho, u, v, w, bar_dqdt, dzeta, zs, nx, ny, nz, dx, dy, z_top, bar_q, bar_rho, bar_u, bar_v,
                        bar_w);
}

}  // extern "C"
