// vibe-model_gb300/csrc/tlad.cu
//
// Tangent-linear and adjoint of the reference's simplified collocated RK3
// (src/da/tangent_linear.cpp:72-603) on the GPU.
//
// TL operator F(xb, dx) (tendency_tl, :295-412), all differences 2nd-order
// central on interior points only (1 <= i <= nx-2 for d/dx, likewise j, k),
// D_x f = (f(i+1) - f(i-1)) * 0.5/max(dx, 1e-6), D_z with 0.5*inv_dz(i,j,k),
// inv_dz = 1/(dzeta(k)(z_top - zs)) (0 if not positive):
//   scalars s (theta, q*): -ub.D(ds) - du.D(sb)
//   rho: -rhob div(du) - ub.D(drho) - div(ub) drho - du.D(rhob)
//   pi:  -ub.D(dpi) - du.D(pib) - (Rd/cv)(pib div(du) + div(ub) dpi)
//   u:   -ub.D(du) - du.D(ub) - cp thb D_x(dpi) - cp dth D_x(pib) + f dv
//   v:   -ub.D(dv) - du.D(vb) - cp thb D_y(dpi) - cp dth D_y(pib) - f du
//   w:   -ub.D(dw) - du.D(wb) - cp thb D_z(dpi) - cp dth D_z(pib) + g dth/max(thb,1)
// with f = 2 Omega sin(45 deg). The adjoint (tendency_ad, :414-549) is its
// transpose; here it is formed as a gather: every output point collects the
// terms of the TL statements that read it (a term a(p) (x(p+1) - x(p-1))
// inv(p) gives x(q) the weights +a(q-1)inv(q-1) and -a(q+1)inv(q+1); a term
// c(p) G(p) with a perturbed coefficient c gives c(q) the weight G(q)), so
// each output point is written by one thread, without atomics.
//
// One RK3 step (rk3_tl, :559-572; rk3_ad, :574-603) is three fused
// launches: each writes dx_in + a F(xb, dx_stage) (TL) or the next adjoint
// stage (AD) directly. Fields use the model's device layout (one index for
// all staggers); points outside the nx x ny x nz cells pass through
// unchanged, as the reference's whole-storage updates leave them.
// Compute type T: double (FP64) or float (FP32 compute, FP64 storage).
#include <cmath>
#include <string>
#include <vector>

#include "vibe_internal.cuh"
#include "vibe_tlad.h"

namespace vgb {
namespace {

constexpr int kSp = NSPECIES;
__constant__ int kScal[7] = {THETA, QV, QC, QR, QI, QS, QG};

struct F12 {
  const double* f[kSp];
};
struct M12 {
  double* f[kSp];
};

struct TlGeo {
  Dims d;
  double ix, iy;          // 0.5/max(dx,1e-6), 0.5/max(dy,1e-6)
  const double* izh;      // nx*ny*nz: 0.5*inv_dz(i,j,k)
  double fcor, rdcv, cp, g;
};

template <typename T>
struct Pt {
  const TlGeo& g;
  size_t c;
  int i, j, k;
  bool vx, vy, vz;  // interior in x / y / z
  T ix, iy, iz;
  __device__ Pt(const TlGeo& g_, int i_, int j_, int k_) : g(g_), i(i_), j(j_), k(k_) {
    c = g.d.idx(i, j, k);
    vx = i >= 1 && i + 1 < g.d.nx;
    vy = j >= 1 && j + 1 < g.d.ny;
    vz = k >= 1 && k + 1 < g.d.nz;
    ix = (T)g.ix;
    iy = (T)g.iy;
    iz = (T)g.izh[((size_t)k * g.d.ny + j) * g.d.nx + i];
  }
  __device__ T v(const double* f, size_t o) const { return (T)f[o]; }
  __device__ T Dx(const double* f) const { return vx ? (v(f, c + 1) - v(f, c - 1)) * ix : (T)0; }
  __device__ T Dy(const double* f) const { return vy ? (v(f, c + g.d.P) - v(f, c - g.d.P)) * iy : (T)0; }
  __device__ T Dz(const double* f) const { return vz ? (v(f, c + g.d.plane) - v(f, c - g.d.plane)) * iz : (T)0; }
};

// out = in + a * F(xb, x) over the box; F zero outside the cells
template <typename T>
__global__ void k_tl(TlGeo g, const __grid_constant__ F12 xb, const __grid_constant__ F12 x,
                     const __grid_constant__ F12 in, const __grid_constant__ M12 out, double a) {
  const Dims& d = g.d;
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
  if (i > d.nx || j > d.ny) return;
  const size_t c = d.idx(i, j, k);
  if (i >= d.nx || j >= d.ny || k >= d.nz) {
    for (int q = 0; q < kSp; ++q) out.f[q][c] = in.f[q][c];
    return;
  }
  const Pt<T> p(g, i, j, k);
  const T ub = p.v(xb.f[U], c), vb = p.v(xb.f[V], c), wb = p.v(xb.f[W], c);
  const T du = p.v(x.f[U], c), dv = p.v(x.f[V], c), dw = p.v(x.f[W], c);
  const T divb = p.Dx(xb.f[U]) + p.Dy(xb.f[V]) + p.Dz(xb.f[W]);
  const T divd = p.Dx(x.f[U]) + p.Dy(x.f[V]) + p.Dz(x.f[W]);
  const T cp = (T)g.cp, rdcv = (T)g.rdcv, fc = (T)g.fcor;
  auto adv = [&](const double* df, const double* bf) {  // -ub.D(df) - du.D(bf)
    return -(ub * p.Dx(df) + vb * p.Dy(df) + wb * p.Dz(df)) - (du * p.Dx(bf) + dv * p.Dy(bf) + dw * p.Dz(bf));
  };
  T r[kSp];
  for (int s = 0; s < 7; ++s) r[kScal[s]] = adv(x.f[kScal[s]], xb.f[kScal[s]]);
  const T rhob = p.v(xb.f[RHO], c), drho = p.v(x.f[RHO], c);
  r[RHO] = -rhob * divd - (ub * p.Dx(x.f[RHO]) + vb * p.Dy(x.f[RHO]) + wb * p.Dz(x.f[RHO])) - divb * drho -
           (du * p.Dx(xb.f[RHO]) + dv * p.Dy(xb.f[RHO]) + dw * p.Dz(xb.f[RHO]));
  const T pib = p.v(xb.f[PI], c), dpi = p.v(x.f[PI], c);
  r[PI] = adv(x.f[PI], xb.f[PI]) - rdcv * (pib * divd + divb * dpi);
  const T thb = p.v(xb.f[THETA], c), dth = p.v(x.f[THETA], c);
  r[U] = adv(x.f[U], xb.f[U]) - cp * thb * p.Dx(x.f[PI]) - cp * dth * p.Dx(xb.f[PI]) + fc * dv;
  r[V] = adv(x.f[V], xb.f[V]) - cp * thb * p.Dy(x.f[PI]) - cp * dth * p.Dy(xb.f[PI]) - fc * du;
  r[W] = adv(x.f[W], xb.f[W]) - cp * thb * p.Dz(x.f[PI]) - cp * dth * p.Dz(xb.f[PI]) +
         (T)g.g * dth / (thb < (T)1 ? (T)1 : thb);
  for (int q = 0; q < kSp; ++q) out.f[q][c] = in.f[q][c] + a * (double)r[q];
}

// out = in + a * N(x): the nonlinear collocated tendency whose Jacobian at
// xb is F(xb, .) (nl_tendency of the reference's TL/AD test,
// tests/unit/test_tl_ad.cpp:100-180): -u.D(s) for the scalars,
// -rho div(u) - u.D(rho), -u.D(pi) - (Rd/cv) pi div(u), momentum
// -u.D(u) - cp theta D(pi) +- f (v, u), and buoyancy g (theta/max(thb,1) - 1)
// with thb the base state's theta.
template <typename T>
__global__ void k_nl(TlGeo g, const __grid_constant__ F12 xb, const __grid_constant__ F12 x,
                     const __grid_constant__ F12 in, const __grid_constant__ M12 out, double a) {
  const Dims& d = g.d;
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
  if (i > d.nx || j > d.ny) return;
  const size_t c = d.idx(i, j, k);
  if (i >= d.nx || j >= d.ny || k >= d.nz) {
    for (int q = 0; q < kSp; ++q) out.f[q][c] = in.f[q][c];
    return;
  }
  const Pt<T> p(g, i, j, k);
  const T u = p.v(x.f[U], c), v = p.v(x.f[V], c), w = p.v(x.f[W], c);
  const T div = p.Dx(x.f[U]) + p.Dy(x.f[V]) + p.Dz(x.f[W]);
  const T cp = (T)g.cp, rdcv = (T)g.rdcv, fc = (T)g.fcor;
  auto adv = [&](const double* f) { return -(u * p.Dx(f) + v * p.Dy(f) + w * p.Dz(f)); };
  T r[kSp];
  for (int s = 0; s < 7; ++s) r[kScal[s]] = adv(x.f[kScal[s]]);
  r[RHO] = -p.v(x.f[RHO], c) * div + adv(x.f[RHO]);
  r[PI] = adv(x.f[PI]) - rdcv * p.v(x.f[PI], c) * div;
  const T th = p.v(x.f[THETA], c), thb = p.v(xb.f[THETA], c);
  r[U] = adv(x.f[U]) - cp * th * p.Dx(x.f[PI]) + fc * v;
  r[V] = adv(x.f[V]) - cp * th * p.Dy(x.f[PI]) - fc * u;
  r[W] = adv(x.f[W]) - cp * th * p.Dz(x.f[PI]) + (T)g.g * (th / (thb < (T)1 ? (T)1 : thb) - (T)1);
  for (int q = 0; q < kSp; ++q) out.f[q][c] = in.f[q][c] + a * (double)r[q];
}

// Adjoint of F at one point: bar_x(q) = sum of the transposed TL terms.
// b = the adjoint input field (bar of the tendency), scaled by `a`.
template <typename T>
struct AdPt {
  const Pt<T>& p;
  const F12& xb;
  const F12& b;
  const TlGeo& g;
  // value of the bar field q at offset o from the point (caller checks range)
  __device__ T bv(int q, size_t o) const { return (T)b.f[q][o]; }
  // transpose of an f-term with coefficient field coef(p)*scale in direction dir:
  // + scale coef(c-e) inv(c-e) bar(c-e) [valid c-e] - scale coef(c+e) inv(c+e) bar(c+e) [valid c+e]
  template <class Coef>
  __device__ T tf(int dir, int qbar, Coef coef) const {
    const Dims& d = g.d;
    T acc = 0;
    if (dir == 0) {
      if (p.i - 1 >= 1 && p.i - 1 <= d.nx - 2) acc += coef(p.c - 1) * p.ix * bv(qbar, p.c - 1);
      if (p.i + 1 >= 1 && p.i + 1 <= d.nx - 2) acc -= coef(p.c + 1) * p.ix * bv(qbar, p.c + 1);
    } else if (dir == 1) {
      if (p.j - 1 >= 1 && p.j - 1 <= d.ny - 2) acc += coef(p.c - d.P) * p.iy * bv(qbar, p.c - d.P);
      if (p.j + 1 >= 1 && p.j + 1 <= d.ny - 2) acc -= coef(p.c + d.P) * p.iy * bv(qbar, p.c + d.P);
    } else {
      const size_t cc = ((size_t)p.k * d.ny + p.j) * d.nx + p.i, pl = (size_t)d.nx * d.ny;
      if (p.k - 1 >= 1 && p.k - 1 <= d.nz - 2)
        acc += coef(p.c - d.plane) * (T)g.izh[cc - pl] * bv(qbar, p.c - d.plane);
      if (p.k + 1 >= 1 && p.k + 1 <= d.nz - 2)
        acc -= coef(p.c + d.plane) * (T)g.izh[cc + pl] * bv(qbar, p.c + d.plane);
    }
    return acc;
  }
};

// out = base + add1 + add2 + a F^T(b) (absent addends are zero)
template <typename T>
__global__ void k_ad(TlGeo g, const __grid_constant__ F12 xb, const __grid_constant__ F12 b,
                     const __grid_constant__ F12 base, const __grid_constant__ F12 add1,
                     const __grid_constant__ F12 add2, const __grid_constant__ M12 out, double a) {
  const Dims& d = g.d;
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
  if (i > d.nx || j > d.ny) return;
  const size_t c = d.idx(i, j, k);
  double r[kSp];
  for (int q = 0; q < kSp; ++q) {
    r[q] = base.f[0] ? base.f[q][c] : 0.0;
    if (add1.f[0]) r[q] += add1.f[q][c];
    if (add2.f[0]) r[q] += add2.f[q][c];
  }
  if (i < d.nx && j < d.ny && k < d.nz) {
    const Pt<T> p(g, i, j, k);
    const AdPt<T> A{p, xb, b, g};
    const T cp = (T)g.cp, rdcv = (T)g.rdcv, fc = (T)g.fcor;
    auto X = [&](int q) { return [&, q](size_t o) { return (T)xb.f[q][o]; }; };
    T bs[kSp];
    for (int q = 0; q < kSp; ++q) bs[q] = (T)b.f[q][c];
    // f-terms with the base winds as coefficient, for every advected field
    // (scalars, rho, pi, u, v, w): bar_f += transpose of -ub D_x f - vb D_y f - wb D_z f
    auto adv_t = [&](int q) {
      return -(A.tf(0, q, X(U)) + A.tf(1, q, X(V)) + A.tf(2, q, X(W)));
    };
    T o[kSp];
    for (int q = 0; q < kSp; ++q) o[q] = 0;
    for (int s = 0; s < 7; ++s) o[kScal[s]] += adv_t(kScal[s]);
    const T divb = p.Dx(xb.f[U]) + p.Dy(xb.f[V]) + p.Dz(xb.f[W]);
    o[RHO] += adv_t(RHO) - divb * bs[RHO];
    o[PI] += adv_t(PI) - rdcv * divb * bs[PI];
    o[U] += adv_t(U);
    o[V] += adv_t(V);
    o[W] += adv_t(W);
    // c-terms du.D(base) of every equation: bar_u += -D_x(base_Y) bar_Y, etc.
    for (int s = 0; s < 7; ++s) {
      const int q = kScal[s];
      o[U] -= p.Dx(xb.f[q]) * bs[q];
      o[V] -= p.Dy(xb.f[q]) * bs[q];
      o[W] -= p.Dz(xb.f[q]) * bs[q];
    }
    const int bases[5] = {RHO, PI, U, V, W};
    for (int t = 0; t < 5; ++t) {
      const int q = bases[t];
      o[U] -= p.Dx(xb.f[q]) * bs[q];
      o[V] -= p.Dy(xb.f[q]) * bs[q];
      o[W] -= p.Dz(xb.f[q]) * bs[q];
    }
    // rho: -rhob div(du): f-terms of du, dv, dw with coefficient rhob
    o[U] -= A.tf(0, RHO, X(RHO));
    o[V] -= A.tf(1, RHO, X(RHO));
    o[W] -= A.tf(2, RHO, X(RHO));
    // pi: -(Rd/cv) pib div(du)
    o[U] -= rdcv * A.tf(0, PI, X(PI));
    o[V] -= rdcv * A.tf(1, PI, X(PI));
    o[W] -= rdcv * A.tf(2, PI, X(PI));
    // momentum pressure terms: -cp thb D(dpi) (f-term in dpi), -cp dth D(pib) (c-term in dth)
    o[PI] -= cp * (A.tf(0, U, X(THETA)) + A.tf(1, V, X(THETA)) + A.tf(2, W, X(THETA)));
    o[THETA] -= cp * (p.Dx(xb.f[PI]) * bs[U] + p.Dy(xb.f[PI]) * bs[V] + p.Dz(xb.f[PI]) * bs[W]);
    // Coriolis and buoyancy
    o[V] += fc * bs[U];
    o[U] -= fc * bs[V];
    const T thb = (T)xb.f[THETA][c];
    o[THETA] += (T)g.g * bs[W] / (thb < (T)1 ? (T)1 : thb);
    for (int q = 0; q < kSp; ++q) r[q] += a * (double)o[q];
  }
  for (int q = 0; q < kSp; ++q) out.f[q][c] = r[q];
}

thread_local std::string g_terr;

}  // namespace
}  // namespace vgb

using namespace vgb;

struct vibe_tlad {
  Dims d{};
  TlGeo g{};
  int precision = 0;
  cudaStream_t stream = nullptr;
  std::vector<void*> allocs;
  double* xb[kSp] = {};
  double* const* base = nullptr;  // linearisation point in use (xb, or a trajectory state)
  double* w[6][kSp] = {};  // work states
  double* izh = nullptr;
  std::vector<double> host;  // staging
};

namespace {
constexpr int kH = 4;

bool ok(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return true;
  g_terr = std::string(what) + ": " + cudaGetErrorString(e);
  return false;
}
double* dal(vibe_tlad* t, size_t n) {
  void* p = nullptr;
  if (cudaMalloc(&p, n * sizeof(double)) != cudaSuccess) return nullptr;
  cudaMemset(p, 0, n * sizeof(double));
  t->allocs.push_back(p);
  return (double*)p;
}
size_t field_count(const vibe_tlad* t) { return t->d.plane * (size_t)(t->d.nz + 1); }
void dims_of(const vibe_tlad* t, int q, int& nsx, int& nsy, int& nsz) {
  nsx = t->d.nx + 2 * kH + (q == U);
  nsy = t->d.ny + 2 * kH + (q == V);
  nsz = t->d.nz + 2 * kH + (q == W);
}
// FieldT storage -> device layout over the interior incl. the extra face
bool upload12(vibe_tlad* t, const double* const* h, double* const* dst) {
  for (int q = 0; q < kSp; ++q) {
    if (!h[q]) {
      g_terr = "NULL field";
      return false;
    }
    int nsx, nsy, nsz;
    dims_of(t, q, nsx, nsy, nsz);
    std::fill(t->host.begin(), t->host.end(), 0.0);
    const int ni = t->d.nx + (q == U), nj = t->d.ny + (q == V), nk = t->d.nz + (q == W);
    for (int k = 0; k < nk; ++k)
      for (int j = 0; j < nj; ++j)
        for (int i = 0; i < ni; ++i)
          t->host[t->d.idx(i, j, k)] = h[q][((size_t)(k + kH) * nsy + (j + kH)) * nsx + (i + kH)];
    if (!ok(cudaMemcpy(dst[q], t->host.data(), field_count(t) * sizeof(double), cudaMemcpyHostToDevice), "upload"))
      return false;
  }
  return true;
}
// device layout -> FieldT storage; points the device does not hold are
// taken from `keep` (the input's halo passes through, as in the reference)
bool download12(vibe_tlad* t, double* const* src, const double* const* keep, double* const* h) {
  for (int q = 0; q < kSp; ++q) {
    int nsx, nsy, nsz;
    dims_of(t, q, nsx, nsy, nsz);
    const size_t ns = (size_t)nsx * nsy * nsz;
    if (!ok(cudaMemcpy(t->host.data(), src[q], field_count(t) * sizeof(double), cudaMemcpyDeviceToHost), "download"))
      return false;
    if (keep && keep[q] != h[q]) std::copy(keep[q], keep[q] + ns, h[q]);
    if (!keep) std::fill(h[q], h[q] + ns, 0.0);
    const int ni = t->d.nx + (q == U), nj = t->d.ny + (q == V), nk = t->d.nz + (q == W);
    for (int k = 0; k < nk; ++k)
      for (int j = 0; j < nj; ++j)
        for (int i = 0; i < ni; ++i)
          h[q][((size_t)(k + kH) * nsy + (j + kH)) * nsx + (i + kH)] = t->host[t->d.idx(i, j, k)];
  }
  return true;
}

F12 cf(double* const* a) {
  F12 f;
  for (int q = 0; q < kSp; ++q) f.f[q] = a ? a[q] : nullptr;
  return f;
}
M12 mf(double* const* a) {
  M12 f;
  for (int q = 0; q < kSp; ++q) f.f[q] = a[q];
  return f;
}

void launch_tl(vibe_tlad* t, double* const* x, double* const* in, double* const* out, double a) {
  const dim3 b(32, 4), gr((t->d.nx + 1 + 31) / 32, (t->d.ny + 1 + 3) / 4, t->d.nz + 1);
  if (t->precision == 1)
    k_tl<float><<<gr, b, 0, t->stream>>>(t->g, cf(t->base), cf(x), cf(in), mf(out), a);
  else
    k_tl<double><<<gr, b, 0, t->stream>>>(t->g, cf(t->base), cf(x), cf(in), mf(out), a);
}
// out = base + add1 + add2 + a * F^T(b)
void launch_ad(vibe_tlad* t, double* const* b, double* const* base, double* const* add1, double* const* add2,
               double* const* out, double a) {
  const dim3 bl(32, 4), gr((t->d.nx + 1 + 31) / 32, (t->d.ny + 1 + 3) / 4, t->d.nz + 1);
  if (t->precision == 1)
    k_ad<float><<<gr, bl, 0, t->stream>>>(t->g, cf(t->base), cf(b), cf(base), cf(add1), cf(add2), mf(out), a);
  else
    k_ad<double><<<gr, bl, 0, t->stream>>>(t->g, cf(t->base), cf(b), cf(base), cf(add1), cf(add2), mf(out), a);
}

void launch_nl(vibe_tlad* t, double* const* x, double* const* in, double* const* out, double a) {
  const dim3 b(32, 4), gr((t->d.nx + 1 + 31) / 32, (t->d.ny + 1 + 3) / 4, t->d.nz + 1);
  if (t->precision == 1)
    k_nl<float><<<gr, b, 0, t->stream>>>(t->g, cf(t->xb), cf(x), cf(in), mf(out), a);
  else
    k_nl<double><<<gr, b, 0, t->stream>>>(t->g, cf(t->xb), cf(x), cf(in), mf(out), a);
}

// nl_rk3 (tests/unit/test_tl_ad.cpp:186-199) on device: in -> out; uses w[4]
void nl_step_dev(vibe_tlad* t, double* const* in, double* const* out, double dt) {
  double* const* s1 = t->w[4];
  launch_nl(t, in, in, s1, dt / 3.0);
  launch_nl(t, s1, in, out, dt / 2.0);
  launch_nl(t, out, in, s1, dt);
  for (int q = 0; q < kSp; ++q)
    cudaMemcpyAsync(out[q], s1[q], field_count(t) * sizeof(double), cudaMemcpyDeviceToDevice, t->stream);
}

// rk3_tl on device: in -> out (out distinct from in); uses w[4]
void tl_step_dev(vibe_tlad* t, double* const* in, double* const* out, double dt) {
  double* const* s1 = t->w[4];
  launch_tl(t, in, in, s1, dt / 3.0);
  launch_tl(t, s1, in, out, dt / 2.0);  // out holds dx2 temporarily
  launch_tl(t, out, in, s1, dt);
  for (int q = 0; q < kSp; ++q)
    cudaMemcpyAsync(out[q], s1[q], field_count(t) * sizeof(double), cudaMemcpyDeviceToDevice, t->stream);
}
// rk3_ad on device: bar_out -> bar_in (distinct); uses w[4], w[5]
void ad_step_dev(vibe_tlad* t, double* const* bo, double* const* bi, double dt) {
  double* const* b2 = t->w[4];
  double* const* b1 = t->w[5];
  launch_ad(t, bo, nullptr, nullptr, nullptr, b2, dt);        // bar_dx2 = F^T(dt bar_out)
  launch_ad(t, b2, nullptr, nullptr, nullptr, b1, dt / 2.0);  // bar_dx1 = F^T(dt/2 bar_dx2)
  launch_ad(t, b1, bo, b2, b1, bi, dt / 3.0);  // bar_out + bar_dx2 + bar_dx1 + F^T(dt/3 bar_dx1)
}

}  // namespace

extern "C" {

const char* vibe_tlad_last_error(void) { return g_terr.c_str(); }

int vibe_tlad_create(int nx, int ny, int nz, double dx, double dy, double z_top, const double* dzeta, const double* zs,
                     int precision, vibe_tlad** out) {
  if (!out || nx < 1 || ny < 1 || nz < 1 || !dzeta || (precision != 0 && precision != 1)) {
    g_terr = "vibe_tlad_create: bad argument";
    return VIBE_C_ERR_BAD_ARG;
  }
  auto* t = new vibe_tlad();
  t->precision = precision;
  t->d.nx = nx;
  t->d.ny = ny;
  t->d.nz = nz;
  t->d.P = (nx + 1 + 7) / 8 * 8;
  t->d.NY1 = ny + 1;
  t->d.plane = (size_t)t->d.NY1 * t->d.P;
  const size_t n = field_count(t);
  t->host.resize(n);
  bool good = ok(cudaStreamCreateWithFlags(&t->stream, cudaStreamNonBlocking), "stream");
  for (int q = 0; q < kSp && good; ++q) good = (t->xb[q] = dal(t, n)) != nullptr;
  for (int s = 0; s < 6 && good; ++s)
    for (int q = 0; q < kSp && good; ++q) good = (t->w[s][q] = dal(t, n)) != nullptr;
  // 0.5 * inv_dz(i,j,k) (Grid::inv_dz, geometry.cpp:265-270)
  std::vector<double> iz((size_t)nx * ny * nz);
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const double dz = dzeta[k] * (z_top - (zs ? zs[(size_t)j * nx + i] : 0.0));
        iz[((size_t)k * ny + j) * nx + i] = 0.5 * (dz > 0.0 ? 1.0 / dz : 0.0);
      }
  if (good) good = (t->izh = dal(t, iz.size())) != nullptr;
  if (good) good = ok(cudaMemcpy(t->izh, iz.data(), iz.size() * sizeof(double), cudaMemcpyHostToDevice), "upload");
  if (!good) {
    vibe_tlad_destroy(t);
    return VIBE_C_ERR_DEVICE;
  }
  t->g.d = t->d;
  t->g.ix = 0.5 / dmax(dx, 1e-6);
  t->g.iy = 0.5 / dmax(dy, 1e-6);
  t->g.izh = t->izh;
  t->g.fcor = 2.0 * kOmega * std::sin(45.0 * (kPi / 180.0));  // kCoriolis, tangent_linear.cpp:79
  t->g.rdcv = kRd / kCv;
  t->g.cp = kCp;
  t->g.g = kG;
  t->base = t->xb;
  *out = t;
  return VIBE_C_OK;
}

void vibe_tlad_destroy(vibe_tlad* t) {
  if (!t) return;
  if (t->stream) cudaStreamSynchronize(t->stream);
  for (void* p : t->allocs) cudaFree(p);
  if (t->stream) cudaStreamDestroy(t->stream);
  delete t;
}

int vibe_tlad_set_base(vibe_tlad* t, const double* const* xb) {
  if (!t || !xb) return VIBE_C_ERR_BAD_ARG;
  return upload12(t, xb, t->xb) ? VIBE_C_OK : VIBE_C_ERR_BAD_ARG;
}

int vibe_tl_tendency(vibe_tlad* t, const double* const* dx, double* const* d) {
  if (!t || !dx || !d) return VIBE_C_ERR_BAD_ARG;
  if (!upload12(t, dx, t->w[0])) return VIBE_C_ERR_DEVICE;
  for (int q = 0; q < kSp; ++q) cudaMemsetAsync(t->w[1][q], 0, field_count(t) * sizeof(double), t->stream);
  launch_tl(t, t->w[0], t->w[1], t->w[2], 1.0);  // 0 + 1*F
  if (!ok(cudaStreamSynchronize(t->stream), "tl tendency")) return VIBE_C_ERR_DEVICE;
  return download12(t, t->w[2], nullptr, d) ? VIBE_C_OK : VIBE_C_ERR_DEVICE;
}

int vibe_ad_tendency(vibe_tlad* t, const double* const* bar_d, double* const* bar_dx) {
  if (!t || !bar_d || !bar_dx) return VIBE_C_ERR_BAD_ARG;
  if (!upload12(t, bar_d, t->w[0]) || !upload12(t, bar_dx, t->w[1])) return VIBE_C_ERR_DEVICE;
  launch_ad(t, t->w[0], t->w[1], nullptr, nullptr, t->w[2], 1.0);  // bar_dx + F^T(bar_d)
  if (!ok(cudaStreamSynchronize(t->stream), "ad tendency")) return VIBE_C_ERR_DEVICE;
  return download12(t, t->w[2], bar_dx, bar_dx) ? VIBE_C_OK : VIBE_C_ERR_DEVICE;
}

int vibe_tl_propagate(vibe_tlad* t, double dt, int n_steps, const double* const* dx0, double* const* dx_out) {
  if (!t || !dx0 || !dx_out || n_steps < 0) return VIBE_C_ERR_BAD_ARG;
  if (!upload12(t, dx0, t->w[0])) return VIBE_C_ERR_DEVICE;
  int cur = 0;
  for (int s = 0; s < n_steps; ++s) {
    tl_step_dev(t, t->w[cur], t->w[1 - cur], dt);
    cur = 1 - cur;
  }
  if (!ok(cudaStreamSynchronize(t->stream), "tl propagate")) return VIBE_C_ERR_DEVICE;
  return download12(t, t->w[cur], dx0, dx_out) ? VIBE_C_OK : VIBE_C_ERR_DEVICE;
}

int vibe_tl_step(vibe_tlad* t, double dt, const double* const* dx, double* const* dx_out) {
  return vibe_tl_propagate(t, dt, 1, dx, dx_out);
}

int vibe_ad_propagate(vibe_tlad* t, double dt, int n_steps, const double* const* dy, double* const* dx0_adjoint) {
  if (!t || !dy || !dx0_adjoint || n_steps < 0) return VIBE_C_ERR_BAD_ARG;
  if (!upload12(t, dy, t->w[0])) return VIBE_C_ERR_DEVICE;
  int cur = 0;
  for (int s = 0; s < n_steps; ++s) {
    ad_step_dev(t, t->w[cur], t->w[1 - cur], dt);
    cur = 1 - cur;
  }
  if (!ok(cudaStreamSynchronize(t->stream), "ad propagate")) return VIBE_C_ERR_DEVICE;
  return download12(t, t->w[cur], dy, dx0_adjoint) ? VIBE_C_OK : VIBE_C_ERR_DEVICE;
}

int vibe_ad_step(vibe_tlad* t, double dt, const double* const* dx_next, double* const* dx_prev) {
  return vibe_ad_propagate(t, dt, 1, dx_next, dx_prev);
}

int vibe_nl_tendency(vibe_tlad* t, const double* const* x, double* const* d) {
  if (!t || !x || !d) return VIBE_C_ERR_BAD_ARG;
  if (!upload12(t, x, t->w[0])) return VIBE_C_ERR_DEVICE;
  for (int q = 0; q < kSp; ++q) cudaMemsetAsync(t->w[1][q], 0, field_count(t) * sizeof(double), t->stream);
  launch_nl(t, t->w[0], t->w[1], t->w[2], 1.0);  // 0 + 1*N
  if (!ok(cudaStreamSynchronize(t->stream), "nl tendency")) return VIBE_C_ERR_DEVICE;
  return download12(t, t->w[2], nullptr, d) ? VIBE_C_OK : VIBE_C_ERR_DEVICE;
}

int vibe_nl_propagate(vibe_tlad* t, double dt, int n_steps, const double* const* x0, double* const* x_out) {
  if (!t || !x0 || !x_out || n_steps < 0) return VIBE_C_ERR_BAD_ARG;
  if (!upload12(t, x0, t->w[0])) return VIBE_C_ERR_DEVICE;
  int cur = 0;
  for (int s = 0; s < n_steps; ++s) {
    nl_step_dev(t, t->w[cur], t->w[1 - cur], dt);
    cur = 1 - cur;
  }
  if (!ok(cudaStreamSynchronize(t->stream), "nl propagate")) return VIBE_C_ERR_DEVICE;
  return download12(t, t->w[cur], x0, x_out) ? VIBE_C_OK : VIBE_C_ERR_DEVICE;
}

}  // extern "C"

// ---- device-side access for trajectory runs (tlad_internal.cuh) ----
namespace vgb {
void tlad_grid(const vibe_tlad* t, int* nx, int* ny, int* nz) {
  *nx = t->d.nx;
  *ny = t->d.ny;
  *nz = t->d.nz;
}
cudaStream_t tlad_stream(vibe_tlad* t) { return t->stream; }
double* const* tlad_work(vibe_tlad* t, int s) { return t->w[s]; }
void tlad_use_base(vibe_tlad* t, double* const* base) { t->base = base ? base : t->xb; }
void tlad_tl_step(vibe_tlad* t, double* const* in, double* const* out, double dt) { tl_step_dev(t, in, out, dt); }
void tlad_ad_step(vibe_tlad* t, double* const* bo, double* const* bi, double dt) { ad_step_dev(t, bo, bi, dt); }
bool tlad_upload(vibe_tlad* t, const double* const* host, double* const* dst) { return upload12(t, host, dst); }
bool tlad_download(vibe_tlad* t, double* const* src, const double* const* keep, double* const* host) {
  return download12(t, src, keep, host);
}
void tlad_set_error(const char* msg) { g_terr = msg; }
}  // namespace vgb
