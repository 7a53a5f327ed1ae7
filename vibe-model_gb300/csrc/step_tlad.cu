// vibe-model_gb300/csrc/step_tlad.cu
//
// Tangent-linear and adjoint of the model's own slow tendency R(s): the
// function the FP64 path evaluates in k_tend_u / k_tend_v / k_tend_w,
// k_tend_cells and k_weno_faces / k_weno_cells (Equations::tendencies,
// equations.cpp:60-150, with Advection::momentum, advection.cpp:250-319, the
// WENO5 flux form of Advection::scalar, :144-187, or
// Advection::scalar_nonconservative, :224-244, Coriolis, the buoyancy and the
// split / perturbation-pressure-gradient switches), linearised about a base
// state held on the device. Same stencils, clamps and ghost reads as those
// kernels.
//
// Every output point is written once, as a template over its arithmetic:
//   * Jet<R> carries a value and one directional derivative. With the
//     perturbation as the loads' derivatives the point function returns R
//     and dR (the tangent-linear). The WENO5 weights and the Lax-Friedrichs
//     switch at |u| = 1e-3 are differentiated exactly; where the positivity
//     clip of the moisture species is active the derivative is zero.
//   * The adjoint evaluates the same point function once per load, with a
//     unit derivative on that load alone (forward mode, one column of the
//     point's Jacobian row per pass), and adds (dR/dload) * bar_R to the bar
//     of the loaded point with atomicAdd. Loads that alias through index
//     clamps add up, so the scatter is the exact transpose of the tangent.
//   * A WENO5 face flux is shared by the two cells beside the face, so its
//     adjoint runs per face: bar_F is gathered from the two cells' bars (zero
//     where the clip is active) and then scattered to the face's six loads.
//     Face fluxes are carried as F(q - c) with c = q at the stencil centre,
//     and the cells add the c u parts back as (q - c) u, so that the large
//     products q u of the flux and advective forms never cancel (this keeps
//     FP32 tangents and adjoints consistent to ~1e-7).
// The pressure-gradient and mass-flux terms that split_fast moves to the
// acoustic substeps are folded into the slow ones they cancel (theta -
// theta0, rho - rho0 beside each wind), so no two loads carry large
// derivatives that cancel.
// R = double for FP64 models; R = float for mixed models (FP32 arithmetic;
// base state, perturbations and bars stay FP64 in storage).
#include <algorithm>

#include "step_kernels.cuh"

namespace vgb {
namespace {

template <class R>
struct Jet {
  R v, d;
};
template <class R>
__device__ __forceinline__ Jet<R> operator+(Jet<R> a, Jet<R> b) {
  return {a.v + b.v, a.d + b.d};
}
template <class R>
__device__ __forceinline__ Jet<R> operator-(Jet<R> a, Jet<R> b) {
  return {a.v - b.v, a.d - b.d};
}
template <class R>
__device__ __forceinline__ Jet<R> operator-(Jet<R> a) {
  return {-a.v, -a.d};
}
template <class R>
__device__ __forceinline__ Jet<R> operator*(Jet<R> a, Jet<R> b) {
  return {a.v * b.v, a.d * b.v + a.v * b.d};
}
template <class R>
__device__ __forceinline__ Jet<R> operator*(Jet<R> a, double c) {
  return {a.v * (R)c, a.d * (R)c};
}
template <class R>
__device__ __forceinline__ Jet<R> operator*(double c, Jet<R> a) {
  return {(R)c * a.v, (R)c * a.d};
}
template <class R>
__device__ __forceinline__ Jet<R> operator+(Jet<R> a, double c) {
  return {a.v + (R)c, a.d};
}
template <class R>
__device__ __forceinline__ Jet<R> operator-(Jet<R> a, double c) {
  return {a.v - (R)c, a.d};
}
template <class R>
__device__ __forceinline__ Jet<R> operator/(Jet<R> a, Jet<R> b) {
  const R q = a.v / b.v;
  return {q, (a.d - q * b.d) / b.v};
}

struct F12 {  // base fields (device layout)
  const double* f[NSPECIES];
};
struct B12 {  // writable fields: tangents out, or bars accumulated
  double* f[NSPECIES];
};

// Loads. Tangent-linear: the derivative is the perturbation at the point.
// Every loader also offers operator()(q, c, ref): the value minus a
// reference, the difference taken in FP64 before the conversion, so FP32
// arithmetic sees theta - theta0 (~1 K), not theta (~300 K).
template <class R>
struct TlLoad {
  const F12* s;
  const F12* p;
  __device__ __forceinline__ Jet<R> operator()(int q, size_t c, double ref = 0.0) {
    return {(R)(s->f[q][c] - ref), (R)p->f[q][c]};
  }
};
// Adjoint pass: a unit derivative on load number `seed` only; remembers
// which point that load read.
template <class R>
struct AdLoad {
  const F12* s;
  int seed, n, hq;
  size_t hc;
  __device__ __forceinline__ Jet<R> operator()(int q, size_t c, double ref = 0.0) {
    Jet<R> r{(R)(s->f[q][c] - ref), (R)0};
    if (n == seed) {
      r.d = (R)1;
      hq = q;
      hc = c;
    }
    ++n;
    return r;
  }
};
// Values only.
template <class R>
struct ValLoad {
  const F12* s;
  __device__ __forceinline__ Jet<R> operator()(int q, size_t c, double ref = 0.0) {
    return {(R)(s->f[q][c] - ref), (R)0};
  }
};

constexpr int kMaxLoads = 48;  // more than any point function below reads

#define LD(q, i, j, k) L((q), d.idx((i), (j), (k)))
#define LDS(q, i, j, k, ref) L((q), d.idx((i), (j), (k)), (ref))
#define LDC(q, i, j, k) L((q), d.idx(iclamp((i), 0, d.nx - 1), iclamp((j), 0, d.ny - 1), iclamp((k), 0, d.nz - 1)))

__device__ __forceinline__ double dzeta_(const Metric& m, const Dims& d, int k) {
  return m.dzeta[iclamp(k, 0, d.nz - 1)];
}
__device__ __forceinline__ double scale_(const Metric& m, const Dims& d, int i, int j) {
  return m.scale[(size_t)iclamp(j, 0, d.ny - 1) * d.nx + iclamp(i, 0, d.nx - 1)];
}
__device__ __forceinline__ double ref_(const double* f, const Dims& d, int i, int j, int k) {
  return f[d.idx(i, j, k)];
}
// coriolis.cpp:25-59 (f-plane or beta-plane about the domain centre)
__device__ __forceinline__ double corf_(const Metric& m, const Flags& fl, const Dims& d, int j) {
  if (fl.coriolis != 2) return m.f0;
  return m.f0 + m.beta * (((double)j + 0.5) * m.dy - 0.5 * (double)d.ny * m.dy);
}

// Exner difference of the pressure-gradient terms (pi or pi - pi0)
template <class R, class Ld>
__device__ __forceinline__ Jet<R> dpi_(const Dims& d, const Metric& m, const Flags& fl, Ld& L, int ia, int ja, int ka,
                                       int ib, int jb, int kb) {
  if (!fl.pgf_pert) return LD(PI, ia, ja, ka) - LD(PI, ib, jb, kb);
  return LDS(PI, ia, ja, ka, ref_(m.pi0, d, ia, ja, ka)) - LDS(PI, ib, jb, kb, ref_(m.pi0, d, ib, jb, kb));
}

// u face (i, j, k), i = 0..nx: k_tend_u
template <class R, class Ld>
__device__ __forceinline__ Jet<R> pt_u(const Dims& d, const Metric& m, const Flags& fl, Ld& L, int i, int j, int k) {
  using T = Jet<R>;
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const int ip = imin(i, nx - 1), im = imax(i - 1, 0);
  const double dz = dzeta_(m, d, imin(k, nz - 1)) * scale_(m, d, ip, j);
  const T um = LD(U, im, j, k), up = LD(U, ip, j, k);
  const T uc = 0.5 * (um + up);
  const T ux = (up - um) * m.inv_dx;
  const T uy = (LD(U, ip, imin(j + 1, ny - 1), k) - LD(U, ip, imax(j - 1, 0), k)) * (0.5 * m.inv_dy);
  const T uz = (LD(U, ip, j, imin(k + 1, nz - 1)) - LD(U, ip, j, imax(k - 1, 0))) * (1.0 / (2.0 * dz));
  const T vc = 0.25 * (LD(V, im, imax(j - 1, 0), k) + LD(V, ip, imax(j - 1, 0), k) + LD(V, im, j, k) + LD(V, ip, j, k));
  const T wc = 0.5 * (LD(W, ip, j, k) + LD(W, ip, j, imin(k + 1, nz - 1)));
  T acc = -(uc * ux + vc * uy + wc * uz);
  if (fl.coriolis) acc = acc + corf_(m, fl, d, j) * vc;  // v at the u face: the same four points
  const bool sp = fl.split_fast;  // the slow part takes theta - theta0
  const T th = 0.5 * (LDS(THETA, im, j, k, sp ? ref_(m.th0, d, im, j, k) : 0.0) +
                      LDS(THETA, ip, j, k, sp ? ref_(m.th0, d, ip, j, k) : 0.0));
  return acc - kCp * (th * dpi_<R>(d, m, fl, L, ip, j, k, im, j, k)) * m.inv_dx;
}

// v face (i, j, k), j = 0..ny: k_tend_v
template <class R, class Ld>
__device__ __forceinline__ Jet<R> pt_v(const Dims& d, const Metric& m, const Flags& fl, Ld& L, int i, int j, int k) {
  using T = Jet<R>;
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const int jp = imin(j, ny - 1), jm = imax(j - 1, 0);
  const double dz = dzeta_(m, d, imin(k, nz - 1)) * scale_(m, d, i, jp);
  const T vm = LD(V, i, jm, k), vp = LD(V, i, jp, k);
  const T vc = 0.5 * (vm + vp);
  const T vy = (vp - vm) * m.inv_dy;
  const T vx = (LD(V, imin(i + 1, nx - 1), jp, k) - LD(V, imax(i - 1, 0), jp, k)) * (0.5 * m.inv_dx);
  const T vz = (LD(V, i, jp, imin(k + 1, nz - 1)) - LD(V, i, jp, imax(k - 1, 0))) * (1.0 / (2.0 * dz));
  const int ia = imax(i - 1, 0);
  const T uc = 0.25 * (LD(U, ia, jm, k) + LD(U, i, jm, k) + LD(U, ia, jp, k) + LD(U, i, jp, k));
  const T wc = 0.5 * (LD(W, i, jp, k) + LD(W, i, jp, imin(k + 1, nz - 1)));
  T acc = -(uc * vx + vc * vy + wc * vz);
  if (fl.coriolis) acc = acc - corf_(m, fl, d, j) * uc;
  const bool sp = fl.split_fast;
  const T th = 0.5 * (LDS(THETA, i, jm, k, sp ? ref_(m.th0, d, i, jm, k) : 0.0) +
                      LDS(THETA, i, jp, k, sp ? ref_(m.th0, d, i, jp, k) : 0.0));
  return acc - kCp * (th * dpi_<R>(d, m, fl, L, i, jp, k, i, jm, k)) * m.inv_dy;
}

// w face (i, j, k), k = 0..nz: k_tend_w
template <class R, class Ld>
__device__ __forceinline__ Jet<R> pt_w(const Dims& d, const Metric& m, const Flags& fl, Ld& L, int i, int j, int k) {
  using T = Jet<R>;
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const int kc = imin(imax(k, 0), nz - 1), kt = imin(k, nz), km = imax(k - 1, 0);
  const double dz = dzeta_(m, d, kc) * scale_(m, d, i, j);
  const T wt = LD(W, i, j, kt);
  const T wc = 0.5 * (LD(W, i, j, kc) + wt);
  const T wz = (wt - LD(W, i, j, km)) * (1.0 / dz);
  const T wx = (LD(W, imin(i + 1, nx - 1), j, kt) - LD(W, imax(i - 1, 0), j, kt)) * (0.5 * m.inv_dx);
  const T wy = (LD(W, i, imin(j + 1, ny - 1), kt) - LD(W, i, imax(j - 1, 0), kt)) * (0.5 * m.inv_dy);
  const T uc = 0.5 * (LD(U, i, j, kc) + LD(U, i + 1, j, kc));
  const T vc = 0.5 * (LD(V, i, j, kc) + LD(V, i, j + 1, kc));
  T acc = -(uc * wx + vc * wy + wc * wz);
  const double dz1 = dmax(dz, 1.0);
  const bool sp = fl.split_fast;
  const T th = 0.5 * (LDS(THETA, i, j, km, sp ? ref_(m.th0, d, i, j, km) : 0.0) +
                      LDS(THETA, i, j, kc, sp ? ref_(m.th0, d, i, j, kc) : 0.0));
  acc = acc - kCp * (th * dpi_<R>(d, m, fl, L, i, j, kc, i, j, km)) * (1.0 / dz1);
  const double th0 = ref_(m.th0, d, i, j, kc);
  const T thp = LDS(THETA, i, j, kc, th0);
  const T qcond = LD(QC, i, j, kc) + LD(QR, i, j, kc) + LD(QI, i, j, kc) + LD(QS, i, j, kc) + LD(QG, i, j, kc);
  return acc + kG * (thp * (1.0 / dmax(th0, 1.0)) + kBuoyMoist * LD(QV, i, j, kc) - qcond);
}

// rho cell (i, j, k): the mass-flux divergence of k_tend_cells; with
// split_fast the linear part -div(rho0 u) is taken out face by face
template <class R, class Ld>
__device__ __forceinline__ Jet<R> pt_rho(const Dims& d, const Metric& m, const Flags& fl, Ld& L, int i, int j,
                                         int k) {
  using T = Jet<R>;
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const bool sp = fl.split_fast;
  const double* r0 = m.rho0;
  const double dz = dmax(dzeta_(m, d, k) * scale_(m, d, i, j), 1.0);
  // rho at point p minus (with split) rho0 at point p0 (mass_div0 reads rho0
  // at clamped neighbours where the flux reads rho's ghost line)
  auto rr = [&](int a, int b, int c, int a0, int b0, int c0) {
    return LDS(RHO, a, b, c, sp ? ref_(r0, d, a0, b0, c0) : 0.0);
  };
  const T rc = rr(i, j, k, i, j, k);
  const T ex = 0.5 * (rc + rr(i + 1, j, k, imin(i + 1, nx - 1), j, k));
  const T wx = 0.5 * (rr(imax(i - 1, 0), j, k, imax(i - 1, 0), j, k) + rc);
  const T fx = LD(U, i + 1, j, k) * ex - LD(U, i, j, k) * wx;
  const T ny_ = 0.5 * (rc + rr(i, j + 1, k, i, imin(j + 1, ny - 1), k));
  const T sy = 0.5 * (rr(i, imax(j - 1, 0), k, i, imax(j - 1, 0), k) + rc);
  const T fy = LD(V, i, j + 1, k) * ny_ - LD(V, i, j, k) * sy;
  const int kp = imin(k + 1, nz - 1), km = imax(k - 1, 0);
  const T tz = 0.5 * (rc + rr(i, j, kp, i, j, kp));
  const T bz = 0.5 * (rr(i, j, km, i, j, km) + rc);
  const T fz = LD(W, i, j, k + 1) * tz - LD(W, i, j, k) * bz;
  return -(fx * m.inv_dx + fy * m.inv_dy + fz * (1.0 / dz));
}

// pi cell: second-order divergence damping (damping.cpp:48-53)
template <class R, class Ld>
__device__ __forceinline__ Jet<R> pt_pi(const Dims& d, const Metric& m, const Flags& fl, Ld& L, int i, int j, int k) {
  using T = Jet<R>;
  const T pc = LD(PI, i, j, k);
  const T lap = (LDC(PI, i + 1, j, k) - 2.0 * pc + LDC(PI, i - 1, j, k)) * (1.0 / (m.dx * m.dx)) +
                (LDC(PI, i, j + 1, k) - 2.0 * pc + LDC(PI, i, j - 1, k)) * (1.0 / (m.dy * m.dy));
  return -fl.div_damp * lap;
}

// central gradient of order 2/4/6 along one axis (advection.cpp:106-136)
template <class R>
__device__ __forceinline__ Jet<R> gradc_(Jet<R> m3, Jet<R> m2, Jet<R> m1, Jet<R> p1, Jet<R> p2, Jet<R> p3, double inv,
                                         int order) {
  switch (order) {
    case 4: return (m2 - 8.0 * m1 + 8.0 * p1 - p2) * (inv / 12.0);
    case 6: return (-m3 + 9.0 * m2 - 45.0 * m1 + 45.0 * p1 - 9.0 * p2 + p3) * (inv / 60.0);
    default: return (p1 - m1) * (0.5 * inv);
  }
}

// scalar q cell with the non-conservative central scheme (adv_nc) and the
// positivity clip of the moisture species
template <class R, class Ld>
__device__ __forceinline__ Jet<R> pt_scalar_nc(const Dims& d, const Metric& m, const Flags& fl, Ld& L, int q, int i,
                                               int j, int k) {
  using T = Jet<R>;
  const double dz = dzeta_(m, d, k) * scale_(m, d, i, j);
  const T ua = 0.5 * (LD(U, i, j, k) + LD(U, i + 1, j, k));
  const T va = 0.5 * (LD(V, i, j, k) + LD(V, i, j + 1, k));
  const T wa = 0.5 * (LD(W, i, j, k) + LD(W, i, j, k + 1));
  const int o = fl.advection;
  const bool w3 = (o == 6), w2 = (o == 4 || o == 6);
  const T z{(R)0, (R)0};
  const T gx = gradc_<R>(w3 ? LDC(q, i - 3, j, k) : z, w2 ? LDC(q, i - 2, j, k) : z, LDC(q, i - 1, j, k),
                         LDC(q, i + 1, j, k), w2 ? LDC(q, i + 2, j, k) : z, w3 ? LDC(q, i + 3, j, k) : z,
                         1.0 / m.dx, o);
  const T gy = gradc_<R>(w3 ? LDC(q, i, j - 3, k) : z, w2 ? LDC(q, i, j - 2, k) : z, LDC(q, i, j - 1, k),
                         LDC(q, i, j + 1, k), w2 ? LDC(q, i, j + 2, k) : z, w3 ? LDC(q, i, j + 3, k) : z,
                         1.0 / m.dy, o);
  const T gz = (LDC(q, i, j, k + 1) - LDC(q, i, j, k - 1)) * (0.5 / dz);
  T r = -(ua * gx + va * gy + wa * gz);
  if (q >= QV) {
    const T qc = LD(q, i, j, k);
    if (qc.v <= (R)0 && r.v < (R)0) r = z;
  }
  return r;
}

// WENO5 left-biased reconstruction (Advection::weno5_reconstruct,
// advection.cpp:62-98; the right-biased one is this of the reversed stencil)
template <class R>
__device__ __forceinline__ Jet<R> weno_left_(Jet<R> qm2, Jet<R> qm1, Jet<R> q0, Jet<R> q1, Jet<R> q2) {
  using T = Jet<R>;
  const double s6 = 1.0 / 6.0;
  const T v0 = (2.0 * qm2 - 7.0 * qm1 + 11.0 * q0) * s6;
  const T v1 = (-qm1 + 5.0 * q0 + 2.0 * q1) * s6;
  const T v2 = (2.0 * q0 + 5.0 * q1 - q2) * s6;
  const T e0 = qm2 - 2.0 * qm1 + q0, f0 = qm2 - 4.0 * qm1 + 3.0 * q0;
  const T e1 = qm1 - 2.0 * q0 + q1, f1 = qm1 - q1;
  const T e2 = q0 - 2.0 * q1 + q2, f2 = 3.0 * q0 - 4.0 * q1 + q2;
  const T s0 = (13.0 / 12.0) * (e0 * e0) + 0.25 * (f0 * f0) + 1e-6;
  const T s1 = (13.0 / 12.0) * (e1 * e1) + 0.25 * (f1 * f1) + 1e-6;
  const T s2 = (13.0 / 12.0) * (e2 * e2) + 0.25 * (f2 * f2) + 1e-6;
  // the weights d_k / s_k^2 scaled by (s0 s1 s2)^2: no 1/s^2 of s ~ 1e-6, so
  // the derivatives of the normalisation do not cancel large numbers
  const T p12 = s1 * s2, p02 = s0 * s2, p01 = s0 * s1;
  const T a0 = 0.1 * (p12 * p12), a1 = 0.6 * (p02 * p02), a2 = 0.3 * (p01 * p01);
  return (a0 * v0 + a1 * v1 + a2 * v2) / (a0 + a1 + a2);
}
// Lax-Friedrichs face flux 0.5 (u (qL + qR) - max(|u|, 1e-3) (qR - qL)),
// advection.cpp:160-170
template <class R>
__device__ __forceinline__ Jet<R> weno_flux_(Jet<R> qm2, Jet<R> qm1, Jet<R> q0, Jet<R> q1, Jet<R> q2, Jet<R> vel) {
  const Jet<R> ql = weno_left_<R>(qm2, qm1, q0, q1, q2);
  const Jet<R> qr = weno_left_<R>(q2, q1, q0, qm1, qm2);
  Jet<R> alpha{(R)1e-3, (R)0};
  if (vel.v >= (R)1e-3) alpha = vel;
  else if (vel.v <= (R)-1e-3) alpha = -vel;
  return 0.5 * (vel * (ql + qr) - alpha * (qr - ql));
}
// The face flux of direction dir (0 x, 1 y, 2 z) at face index (i, j, k)
// (k_weno_faces' stencil CL(f-3..f+1) and the normal wind at the face), as
// G = F(q - c) = F(q) - c u: the reconstruction is translation invariant, so
// shifting the stencil by c = q at its centre point (a value, without
// derivative) changes only the c u part. The small shifted values keep FP32
// accurate; a cell combines G with c and its own q without cancelling the
// large c u terms of its faces (pt_wcell).
template <class R, class Ld>
__device__ __forceinline__ Jet<R> pt_wface(const Dims& d, Ld& L, int q, int dir, int i, int j, int k, double c) {
  Jet<R> z[5];
  int di = 0, dj = 0, dk = 0;
  if (dir == 0) di = 1;
  else if (dir == 1) dj = 1;
  else dk = 1;
#pragma unroll
  for (int m = 0; m < 5; ++m) {
    const int a = iclamp(i + (m - 3) * di, 0, d.nx - 1), b = iclamp(j + (m - 3) * dj, 0, d.ny - 1);
    z[m] = L(q, d.idx(a, b, iclamp(k + (m - 3) * dk, 0, d.nz - 1)), c);
  }
  const Jet<R> vel = LD(dir == 0 ? U : (dir == 1 ? V : W), i, j, k);
  return weno_flux_<R>(z[0], z[1], z[2], z[3], z[4], vel);
}
// c of the face at index (i, j, k): q at the stencil's centre (the cell at
// the face's index, clamped)
__device__ __forceinline__ double wface_shift(const Dims& d, const double* q, int i, int j, int k) {
  return q[d.idx(iclamp(i, 0, d.nx - 1), iclamp(j, 0, d.ny - 1), iclamp(k, 0, d.nz - 1))];
}

// faces that exist for direction dir at index (i, j, k)
__device__ __forceinline__ bool face_exists(const Dims& d, int dir, int i, int j, int k) {
  if (dir == 0) return i <= d.nx && j < d.ny && k < d.nz;
  if (dir == 1) return i < d.nx && j <= d.ny && k < d.nz;
  return i < d.nx && j < d.ny && k <= d.nz;
}

// WENO cell (k_weno_cells) from the face fluxes Fx/Fy/Fz (value and
// derivative of each face, loaded by `face`), the advective-form term and
// the clip
struct FaceArr {
  double* v[3];  // G of the x, y, z faces (values)
  double* t[3];  // their tangents (TL only)
  double* c[3];  // their shifts c
};
// With F = G + c u and div = sum_f s_f u_f / D_f (s_f = +1 on the east,
// north and top faces, -1 on the others), the cell's
//   r = -sum_f s_f F_f / D_f (+ q div with weno_advective)
// is evaluated as
//   r = -sum_f s_f G_f / D_f + sum_f s_f (q - c_f) u_f / D_f   (advective)
//   r = -sum_f s_f (G_f + c_f u_f) / D_f                        (flux form)
// where q - c_f is a difference of two nearby values.
template <class R, class Ld>
__device__ __forceinline__ Jet<R> pt_wcell(const Dims& d, const Metric& m, const Flags& fl, Ld& L, const FaceArr& F,
                                           bool with_t, int q, int i, int j, int k, bool clip = true) {
  using T = Jet<R>;
  const double dz = dzeta_(m, d, k) * scale_(m, d, i, j);
  const double idz = 1.0 / dz;
  const T qc = LD(q, i, j, k);
  const bool vert = (k + 2 < d.nz || k >= 2);
  const bool adv = fl.weno_advective;
  T r{(R)0, (R)0};
  const size_t oc = d.idx(i, j, k);
  auto face = [&](int dir, int a, int b, int c, double sgn, double inv) {
    const size_t o = d.idx(a, b, c);
    const T G{(R)F.v[dir][o], with_t ? (R)F.t[dir][o] : (R)0};
    const double cf = F.c[dir][o];
    const T u = L(dir == 0 ? U : (dir == 1 ? V : W), o);
    if (adv) r = r + (-sgn * inv) * G + (sgn * inv) * (L(q, oc, cf) * u);  // (q - c_f) u
    else r = r + (-sgn * inv) * (G + u * cf);
  };
  face(0, i + 1, j, k, 1.0, m.inv_dx);
  face(0, i, j, k, -1.0, m.inv_dx);
  face(1, i, j + 1, k, 1.0, m.inv_dy);
  face(1, i, j, k, -1.0, m.inv_dy);
  if (vert) {
    face(2, i, j, k + 1, 1.0, idz);
    face(2, i, j, k, -1.0, idz);
  }
  if (clip && q >= QV && qc.v <= (R)0 && r.v < (R)0) r = T{(R)0, (R)0};
  return r;
}

// ---- tangent-linear kernels -------------------------------------------------
template <class R>
__global__ void k_tl_faces(Dims d, Metric m, Flags fl, const __grid_constant__ F12 b, const __grid_constant__ F12 p,
                           B12 out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i > d.nx || j > d.ny || k > d.nz) return;
  TlLoad<R> L{&b, &p};
  const size_t c = d.idx(i, j, k);
  if (j < d.ny && k < d.nz) out.f[U][c] = (double)pt_u<R>(d, m, fl, L, i, j, k).d;
  if (i < d.nx && k < d.nz) out.f[V][c] = (double)pt_v<R>(d, m, fl, L, i, j, k).d;
  if (i < d.nx && j < d.ny) out.f[W][c] = (double)pt_w<R>(d, m, fl, L, i, j, k).d;
}

template <class R>
__global__ void k_tl_cells(Dims d, Metric m, Flags fl, const __grid_constant__ F12 b, const __grid_constant__ F12 p,
                           B12 out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= d.nx || j >= d.ny || k >= d.nz) return;
  TlLoad<R> L{&b, &p};
  const size_t c = d.idx(i, j, k);
  out.f[RHO][c] = (double)pt_rho<R>(d, m, fl, L, i, j, k).d;
  out.f[PI][c] = fl.div_damp > 0.0 ? (double)pt_pi<R>(d, m, fl, L, i, j, k).d : 0.0;
  if (!fl.weno_scalars) {
    const int last = fl.moist ? QG : QV;
    for (int q = THETA; q <= last; ++q)
      if (q != PI) out.f[q][c] = (double)pt_scalar_nc<R>(d, m, fl, L, q, i, j, k).d;
  }
}

// WENO: the three face fluxes at index (i, j, k) (values, and tangents when with_t)
template <class R>
__global__ void k_tl_wface(Dims d, const __grid_constant__ F12 b, const __grid_constant__ F12 p, int q, FaceArr F,
                           int with_t) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i > d.nx || j > d.ny || k > d.nz) return;
  const size_t c = d.idx(i, j, k);
  const double sh = wface_shift(d, b.f[q], i, j, k);
  for (int dir = 0; dir < 3; ++dir) {
    if (!face_exists(d, dir, i, j, k)) continue;
    Jet<R> f;
    if (with_t) {
      TlLoad<R> L{&b, &p};
      f = pt_wface<R>(d, L, q, dir, i, j, k, sh);
      F.t[dir][c] = (double)f.d;
    } else {
      ValLoad<R> L{&b};
      f = pt_wface<R>(d, L, q, dir, i, j, k, sh);
    }
    F.v[dir][c] = (double)f.v;
    F.c[dir][c] = sh;
  }
}

template <class R>
__global__ void k_tl_wcell(Dims d, Metric m, Flags fl, const __grid_constant__ F12 b, const __grid_constant__ F12 p,
                           int q, FaceArr F, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= d.nx || j >= d.ny || k >= d.nz) return;
  TlLoad<R> L{&b, &p};
  out[d.idx(i, j, k)] = (double)pt_wcell<R>(d, m, fl, L, F, true, q, i, j, k).d;
}

// ---- adjoint kernels --------------------------------------------------------
// bar_in += (d pf / d loads) * lam, one pass per load
template <class R, class PF>
__device__ __forceinline__ void ad_scatter(const F12& b, const B12& bar, double lam, PF pf) {
  AdLoad<R> L{&b, 0, 0, -1, 0};
  for (int seed = 0; seed < kMaxLoads; ++seed) {
    L.seed = seed;
    L.n = 0;
    L.hq = -1;
    const Jet<R> r = pf(L);
    if (L.hq < 0) break;
    const double g = (double)r.d * lam;
    if (g != 0.0) atomicAdd(&bar.f[L.hq][L.hc], g);
  }
}

template <class R>
__global__ void k_ad_faces(Dims d, Metric m, Flags fl, const __grid_constant__ F12 b, const __grid_constant__ F12 bo,
                           const __grid_constant__ B12 bi) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i > d.nx || j > d.ny || k > d.nz) return;
  const size_t c = d.idx(i, j, k);
  if (j < d.ny && k < d.nz && bo.f[U][c] != 0.0)
    ad_scatter<R>(b, bi, bo.f[U][c], [&](AdLoad<R>& L) { return pt_u<R>(d, m, fl, L, i, j, k); });
  if (i < d.nx && k < d.nz && bo.f[V][c] != 0.0)
    ad_scatter<R>(b, bi, bo.f[V][c], [&](AdLoad<R>& L) { return pt_v<R>(d, m, fl, L, i, j, k); });
  if (i < d.nx && j < d.ny && bo.f[W][c] != 0.0)
    ad_scatter<R>(b, bi, bo.f[W][c], [&](AdLoad<R>& L) { return pt_w<R>(d, m, fl, L, i, j, k); });
}

template <class R>
__global__ void k_ad_cells(Dims d, Metric m, Flags fl, const __grid_constant__ F12 b, const __grid_constant__ F12 bo,
                           const __grid_constant__ B12 bi) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= d.nx || j >= d.ny || k >= d.nz) return;
  const size_t c = d.idx(i, j, k);
  if (bo.f[RHO][c] != 0.0)
    ad_scatter<R>(b, bi, bo.f[RHO][c], [&](AdLoad<R>& L) { return pt_rho<R>(d, m, fl, L, i, j, k); });
  if (fl.div_damp > 0.0 && bo.f[PI][c] != 0.0)
    ad_scatter<R>(b, bi, bo.f[PI][c], [&](AdLoad<R>& L) { return pt_pi<R>(d, m, fl, L, i, j, k); });
  if (!fl.weno_scalars) {
    const int last = fl.moist ? QG : QV;
    for (int q = THETA; q <= last; ++q)
      if (q != PI && bo.f[q][c] != 0.0)
        ad_scatter<R>(b, bi, bo.f[q][c], [&](AdLoad<R>& L) { return pt_scalar_nc<R>(d, m, fl, L, q, i, j, k); });
  }
}

// WENO cells: the bar each face flux sees (zero where the clip is active),
// into ebar, and the advective-form term's own scatter
template <class R>
__global__ void k_ad_wcell(Dims d, Metric m, Flags fl, const __grid_constant__ F12 b, int q, FaceArr F,
                           const double* __restrict__ bo, double* __restrict__ ebar, const __grid_constant__ B12 bi) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= d.nx || j >= d.ny || k >= d.nz) return;
  const size_t c = d.idx(i, j, k);
  double lam = bo[c];
  if (lam != 0.0 && q >= QV) {
    ValLoad<R> VL{&b};
    const Jet<R> r = pt_wcell<R>(d, m, fl, VL, F, false, q, i, j, k, false);
    if (VL(q, c).v <= (R)0 && r.v < (R)0) lam = 0.0;  // the clip holds R at zero
  }
  ebar[c] = lam;
  if (lam == 0.0 || !fl.weno_advective) return;
  // the cell's own q enters r (beyond its faces' G) through (q - c_f) u_f:
  // dr/dq = div; the winds' part is scattered per face (k_ad_wface)
  const double dz = dzeta_(m, d, k) * scale_(m, d, i, j);
  const bool vert = (k + 2 < d.nz || k >= 2);
  R div = ((R)b.f[U][d.idx(i + 1, j, k)] - (R)b.f[U][c]) * (R)m.inv_dx +
          ((R)b.f[V][d.idx(i, j + 1, k)] - (R)b.f[V][c]) * (R)m.inv_dy;
  if (vert) div += ((R)b.f[W][d.idx(i, j, k + 1)] - (R)b.f[W][c]) * (R)(1.0 / dz);
  atomicAdd(&bi.f[q][c], (double)div * lam);
}

// WENO faces: bar_F from the two cells beside each face, then the face's loads
// Face at index (i, j, k) of direction dir: cell R = the cell at that index
// (the face is its west / south / bottom face), cell L the one before it.
// aR = bar(R) / D_R and aL = bar(L) / D_L where the cell exists and uses the
// face (vertical faces only where the cell's vertical terms are on); then
// bar_G = aR - aL, and the face's wind also carries the cells' (q - c) u and
// c u parts (pt_wcell).
template <class R>
__global__ void k_ad_wface(Dims d, Metric m, Flags fl, const __grid_constant__ F12 b, int q,
                           const double* __restrict__ ebar, const __grid_constant__ B12 bi) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i > d.nx || j > d.ny || k > d.nz) return;
  const double sh = wface_shift(d, b.f[q], i, j, k);
  for (int dir = 0; dir < 3; ++dir) {
    if (!face_exists(d, dir, i, j, k)) continue;
    const int li = i - (dir == 0), lj = j - (dir == 1), lk = k - (dir == 2);
    bool hasR, hasL;
    double invR, invL;
    if (dir == 0) {
      hasR = i < d.nx;
      hasL = i >= 1;
      invR = invL = m.inv_dx;
    } else if (dir == 1) {
      hasR = j < d.ny;
      hasL = j >= 1;
      invR = invL = m.inv_dy;
    } else {
      hasR = k < d.nz && (k + 2 < d.nz || k >= 2);
      hasL = k >= 1 && (lk + 2 < d.nz || lk >= 2);
      invR = hasR ? 1.0 / (dzeta_(m, d, k) * scale_(m, d, i, j)) : 0.0;
      invL = hasL ? 1.0 / (dzeta_(m, d, lk) * scale_(m, d, i, j)) : 0.0;
    }
    const double aR = hasR ? ebar[d.idx(i, j, k)] * invR : 0.0;
    const double aL = hasL ? ebar[d.idx(li, lj, lk)] * invL : 0.0;
    const double lamG = aR - aL;
    if (aR == 0.0 && aL == 0.0) continue;
    double extra;  // the wind's part beyond G
    if (fl.weno_advective) {
      const R dR = hasR ? (R)(b.f[q][d.idx(i, j, k)] - sh) : (R)0;
      const R dL = hasL ? (R)(b.f[q][d.idx(li, lj, lk)] - sh) : (R)0;
      extra = -(double)dR * aR + (double)dL * aL;
    } else {
      extra = sh * lamG;
    }
    const int vq = dir == 0 ? U : (dir == 1 ? V : W);
    AdLoad<R> L{&b, 0, 0, -1, 0};
    for (int seed = 0; seed < kMaxLoads; ++seed) {
      L.seed = seed;
      L.n = 0;
      L.hq = -1;
      const Jet<R> g = pt_wface<R>(d, L, q, dir, i, j, k, sh);
      if (L.hq < 0) break;
      double v = (double)g.d * lamG;
      if (L.hq == vq) v += extra;
      if (v != 0.0) atomicAdd(&bi.f[L.hq][L.hc], v);
    }
  }
}

// ---- element-wise operations on whole perturbation fields ---------------------
__global__ void k_lin_axpy(size_t n, const double* __restrict__ x0, const double* __restrict__ r, double a,
                           double* __restrict__ out) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x)
    out[e] = x0[e] + a * r[e];
}
__global__ void k_lin_scale_add(size_t n, const double* __restrict__ x, double a, double* __restrict__ acc) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x)
    acc[e] += a * x[e];
}
__global__ void k_lin_f64_to_f32(size_t n, const double* __restrict__ x, float* __restrict__ y) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x)
    y[e] = (float)x[e];
}
__global__ void k_lin_f32_to_f64(size_t n, const float* __restrict__ x, double* __restrict__ y) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x)
    y[e] = (double)x[e];
}
// FP32 working state (perturbation form, per-level reference) -> FP64 totals
__global__ void k_working_to_f64(Dims d, const double* __restrict__ r0, const double* __restrict__ t0,
                                 const double* __restrict__ p0, const __grid_constant__ WS w, B12 out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i > d.nx || j > d.ny || k > d.nz) return;
  const size_t c = d.idx(i, j, k);
  if (j < d.ny && k < d.nz) out.f[U][c] = (double)w.f[U][c];
  if (i < d.nx && k < d.nz) out.f[V][c] = (double)w.f[V][c];
  if (i < d.nx && j < d.ny) out.f[W][c] = (double)w.f[W][c];
  if (k < d.nz) {  // cells incl. the ghost column and row
    out.f[RHO][c] = (double)w.f[RHO][c] + r0[k];
    out.f[THETA][c] = (double)w.f[THETA][c] + t0[k];
    out.f[PI][c] = (double)w.f[PI][c] + p0[k];
    for (int q = QV; q < NSPECIES; ++q)
      if (w.f[q]) out.f[q][c] = (double)w.f[q][c];
  }
}

dim3 grid3_(const Dims& d, int ni, int nj, int nk, dim3 blk) {
  return dim3((ni + blk.x - 1) / blk.x, (nj + blk.y - 1) / blk.y, nk);
}
const dim3 kB(32, 4, 1);

F12 f12(double* const* f) {
  F12 s;
  for (int q = 0; q < NSPECIES; ++q) s.f[q] = f[q];
  return s;
}
B12 b12(double* const* f) {
  B12 s;
  for (int q = 0; q < NSPECIES; ++q) s.f[q] = f[q];
  return s;
}
FaceArr face_arr(const Dims& d, double* face) {
  const size_t nf = d.plane * (size_t)(d.nz + 1);
  FaceArr F;
  for (int a = 0; a < 3; ++a) {
    F.v[a] = face + a * nf;
    F.t[a] = face + (3 + a) * nf;
    F.c[a] = face + (6 + a) * nf;
  }
  return F;
}
int scalar_last(const Flags& fl) { return fl.moist ? QG : QV; }

template <class R>
void tend_tl_t(const Dims& d, const Metric& m, const Flags& fl, double* const* base, double* const* pert,
               double* const* out, double* face, cudaStream_t s) {
  const size_t nf = d.plane * (size_t)(d.nz + 1);
  for (int q = 0; q < NSPECIES; ++q) cudaMemsetAsync(out[q], 0, nf * sizeof(double), s);
  const F12 b = f12(base), p = f12(pert);
  const B12 o = b12(out);
  k_tl_faces<R><<<grid3_(d, d.nx + 1, d.ny + 1, d.nz + 1, kB), kB, 0, s>>>(d, m, fl, b, p, o);
  k_tl_cells<R><<<grid3_(d, d.nx, d.ny, d.nz, kB), kB, 0, s>>>(d, m, fl, b, p, o);
  if (fl.weno_scalars) {
    const FaceArr F = face_arr(d, face);
    for (int q = THETA; q <= scalar_last(fl); ++q) {
      if (q == PI) continue;
      k_tl_wface<R><<<grid3_(d, d.nx + 1, d.ny + 1, d.nz + 1, kB), kB, 0, s>>>(d, b, p, q, F, 1);
      k_tl_wcell<R><<<grid3_(d, d.nx, d.ny, d.nz, kB), kB, 0, s>>>(d, m, fl, b, p, q, F, out[q]);
    }
  }
}

template <class R>
void tend_ad_t(const Dims& d, const Metric& m, const Flags& fl, double* const* base, double* const* bar_out,
               double* const* bar_in, double* face, double* cell_scr, cudaStream_t s) {
  const F12 b = f12(base), bo = f12(bar_out);
  const B12 bi = b12(bar_in);
  k_ad_faces<R><<<grid3_(d, d.nx + 1, d.ny + 1, d.nz + 1, kB), kB, 0, s>>>(d, m, fl, b, bo, bi);
  k_ad_cells<R><<<grid3_(d, d.nx, d.ny, d.nz, kB), kB, 0, s>>>(d, m, fl, b, bo, bi);
  if (fl.weno_scalars) {
    const FaceArr F = face_arr(d, face);
    for (int q = THETA; q <= scalar_last(fl); ++q) {
      if (q == PI) continue;
      k_tl_wface<R><<<grid3_(d, d.nx + 1, d.ny + 1, d.nz + 1, kB), kB, 0, s>>>(d, b, b, q, F, 0);
      k_ad_wcell<R><<<grid3_(d, d.nx, d.ny, d.nz, kB), kB, 0, s>>>(d, m, fl, b, q, F, bar_out[q], cell_scr, bi);
      k_ad_wface<R><<<grid3_(d, d.nx + 1, d.ny + 1, d.nz + 1, kB), kB, 0, s>>>(d, m, fl, b, q, cell_scr, bi);
    }
  }
}

int lin_blocks(size_t n) { return (int)std::min<size_t>((n + 255) / 256, 152 * 16); }

}  // namespace

void tend_tl(const Dims& d, const Metric& m, const Flags& fl, double* const* base, double* const* pert,
             double* const* out, double* face, bool f32, cudaStream_t s) {
  if (f32) tend_tl_t<float>(d, m, fl, base, pert, out, face, s);
  else tend_tl_t<double>(d, m, fl, base, pert, out, face, s);
}

void tend_ad(const Dims& d, const Metric& m, const Flags& fl, double* const* base, double* const* bar_out,
             double* const* bar_in, double* face, double* cell_scr, bool f32, cudaStream_t s) {
  if (f32) tend_ad_t<float>(d, m, fl, base, bar_out, bar_in, face, cell_scr, s);
  else tend_ad_t<double>(d, m, fl, base, bar_out, bar_in, face, cell_scr, s);
}

void lin_axpy(size_t n, const double* x0, const double* r, double a, double* out, cudaStream_t s) {
  k_lin_axpy<<<lin_blocks(n), 256, 0, s>>>(n, x0, r, a, out);
}
void lin_scale_add(size_t n, const double* x, double a, double* acc, cudaStream_t s) {
  k_lin_scale_add<<<lin_blocks(n), 256, 0, s>>>(n, x, a, acc);
}
void lin_to_f32(size_t n, const double* x, float* y, cudaStream_t s) {
  k_lin_f64_to_f32<<<lin_blocks(n), 256, 0, s>>>(n, x, y);
}
void lin_to_f64(size_t n, const float* x, double* y, cudaStream_t s) {
  k_lin_f32_to_f64<<<lin_blocks(n), 256, 0, s>>>(n, x, y);
}
void working_to_f64(const Dims& d, const Tab& t, const WS& w, double* const* out, cudaStream_t s) {
  k_working_to_f64<<<grid3_(d, d.nx + 1, d.ny + 1, d.nz + 1, kB), kB, 0, s>>>(d, t.r0d, t.t0dd, t.p0d, w, b12(out));
}

}  // namespace vgb
