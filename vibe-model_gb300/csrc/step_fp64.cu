// vibe-model_gb300/csrc/step_fp64.cu
//
// Plain FP64 path of the dynamics step. Each kernel restates one loop nest of
// the reference's serial step in the same operation order, one thread per
// output point, so results agree with the reference to rounding (FMA
// contraction is the only source of difference). On GB300 FP64 runs at
// ~1/73 of the FP32 rate, so this path is FP64-ALU bound; it exists as the
// exact baseline the mixed path is measured against.
#include "step_kernels.cuh"

// Built twice: as is (FMA contraction on, the fast FP64 path) and with
// -DVGB_FP64_EXACT --fmad=false, which keeps every multiply and add
// separately rounded in the reference's operation order, so results equal
// the serial reference bit for bit.
#ifdef VGB_FP64_EXACT
#define FP64_FN(name) name##_exact
#else
#define FP64_FN(name) name
#endif

// a / b as the reference writes it (bit-exact build), or a * rb with the
// reciprocal rb = 1/b computed once (fast build: an FP64 division costs a
// dozen FP64 operations on this GPU, which has few of them)
#ifdef VGB_FP64_EXACT
#define DIVR(a, b, rb) ((a) / (b))
#else
#define DIVR(a, b, rb) ((a) * (rb))
#endif

namespace vgb {
namespace {

struct CS {  // const state view
  const double* __restrict__ f[NSPECIES];
};
struct MS {  // mutable state view
  double* __restrict__ f[NSPECIES];
};

#define IDX(i, j, k) (d.idx((i), (j), (k)))
#define SF(sp, i, j, k) (s.f[sp][IDX(i, j, k)])
#define CLP(sp, i, j, k) \
  (s.f[sp][IDX(iclamp((i), 0, d.nx - 1), iclamp((j), 0, d.ny - 1), iclamp((k), 0, d.nz - 1))])

__device__ inline double dzeta(const Metric& m, const Dims& d, int k) { return m.dzeta[iclamp(k, 0, d.nz - 1)]; }
__device__ inline double scale_at(const Metric& m, const Dims& d, int i, int j) {
  return m.scale[(size_t)iclamp(j, 0, d.ny - 1) * d.nx + iclamp(i, 0, d.nx - 1)];
}
__device__ inline double R3(const double* f, const Dims& d, int i, int j, int k) { return f[d.idx(i, j, k)]; }

// Exner difference of the pressure-gradient terms (total or pi').
__device__ inline double dpi(const CS& s, const Metric& m, const Dims& d, const Flags& fl,
                             int ia, int ja, int ka, int ib, int jb, int kb) {
  if (!fl.pgf_pert) return SF(PI, ia, ja, ka) - SF(PI, ib, jb, kb);
  return (SF(PI, ia, ja, ka) - R3(m.pi0, d, ia, ja, ka)) - (SF(PI, ib, jb, kb) - R3(m.pi0, d, ib, jb, kb));
}

// Advection::weno5_reconstruct, advection.cpp:62-98
__device__ inline void weno5(double qm2, double qm1, double q0, double q1, double q2, double& ql, double& qr) {
  const double eps = 1e-6, d0 = 0.1, d1 = 0.6, d2 = 0.3;
  const double v0 = (2.0 * qm2 - 7.0 * qm1 + 11.0 * q0) / 6.0;
  const double v1 = (-qm1 + 5.0 * q0 + 2.0 * q1) / 6.0;
  const double v2 = (2.0 * q0 + 5.0 * q1 - q2) / 6.0;
  const double e0 = qm2 - 2.0 * qm1 + q0, f0 = qm2 - 4.0 * qm1 + 3.0 * q0;
  const double e1 = qm1 - 2.0 * q0 + q1, f1 = qm1 - q1;
  const double e2 = q0 - 2.0 * q1 + q2, f2 = 3.0 * q0 - 4.0 * q1 + q2;
  const double b0 = (13.0 / 12.0) * (e0 * e0) + 0.25 * (f0 * f0);
  const double b1 = (13.0 / 12.0) * (e1 * e1) + 0.25 * (f1 * f1);
  const double b2 = (13.0 / 12.0) * (e2 * e2) + 0.25 * (f2 * f2);
  const double a0 = d0 / ((eps + b0) * (eps + b0));
  const double a1 = d1 / ((eps + b1) * (eps + b1));
  const double a2 = d2 / ((eps + b2) * (eps + b2));
  ql = (a0 * v0 + a1 * v1 + a2 * v2) / (a0 + a1 + a2);
  const double u0 = (2.0 * q2 - 7.0 * q1 + 11.0 * q0) / 6.0;
  const double u1 = (-q1 + 5.0 * q0 + 2.0 * qm1) / 6.0;
  const double u2 = (2.0 * q0 + 5.0 * qm1 - qm2) / 6.0;
  const double g0e = q2 - 2.0 * q1 + q0, g0f = q2 - 4.0 * q1 + 3.0 * q0;
  const double g1e = q1 - 2.0 * q0 + qm1, g1f = q1 - qm1;
  const double g2e = q0 - 2.0 * qm1 + qm2, g2f = 3.0 * q0 - 4.0 * qm1 + qm2;
  const double g0 = (13.0 / 12.0) * (g0e * g0e) + 0.25 * (g0f * g0f);
  const double g1 = (13.0 / 12.0) * (g1e * g1e) + 0.25 * (g1f * g1f);
  const double g2 = (13.0 / 12.0) * (g2e * g2e) + 0.25 * (g2f * g2f);
  const double c0 = d0 / ((eps + g0) * (eps + g0));
  const double c1 = d1 / ((eps + g1) * (eps + g1));
  const double c2 = d2 / ((eps + g2) * (eps + g2));
  qr = (c0 * u0 + c1 * u1 + c2 * u2) / (c0 + c1 + c2);
}
#ifdef VGB_FP64_EXACT
__device__ inline double weno_face(double qm2, double qm1, double q0, double q1, double q2, double vel) {
  double ql, qr;
  weno5(qm2, qm1, q0, q1, q2, ql, qr);
  const double alpha = dmax(fabs(vel), 1e-3);
  return 0.5 * (vel * (ql + qr) - alpha * (qr - ql));
}
#else
// The same face flux with the arithmetic arranged for the FP64 pipe: the
// right-biased reconstruction is the left-biased one of the reversed
// stencil (same three smoothness indicators, reversed), the weights
// a_k = d_k / s_k^2 (s_k = eps + beta_k) are normalised with one division
// by scaling numerator and denominator with (s0 s1 s2)^2, the 1/6 is a
// multiplication, and for |vel| >= 1e-3 the Lax-Friedrichs flux
// 0.5*(vel*(ql+qr) - |vel|*(qr-ql)) is vel times the upwind reconstruction
// alone. Equal to the reference's to rounding.
__device__ inline double weno_left_d(double qm2, double qm1, double q0, double q1, double q2, double s0, double s1,
                                     double s2) {
  const double sixth = 1.0 / 6.0;
  const double v0 = (2.0 * qm2 - 7.0 * qm1 + 11.0 * q0) * sixth;
  const double v1 = (-qm1 + 5.0 * q0 + 2.0 * q1) * sixth;
  const double v2 = (2.0 * q0 + 5.0 * q1 - q2) * sixth;
  const double p01 = s0 * s1, p02 = s0 * s2, p12 = s1 * s2;
  const double w0 = 0.1 * (p12 * p12), w1 = 0.6 * (p02 * p02), w2 = 0.3 * (p01 * p01);
  return (w0 * v0 + w1 * v1 + w2 * v2) / (w0 + w1 + w2);
}
__device__ inline double weno_face(double qm2, double qm1, double q0, double q1, double q2, double vel) {
  const double eps = 1e-6;
  const double e0 = qm2 - 2.0 * qm1 + q0, f0 = qm2 - 4.0 * qm1 + 3.0 * q0;
  const double e1 = qm1 - 2.0 * q0 + q1, f1 = qm1 - q1;
  const double e2 = q0 - 2.0 * q1 + q2, f2 = 3.0 * q0 - 4.0 * q1 + q2;
  const double s0 = eps + (13.0 / 12.0) * (e0 * e0) + 0.25 * (f0 * f0);
  const double s1 = eps + (13.0 / 12.0) * (e1 * e1) + 0.25 * (f1 * f1);
  const double s2 = eps + (13.0 / 12.0) * (e2 * e2) + 0.25 * (f2 * f2);
  const bool up = vel >= 0.0;
  const double a0 = up ? qm2 : q2, a1 = up ? qm1 : q1, a3 = up ? q1 : qm1, a4 = up ? q2 : qm2;
  const double t0 = up ? s0 : s2, t2 = up ? s2 : s0;
  const double rec = weno_left_d(a0, a1, q0, a3, a4, t0, s1, t2);
  if (fabs(vel) >= 1e-3) return vel * rec;
  const double oth = weno_left_d(a4, a3, q0, a1, a0, t2, s1, t0);
  const double ql = up ? rec : oth, qr = up ? oth : rec;
  return 0.5 * (vel * (ql + qr) - 1e-3 * (qr - ql));
}
#endif

// grad_x / grad_y, advection.cpp:106-136 (q = species index)
__device__ inline double grad_x(const CS& s, const Dims& d, int q, int i, int j, int k, double inv_dx, int order) {
  switch (order) {
    case 4:
      return (CLP(q, i - 2, j, k) - 8.0 * CLP(q, i - 1, j, k) + 8.0 * CLP(q, i + 1, j, k) - CLP(q, i + 2, j, k)) *
             (inv_dx / 12.0);
    case 6:
      return (-CLP(q, i - 3, j, k) + 9.0 * CLP(q, i - 2, j, k) - 45.0 * CLP(q, i - 1, j, k) +
              45.0 * CLP(q, i + 1, j, k) - 9.0 * CLP(q, i + 2, j, k) + CLP(q, i + 3, j, k)) *
             (inv_dx / 60.0);
    default:
      return (CLP(q, i + 1, j, k) - CLP(q, i - 1, j, k)) * (0.5 * inv_dx);
  }
}
__device__ inline double grad_y(const CS& s, const Dims& d, int q, int i, int j, int k, double inv_dy, int order) {
  switch (order) {
    case 4:
      return (CLP(q, i, j - 2, k) - 8.0 * CLP(q, i, j - 1, k) + 8.0 * CLP(q, i, j + 1, k) - CLP(q, i, j + 2, k)) *
             (inv_dy / 12.0);
    case 6:
      return (-CLP(q, i, j - 3, k) + 9.0 * CLP(q, i, j - 2, k) - 45.0 * CLP(q, i, j - 1, k) +
              45.0 * CLP(q, i, j + 1, k) - 9.0 * CLP(q, i, j + 2, k) + CLP(q, i, j + 3, k)) *
             (inv_dy / 60.0);
    default:
      return (CLP(q, i, j + 1, k) - CLP(q, i, j - 1, k)) * (0.5 * inv_dy);
  }
}

__device__ inline double cor_f(const Metric& m, const Flags& fl, const Dims& d, int j) {
  if (fl.coriolis != 2) return m.f0;
  const double y = (0.0 + (double)j + 0.5) * m.dy;
  const double y0 = 0.5 * (double)d.ny * m.dy;
  return m.f0 + m.beta * (y - y0);
}

// linear mass divergence -div(rho0 u), equations.cpp:187-200
__device__ inline double mass_div0(const CS& s, const Metric& m, const Dims& d, int i, int j, int k) {
  const double* r0 = m.rho0;
  const double dz = dmax(dzeta(m, d, k) * scale_at(m, d, i, j), 1.0);
  const double fx = SF(U, i + 1, j, k) * 0.5 * (R3(r0, d, i, j, k) + R3(r0, d, imin(i + 1, d.nx - 1), j, k)) -
                    SF(U, i, j, k) * 0.5 * (R3(r0, d, imax(i - 1, 0), j, k) + R3(r0, d, i, j, k));
  const double fy = SF(V, i, j + 1, k) * 0.5 * (R3(r0, d, i, j, k) + R3(r0, d, i, imin(j + 1, d.ny - 1), k)) -
                    SF(V, i, j, k) * 0.5 * (R3(r0, d, i, imax(j - 1, 0), k) + R3(r0, d, i, j, k));
  const double fz = SF(W, i, j, k + 1) * 0.5 * (R3(r0, d, i, j, k) + R3(r0, d, i, j, imin(k + 1, d.nz - 1))) -
                    SF(W, i, j, k) * 0.5 * (R3(r0, d, i, j, imax(k - 1, 0)) + R3(r0, d, i, j, k));
  return -(DIVR(fx, m.dx, m.inv_dx) + DIVR(fy, m.dy, m.inv_dy) + DIVR(fz, dz, 1.0 / dz));
}

// acoustic pressure-gradient tendencies, equations.cpp:157-184
__device__ inline double ac_u(const CS& s, const Metric& m, const Dims& d, const Flags& fl, int i, int j, int k) {
  const int ip = imin(i, d.nx - 1), im = imax(i - 1, 0);
  const double t0 = 0.5 * (R3(m.th0, d, im, j, k) + R3(m.th0, d, ip, j, k));
  return DIVR(-kCp * t0 * dpi(s, m, d, fl, ip, j, k, im, j, k), m.dx, m.inv_dx);
}
__device__ inline double ac_v(const CS& s, const Metric& m, const Dims& d, const Flags& fl, int i, int j, int k) {
  const int jp = imin(j, d.ny - 1), jm = imax(j - 1, 0);
  const double t0 = 0.5 * (R3(m.th0, d, i, jm, k) + R3(m.th0, d, i, jp, k));
  return DIVR(-kCp * t0 * dpi(s, m, d, fl, i, jp, k, i, jm, k), m.dy, m.inv_dy);
}
__device__ inline double ac_w(const CS& s, const Metric& m, const Dims& d, const Flags& fl, int i, int j, int k) {
  const int kc = imin(imax(k, 0), d.nz - 1), km = imax(k - 1, 0);
  const double dz = dmax(dzeta(m, d, kc) * scale_at(m, d, i, j), 1.0);
  const double t0 = 0.5 * (R3(m.th0, d, i, j, km) + R3(m.th0, d, i, j, kc));
  return -kCp * t0 * dpi(s, m, d, fl, i, j, kc, i, j, km) / dz;
}

// ---- slow tendencies, equations.cpp:60-150 -------------------------------

// u faces: Advection::momentum u-part (advection.cpp:260-278), Coriolis
// (coriolis.cpp:51-59), PGF (equations.cpp:72-80) [- acoustic u if split].
__global__ void k_tend_u(Dims d, Metric m, Flags fl, CS s, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i > d.nx || j >= d.ny || k >= d.nz) return;
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const int ip = imin(i, nx - 1);
  double acc = 0.0;
  {
    const double dz = dzeta(m, d, imin(k, nz - 1)) * scale_at(m, d, ip, j);
    const double uc = 0.5 * (SF(U, imax(i - 1, 0), j, k) + SF(U, ip, j, k));
    const double ux = DIVR(SF(U, ip, j, k) - SF(U, imax(i - 1, 0), j, k), m.dx, m.inv_dx);
    const double uy = DIVR(SF(U, ip, imin(j + 1, ny - 1), k) - SF(U, ip, imax(j - 1, 0), k), 2.0 * m.dy, 0.5 * m.inv_dy);
    const double uz = (SF(U, ip, j, imin(k + 1, nz - 1)) - SF(U, ip, j, imax(k - 1, 0))) / (2.0 * dz);
    const double vc = 0.25 * (SF(V, imax(i - 1, 0), imax(j - 1, 0), k) + SF(V, ip, imax(j - 1, 0), k) +
                              SF(V, imax(i - 1, 0), j, k) + SF(V, ip, j, k));
    const double wc = 0.5 * (SF(W, ip, j, k) + SF(W, ip, j, imin(k + 1, nz - 1)));
    acc -= uc * ux + vc * uy + wc * uz;
  }
  if (fl.coriolis) {
    const double v_at_u = 0.25 * (SF(V, imax(i - 1, 0), imax(j - 1, 0), k) + SF(V, imin(i, nx - 1), imax(j - 1, 0), k) +
                                  SF(V, imax(i - 1, 0), j, k) + SF(V, imin(i, nx - 1), j, k));
    acc += cor_f(m, fl, d, j) * v_at_u;
  }
  {
    const int im = imax(i - 1, 0);
    const double th = 0.5 * (SF(THETA, im, j, k) + SF(THETA, ip, j, k));
    acc -= DIVR(kCp * th * dpi(s, m, d, fl, ip, j, k, im, j, k), m.dx, m.inv_dx);
  }
  if (fl.split_fast) acc -= ac_u(s, m, d, fl, i, j, k);
  out[IDX(i, j, k)] = acc;
}

__global__ void k_tend_v(Dims d, Metric m, Flags fl, CS s, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= d.nx || j > d.ny || k >= d.nz) return;
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const int jp = imin(j, ny - 1);
  double acc = 0.0;
  {
    const double dz = dzeta(m, d, imin(k, nz - 1)) * scale_at(m, d, i, jp);
    const double vc = 0.5 * (SF(V, i, imax(j - 1, 0), k) + SF(V, i, jp, k));
    const double vy = DIVR(SF(V, i, jp, k) - SF(V, i, imax(j - 1, 0), k), m.dy, m.inv_dy);
    const double vx = DIVR(SF(V, imin(i + 1, nx - 1), jp, k) - SF(V, imax(i - 1, 0), jp, k), 2.0 * m.dx, 0.5 * m.inv_dx);
    const double vz = (SF(V, i, jp, imin(k + 1, nz - 1)) - SF(V, i, jp, imax(k - 1, 0))) / (2.0 * dz);
    const double uc = 0.25 * (SF(U, imax(i - 1, 0), imax(j - 1, 0), k) + SF(U, i, imax(j - 1, 0), k) +
                              SF(U, imax(i - 1, 0), jp, k) + SF(U, i, jp, k));
    const double wc = 0.5 * (SF(W, i, jp, k) + SF(W, i, jp, imin(k + 1, nz - 1)));
    acc -= uc * vx + vc * vy + wc * vz;
  }
  if (fl.coriolis) {
    const double u_at_v = 0.25 * (SF(U, imax(i - 1, 0), imax(j - 1, 0), k) + SF(U, i, imax(j - 1, 0), k) +
                                  SF(U, imax(i - 1, 0), imin(j, ny - 1), k) + SF(U, i, imin(j, ny - 1), k));
    acc -= cor_f(m, fl, d, j) * u_at_v;
  }
  {
    const int jm = imax(j - 1, 0);
    const double th = 0.5 * (SF(THETA, i, jm, k) + SF(THETA, i, jp, k));
    acc -= DIVR(kCp * th * dpi(s, m, d, fl, i, jp, k, i, jm, k), m.dy, m.inv_dy);
  }
  if (fl.split_fast) acc -= ac_v(s, m, d, fl, i, j, k);
  out[IDX(i, j, k)] = acc;
}

__global__ void k_tend_w(Dims d, Metric m, Flags fl, CS s, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= d.nx || j >= d.ny || k > d.nz) return;
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const int kc = imin(imax(k, 0), nz - 1);
  double acc = 0.0;
  {
    const double dz = dzeta(m, d, kc) * scale_at(m, d, i, j);
    const double wc = 0.5 * (SF(W, i, j, kc) + SF(W, i, j, imin(k, nz)));
    const double wz = (SF(W, i, j, imin(k, nz)) - SF(W, i, j, imax(k - 1, 0))) / dz;
    const double wx = DIVR(SF(W, imin(i + 1, nx - 1), j, imin(k, nz)) - SF(W, imax(i - 1, 0), j, imin(k, nz)), 2.0 * m.dx,
                           0.5 * m.inv_dx);
    const double wy = DIVR(SF(W, i, imin(j + 1, ny - 1), imin(k, nz)) - SF(W, i, imax(j - 1, 0), imin(k, nz)), 2.0 * m.dy,
                           0.5 * m.inv_dy);
    const double uc = 0.5 * (SF(U, i, j, kc) + SF(U, i + 1, j, kc));
    const double vc = 0.5 * (SF(V, i, j, kc) + SF(V, i, j + 1, kc));
    acc -= uc * wx + vc * wy + wc * wz;
  }
  {
    const int km = imax(k - 1, 0);
    const double dz = dmax(dzeta(m, d, kc) * scale_at(m, d, i, j), 1.0);
    const double th = 0.5 * (SF(THETA, i, j, km) + SF(THETA, i, j, kc));
    acc -= kCp * th * dpi(s, m, d, fl, i, j, kc, i, j, km) / dz;
    const double th0 = R3(m.th0, d, i, j, kc);
    const double thp = SF(THETA, i, j, kc) - th0;
    const double qcond = SF(QC, i, j, kc) + SF(QR, i, j, kc) + SF(QI, i, j, kc) + SF(QS, i, j, kc) + SF(QG, i, j, kc);
    acc += kG * (thp / dmax(th0, 1.0) + kBuoyMoist * SF(QV, i, j, kc) - qcond);
  }
  if (fl.split_fast) acc -= ac_w(s, m, d, fl, i, j, k);
  out[IDX(i, j, k)] = acc;
}

// Advection::scalar_nonconservative, advection.cpp:224-244
__device__ double adv_nc(const CS& s, const Metric& m, const Dims& d, const Flags& fl, int q, int i, int j, int k) {
  const double dz = dzeta(m, d, k) * scale_at(m, d, i, j);
  const double ua = 0.5 * (SF(U, i, j, k) + SF(U, i + 1, j, k));
  const double va = 0.5 * (SF(V, i, j, k) + SF(V, i, j + 1, k));
  const double wa = 0.5 * (SF(W, i, j, k) + SF(W, i, j, k + 1));
  return -(ua * grad_x(s, d, q, i, j, k, 1.0 / m.dx, fl.advection) +
           va * grad_y(s, d, q, i, j, k, 1.0 / m.dy, fl.advection) +
           wa * (CLP(q, i, j, k + 1) - CLP(q, i, j, k - 1)) * (0.5 / dz));
}

// Advection::scalar WENO5 branch, advection.cpp:144-187, face fluxes.
// Each cell's east flux and its east neighbour's west flux are the same
// number: the clamped stencil of a face is the same seen from either side
// (at i = nx the clamps make the east flux of cell nx-1 the stencil centred
// on face nx). So every face flux is computed once, face f of a direction
// from CL(f-3..f+1) and the normal wind at f:
//   fx(f, j, k), f = 0..nx; fy(i, f, k), f = 0..ny; fz(i, j, f), f = 0..nz.
__global__ void k_weno_faces(Dims d, CS s, int q, double* __restrict__ fx, double* __restrict__ fy,
                             double* __restrict__ fz) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i > d.nx || j > d.ny || k > d.nz) return;
  const size_t c = IDX(i, j, k);
  if (j < d.ny && k < d.nz)
    fx[c] = weno_face(CLP(q, i - 3, j, k), CLP(q, i - 2, j, k), CLP(q, i - 1, j, k), CLP(q, i, j, k),
                      CLP(q, i + 1, j, k), SF(U, i, j, k));
  if (i < d.nx && k < d.nz)
    fy[c] = weno_face(CLP(q, i, j - 3, k), CLP(q, i, j - 2, k), CLP(q, i, j - 1, k), CLP(q, i, j, k),
                      CLP(q, i, j + 1, k), SF(V, i, j, k));
  if (i < d.nx && j < d.ny)
    fz[c] = weno_face(CLP(q, i, j, k - 3), CLP(q, i, j, k - 2), CLP(q, i, j, k - 1), CLP(q, i, j, k),
                      CLP(q, i, j, k + 1), SF(W, i, j, k));
}

// The cell tendency from the face fluxes (+ q div(u) when weno_advective),
// with the positivity clip of the moisture species (equations.cpp:139-149).
__global__ void k_weno_cells(Dims d, Metric m, Flags fl, CS s, int q, const double* __restrict__ fx,
                             const double* __restrict__ fy, const double* __restrict__ fz, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= d.nx || j >= d.ny || k >= d.nz) return;
  const size_t c = IDX(i, j, k);
  const double dz = dzeta(m, d, k) * scale_at(m, d, i, j);
  const double idz = 1.0 / dz;
  const double qc = SF(q, i, j, k);
  const double fe = fx[IDX(i + 1, j, k)], fw = fx[c];
  const double fn = fy[IDX(i, j + 1, k)], fs = fy[c];
  double ft = 0.0, fb = 0.0;
  const bool vert = (k + 2 < d.nz || k >= 2);
  if (vert) {
    ft = fz[IDX(i, j, k + 1)];
    fb = fz[c];
  }
  double r = DIVR(-(fe - fw), m.dx, m.inv_dx) - DIVR(fn - fs, m.dy, m.inv_dy) - DIVR(ft - fb, dz, idz);
  if (fl.weno_advective) {
    double div = DIVR(SF(U, i + 1, j, k) - SF(U, i, j, k), m.dx, m.inv_dx) +
                 DIVR(SF(V, i, j + 1, k) - SF(V, i, j, k), m.dy, m.inv_dy);
    if (vert) div += DIVR(SF(W, i, j, k + 1) - SF(W, i, j, k), dz, idz);
    r += qc * div;
  }
  if (q >= QV && qc <= 0.0 && r < 0.0) r = 0.0;
  out[c] = r;
}

// Damping::tendencies laplacian, damping.cpp:48-53
__device__ inline double lap2(const double* __restrict__ f, const Metric& m, const Dims& d, int i, int j, int k) {
  auto cl = [&](int a, int b, int c) {
    return f[d.idx(iclamp(a, 0, d.nx - 1), iclamp(b, 0, d.ny - 1), iclamp(c, 0, d.nz - 1))];
  };
  const double fc = f[d.idx(i, j, k)];
  return (cl(i + 1, j, k) - 2.0 * fc + cl(i - 1, j, k)) / (m.dx * m.dx) +
         (cl(i, j + 1, k) - 2.0 * fc + cl(i, j - 1, k)) / (m.dy * m.dy);
}

__global__ void k_lap(Dims d, Metric m, const double* __restrict__ f, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= d.nx || j >= d.ny || k >= d.nz) return;
  out[d.idx(i, j, k)] = lap2(f, m, d, i, j, k);
}

// cell tendencies: mass (equations.cpp:112-127) [+ acoustic rho if split],
// scalars (:129-137), positivity clip (:139-149), divergence damping on pi
// (damping.cpp:43-74; lapf = laplacian of pi for order 4, else nullptr).
__global__ void k_tend_cells(Dims d, Metric m, Flags fl, CS s, MS out, const double* __restrict__ lapf) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= d.nx || j >= d.ny || k >= d.nz) return;
  const int nz = d.nz;
  const size_t c = IDX(i, j, k);
  {
    const double dz = dmax(dzeta(m, d, k) * scale_at(m, d, i, j), 1.0);
    const double fx = SF(U, i + 1, j, k) * 0.5 * (SF(RHO, i, j, k) + SF(RHO, i + 1, j, k)) -
                      SF(U, i, j, k) * 0.5 * (SF(RHO, imax(i - 1, 0), j, k) + SF(RHO, i, j, k));
    const double fy = SF(V, i, j + 1, k) * 0.5 * (SF(RHO, i, j, k) + SF(RHO, i, j + 1, k)) -
                      SF(V, i, j, k) * 0.5 * (SF(RHO, i, imax(j - 1, 0), k) + SF(RHO, i, j, k));
    const double fz = SF(W, i, j, k + 1) * 0.5 * (SF(RHO, i, j, k) + SF(RHO, i, j, imin(k + 1, nz - 1))) -
                      SF(W, i, j, k) * 0.5 * (SF(RHO, i, j, imax(k - 1, 0)) + SF(RHO, i, j, k));
    double r = -(DIVR(fx, m.dx, m.inv_dx) + DIVR(fy, m.dy, m.inv_dy) + DIVR(fz, dz, 1.0 / dz));
    if (fl.split_fast) r -= mass_div0(s, m, d, i, j, k);
    out.f[RHO][c] = r;
  }
  {
    double r = 0.0;
    if (fl.div_damp > 0.0) {
      if (fl.div_order <= 2) r -= fl.div_damp * lap2(s.f[PI], m, d, i, j, k);
      else r -= fl.div_damp * lap2(lapf, m, d, i, j, k);
    }
    out.f[PI][c] = r;
  }
  // the advected scalars' tendencies; with WENO5 they come from
  // k_weno_faces / k_weno_cells, launched after this kernel
  const int last = fl.moist ? QG : QV;
  for (int q = THETA; q <= QG; ++q) {
    if (q == PI || (fl.weno_scalars && q <= last)) continue;
    double r = 0.0;
    if (q <= last) r = adv_nc(s, m, d, fl, q, i, j, k);
    if (q >= QV && SF(q, i, j, k) <= 0.0 && r < 0.0) r = 0.0;
    out.f[q][c] = r;
  }
}

// s = s0 + a * R over one field's interior (+ faces). Ghost points untouched.
__global__ void k_axpy_field(Dims d, int ni, int nj, int nk, const double* __restrict__ s0,
                             const double* __restrict__ r, double a, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= ni || j >= nj || k >= nk) return;
  const size_t c = d.idx(i, j, k);
  out[c] = s0[c] + a * r[c];
}

// ---- explicit forward-backward substep, runge_kutta.cpp:65-75 -----------
__global__ void k_fb_mass(Dims d, Metric m, CS s, double* __restrict__ rho, double* __restrict__ pi, double dtau) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= d.nx || j >= d.ny || k >= d.nz) return;
  const size_t c = IDX(i, j, k);
  const double drho = mass_div0(s, m, d, i, j, k);
  const double r0 = dmax(m.rho0[c], 1e-8);
  const double dpi_t = (kRd / kCv) * (m.pi0[c] / r0) * drho;
  rho[c] += dtau * drho;
  pi[c] += dtau * dpi_t;
}

__global__ void k_fb_mom(Dims d, Metric m, Flags fl, CS s, double* __restrict__ u, double* __restrict__ v,
                         double* __restrict__ w, double dtau) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i > d.nx || j > d.ny || k > d.nz) return;
  const size_t c = IDX(i, j, k);
  if (j < d.ny && k < d.nz) u[c] += dtau * ac_u(s, m, d, fl, i, j, k);
  if (i < d.nx && k < d.nz) v[c] += dtau * ac_v(s, m, d, fl, i, j, k);
  if (i < d.nx && j < d.ny) w[c] += dtau * ac_w(s, m, d, fl, i, j, k);
}

// ---- the reference's HEVI substep, acoustic_substep.cpp:67-149 ----------
// update_mass_and_pressure (:67-94); note the operation order of the pi
// update differs from the explicit substep's.
__global__ void k_rhevi_mass(Dims d, Metric m, CS s, double* __restrict__ drho_out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= d.nx || j >= d.ny || k >= d.nz) return;
  const double* r0f = m.rho0;
  const double dz = dmax(dzeta(m, d, k) * scale_at(m, d, i, j), 1.0);
  const double r0 = R3(r0f, d, i, j, k);
  const double fx = SF(U, i + 1, j, k) * 0.5 * (r0 + R3(r0f, d, imin(i + 1, d.nx - 1), j, k)) -
                    SF(U, i, j, k) * 0.5 * (R3(r0f, d, imax(i - 1, 0), j, k) + r0);
  const double fy = SF(V, i, j + 1, k) * 0.5 * (r0 + R3(r0f, d, i, imin(j + 1, d.ny - 1), k)) -
                    SF(V, i, j, k) * 0.5 * (R3(r0f, d, i, imax(j - 1, 0), k) + r0);
  const double fz = SF(W, i, j, k + 1) * 0.5 * (r0 + R3(r0f, d, i, j, imin(k + 1, d.nz - 1))) -
                    SF(W, i, j, k) * 0.5 * (R3(r0f, d, i, j, imax(k - 1, 0)) + r0);
  drho_out[IDX(i, j, k)] = -(fx / m.dx + fy / m.dy + fz / dz);
}
__global__ void k_rhevi_apply(Dims d, Metric m, const double* __restrict__ drho, double* __restrict__ rho,
                              double* __restrict__ pi, double dtau) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= d.nx || j >= d.ny || k >= d.nz) return;
  const size_t c = d.idx(i, j, k);
  const double r0 = dmax(m.rho0[c], 1e-8);
  rho[c] += dtau * drho[c];
  pi[c] += dtau * (kRd / kCv) * (m.pi0[c] / r0) * drho[c];
}
// solve_vertical_implicit (:126-137): one thread per column, Thomas
// (helmholtz.cpp:57-86) with coefficients tri_a/b/c built on the host from
// column (0,0) (:38-65); cp/dp scratch is per thread in local memory.
__global__ void k_rhevi_column(Dims d, const double* __restrict__ ta, const double* __restrict__ tb,
                               const double* __restrict__ tc, double* __restrict__ pi, double* __restrict__ scratch,
                               unsigned* err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= d.nx || j >= d.ny) return;
  const int nz = d.nz;
  const size_t col = (size_t)j * d.nx + i;
  double* cp = scratch + col * 2 * nz;
  double* dp = cp + nz;
  if (nz == 1) { pi[d.idx(i, j, 0)] = pi[d.idx(i, j, 0)] / tb[0]; return; }
  double denom = tb[0];
  cp[0] = tc[0] / denom;
  dp[0] = pi[d.idx(i, j, 0)] / denom;
  for (int k = 1; k < nz; ++k) {
    denom = tb[k] - ta[k - 1] * cp[k - 1];
    if (fabs(denom) < 1e-300) { atomicOr(err, (unsigned)kErrSingular); return; }
    dp[k] = (pi[d.idx(i, j, k)] - ta[k - 1] * dp[k - 1]) / denom;
    if (k < nz - 1) cp[k] = tc[k] / denom;
  }
  double x = dp[nz - 1];
  pi[d.idx(i, j, nz - 1)] = x;
  for (int k = nz - 1; k-- > 0;) {
    x = dp[k] - cp[k] * x;
    pi[d.idx(i, j, k)] = x;
  }
}
// update_momentum (:96-124)
__global__ void k_rhevi_mom(Dims d, Metric m, CS s, double* __restrict__ u, double* __restrict__ v,
                            double* __restrict__ w, double dtau) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i > d.nx || j > d.ny || k > d.nz) return;
  const size_t c = IDX(i, j, k);
  if (j < d.ny && k < d.nz) {
    const int ip = imin(i, d.nx - 1), im = imax(i - 1, 0);
    const double t0 = 0.5 * (R3(m.th0, d, im, j, k) + R3(m.th0, d, ip, j, k));
    u[c] -= dtau * kCp * t0 * (SF(PI, ip, j, k) - SF(PI, im, j, k)) / m.dx;
  }
  if (i < d.nx && k < d.nz) {
    const int jp = imin(j, d.ny - 1), jm = imax(j - 1, 0);
    const double t0 = 0.5 * (R3(m.th0, d, i, jm, k) + R3(m.th0, d, i, jp, k));
    v[c] -= dtau * kCp * t0 * (SF(PI, i, jp, k) - SF(PI, i, jm, k)) / m.dy;
  }
  if (i < d.nx && j < d.ny) {
    const int kc = imin(imax(k, 0), d.nz - 1), km = imax(k - 1, 0);
    const double dz = dmax(dzeta(m, d, kc) * scale_at(m, d, i, j), 1.0);
    const double t0 = 0.5 * (R3(m.th0, d, i, j, km) + R3(m.th0, d, i, j, kc));
    w[c] -= dtau * kCp * t0 * (SF(PI, i, j, kc) - SF(PI, i, j, km)) / dz;
  }
}

// ---- consistent vertically implicit substep (FP64). With weight b, rho0
// and theta0 face averages r_f, t_f and spacings dzf as the explicit operator:
//   w~ = w - dtau (1-b) cp t_f G(pi'),  G on interior faces, 0 on k = 0, nz
//   pi* = pi + dtau kappa (Dh + (1-b) Dv(w) + b Dv(w~))
//   (1 + c_k (T_k + T_k+1)) x_k - c_k T_k x_k-1 - c_k T_k+1 x_k+1 = pi* - P0
//     c_k = (dtau b)^2 kappa_k / dz_k, T_f = r_f cp t_f / dzf_f, x = new pi'
//   w_new = w~ - dtau b cp t_f G(x), rho += dtau (Dh + (1-b) Dv(w) + b Dv(w_new))
// One thread per column; horizontal momentum afterwards (k_uv_backward).
// Scratch is level-major (row r, level k of column col at
// ((r*(nz+1) + k)*ncol + col)), so a warp's 32 columns touch one contiguous
// run per access: rows cp, dp, Dh, w~, w_new and, in the fast build, the
// reciprocal spacings 1/dz of the column (dzf(k) = dzc(min(k, nz-1)), so one
// row serves both).
__global__ void k_chevi_column(Dims d, Metric m, Flags fl, CS s, double* __restrict__ w_out,
                               double* __restrict__ rho_out, double* __restrict__ pi_out,
                               double* __restrict__ scratch, double dtau, unsigned* err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= d.nx || j >= d.ny) return;
  const int nz = d.nz, nx = d.nx, ny = d.ny;
  const double b = fl.hevi_beta, ob = 1.0 - b;
  const int pert = fl.pgf_pert;
  const size_t ncol = (size_t)nx * ny, col = (size_t)j * nx + i;
  auto S = [&](int r, int k) -> double& { return scratch[((size_t)r * (nz + 1) + k) * ncol + col]; };
  enum { CP = 0, DP, DH, WT, WN, IDZ };
  const double sc = m.scale[col];
  auto rf = [&](int k) { return 0.5 * (R3(m.rho0, d, i, j, imax(k - 1, 0)) + R3(m.rho0, d, i, j, imin(k, nz - 1))); };
  auto tf = [&](int k) { return 0.5 * (R3(m.th0, d, i, j, imax(k - 1, 0)) + R3(m.th0, d, i, j, imin(k, nz - 1))); };
  auto dzc = [&](int k) { return dmax(m.dzeta[k] * sc, 1.0); };
  auto dzf = [&](int k) { return dzc(imin(k, nz - 1)); };
#ifndef VGB_FP64_EXACT
  for (int k = 0; k < nz; ++k) S(IDZ, k) = 1.0 / dzc(k);
#endif
  auto idzc = [&](int k) { return S(IDZ, k); };
  auto idzf = [&](int k) { return S(IDZ, imin(k, nz - 1)); };
  auto pp = [&](int k) { return SF(PI, i, j, k) - (pert ? R3(m.pi0, d, i, j, k) : 0.0); };
  for (int k = 0; k <= nz; ++k) {
    double G = 0.0;
    if (k > 0 && k < nz) G = DIVR(pp(k) - pp(k - 1), dzf(k), idzf(k));
    S(WT, k) = SF(W, i, j, k) - dtau * ob * kCp * tf(k) * G;
  }
  // forward elimination (Thomas, helmholtz.cpp:71-83 recurrence)
  double cprev = 0.0, dprev = 0.0;
  for (int k = 0; k < nz; ++k) {
    const double r0 = R3(m.rho0, d, i, j, k);
    const double kap = (kRd / kCv) * (R3(m.pi0, d, i, j, k) / dmax(r0, 1e-8));
    const double fx = SF(U, i + 1, j, k) * 0.5 * (r0 + R3(m.rho0, d, imin(i + 1, nx - 1), j, k)) -
                      SF(U, i, j, k) * 0.5 * (R3(m.rho0, d, imax(i - 1, 0), j, k) + r0);
    const double fy = SF(V, i, j + 1, k) * 0.5 * (r0 + R3(m.rho0, d, i, imin(j + 1, ny - 1), k)) -
                      SF(V, i, j, k) * 0.5 * (R3(m.rho0, d, i, imax(j - 1, 0), k) + r0);
    const double dh = -(DIVR(fx, m.dx, m.inv_dx) + DIVR(fy, m.dy, m.inv_dy));
    S(DH, k) = dh;
    const double rk = rf(k), rk1 = rf(k + 1);
    const double dv_old = DIVR(-(rk1 * SF(W, i, j, k + 1) - rk * SF(W, i, j, k)), dzc(k), idzc(k));
    const double dv_t = DIVR(-(rk1 * S(WT, k + 1) - rk * S(WT, k)), dzc(k), idzc(k));
    const double pstar = SF(PI, i, j, k) + dtau * kap * (dh + ob * dv_old + b * dv_t);
    const double ck = DIVR((dtau * b) * (dtau * b) * kap, dzc(k), idzc(k));
    const double Tk = (k == 0) ? 0.0 : DIVR(rk * kCp * tf(k), dzf(k), idzf(k));
    const double Tk1 = (k + 1 == nz) ? 0.0 : DIVR(rk1 * kCp * tf(k + 1), dzf(k + 1), idzf(k + 1));
    const double a = -ck * Tk, c = -ck * Tk1, bb = 1.0 + ck * (Tk + Tk1);
    const double rhs = pstar - (pert ? R3(m.pi0, d, i, j, k) : 0.0);
    const double denom = (k == 0) ? bb : bb - a * cprev;
    if (fabs(denom) < 1e-300) { atomicOr(err, (unsigned)kErrSingular); return; }
#ifdef VGB_FP64_EXACT
    dprev = (k == 0) ? rhs / denom : (rhs - a * dprev) / denom;
    cprev = (k < nz - 1) ? c / denom : 0.0;
#else
    const double rden = 1.0 / denom;
    dprev = (k == 0) ? rhs * rden : (rhs - a * dprev) * rden;
    cprev = (k < nz - 1) ? c * rden : 0.0;
#endif
    S(CP, k) = cprev;
    S(DP, k) = dprev;
  }
  // back substitution; x_k = pi'_new
  double xk1 = S(DP, nz - 1);
  for (int k = nz - 1; k-- > 0;) {
    xk1 = S(DP, k) - S(CP, k) * xk1;
    S(DP, k) = xk1;
  }
  for (int k = 0; k <= nz; ++k) {
    double g = 0.0;
    if (k > 0 && k < nz) g = DIVR(S(DP, k) - S(DP, k - 1), dzf(k), idzf(k));
    S(WN, k) = S(WT, k) - dtau * b * kCp * tf(k) * g;
  }
  for (int k = 0; k < nz; ++k) {
    const double rk = rf(k), rk1 = rf(k + 1);
    const double dv_old = DIVR(-(rk1 * SF(W, i, j, k + 1) - rk * SF(W, i, j, k)), dzc(k), idzc(k));
    const double dv_new = DIVR(-(rk1 * S(WN, k + 1) - rk * S(WN, k)), dzc(k), idzc(k));
    const size_t c = IDX(i, j, k);
    rho_out[c] = SF(RHO, i, j, k) + dtau * (S(DH, k) + ob * dv_old + b * dv_new);
    pi_out[c] = S(DP, k) + (pert ? R3(m.pi0, d, i, j, k) : 0.0);
  }
  for (int k = 0; k <= nz; ++k) w_out[IDX(i, j, k)] = S(WN, k);
}

__global__ void k_uv_backward(Dims d, Metric m, Flags fl, CS s, double* __restrict__ u, double* __restrict__ v,
                              double dtau) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i > d.nx || j > d.ny || k >= d.nz) return;
  const size_t c = IDX(i, j, k);
  if (j < d.ny) u[c] += dtau * ac_u(s, m, d, fl, i, j, k);
  if (i < d.nx) v[c] += dtau * ac_v(s, m, d, fl, i, j, k);
}

// ---- Damping::apply_sponge, damping.cpp:76-140 ----------------------------
__global__ void k_sponge(Dims d, Metric m, MS s, int kmin, double dt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = kmin + blockIdx.z;
  if (i > d.nx || j > d.ny || k > d.nz) return;
  const double a = m.sponge[imin(k, d.nz - 1)];
  if (a <= 0.0) return;
  const double wgt = 1.0 / (1.0 + dt * a);
  const size_t c = d.idx(i, j, k);
  if (j < d.ny && k < d.nz) s.f[U][c] = wgt * s.f[U][c];
  if (i < d.nx && k < d.nz) s.f[V][c] = wgt * s.f[V][c];
  if (i < d.nx && j < d.ny) s.f[W][c] = wgt * s.f[W][c];
  if (i < d.nx && j < d.ny && k < d.nz) {
    s.f[RHO][c] = wgt * (s.f[RHO][c] + dt * a * m.rho0[c]);
    s.f[THETA][c] = wgt * (s.f[THETA][c] + dt * a * m.th0[c]);
    s.f[PI][c] = wgt * (s.f[PI][c] + dt * a * m.pi0[c]);
  }
}

// State::has_nonfinite over the interior and faces of every species.
__global__ void k_nonfinite(Dims d, CS s, unsigned* err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i > d.nx || j > d.ny || k > d.nz) return;
  const size_t c = d.idx(i, j, k);
  bool bad = false;
  const bool cell = i < d.nx && j < d.ny && k < d.nz;
  if (j < d.ny && k < d.nz) bad |= !isfinite(s.f[U][c]);
  if (i < d.nx && k < d.nz) bad |= !isfinite(s.f[V][c]);
  if (i < d.nx && j < d.ny) bad |= !isfinite(s.f[W][c]);
  if (cell)
    for (int q = RHO; q < NSPECIES; ++q) bad |= !isfinite(s.f[q][c]);
  if (bad) atomicOr(err, (unsigned)kErrNonFinite);
}

// ---- adjoint of the explicit forward-backward substep ---------------------
// The substep (runge_kutta.cpp:65-75 with Equations::acoustic_tendencies,
// equations.cpp:152-209) is linear in (u, v, w, rho, pi) with coefficients
// from the reference state when the gradient is taken of pi itself: phase 1
// adds dtau D(u,v,w) to rho and dtau kappa D to pi (D = mass_div0, kappa =
// (Rd/cv) pi0/max(rho0, 1e-8)); phase 2 adds dtau G(pi) to u, v, w (ac_u,
// ac_v, ac_w). Its tangent-linear is the substep itself on the perturbation;
// its adjoint runs the transposed phases in reverse, each as a gather:
//   bar_pi(c) += dtau sum_faces a_f (+1 if c is the face's upper point, -1 if
//                its lower point) bar_vel(f),   a_f = -cp theta0_f / h_f
//   bar_vel(f) += dtau sum_cells dD(c)/dvel(f) (bar_rho(c) + kappa(c) bar_pi(c))
__device__ inline double ac_coef_u(const Metric& m, const Dims& d, int i, int j, int k) {
  const int ip = imin(i, d.nx - 1), im = imax(i - 1, 0);
  return -kCp * (0.5 * (R3(m.th0, d, im, j, k) + R3(m.th0, d, ip, j, k))) / m.dx;
}
__device__ inline double ac_coef_v(const Metric& m, const Dims& d, int i, int j, int k) {
  const int jp = imin(j, d.ny - 1), jm = imax(j - 1, 0);
  return -kCp * (0.5 * (R3(m.th0, d, i, jm, k) + R3(m.th0, d, i, jp, k))) / m.dy;
}
__device__ inline double ac_coef_w(const Metric& m, const Dims& d, int i, int j, int k) {
  const int kc = imin(imax(k, 0), d.nz - 1), km = imax(k - 1, 0);
  const double dz = dmax(dzeta(m, d, kc) * scale_at(m, d, i, j), 1.0);
  return -kCp * (0.5 * (R3(m.th0, d, i, j, km) + R3(m.th0, d, i, j, kc))) / dz;
}

// phase 2 transposed: cells
__global__ void k_fbad_pi(Dims d, Metric m, const double* __restrict__ bu, const double* __restrict__ bv,
                          const double* __restrict__ bw, double* __restrict__ bpi, double dtau, int with_w) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= d.nx || j >= d.ny || k >= d.nz) return;
  double acc = 0.0;
  // x faces f with ip(f) == i: f = i, and f = nx when i = nx-1; with im(f) == i: f = i+1, and f = 0 when i = 0
  acc += ac_coef_u(m, d, i, j, k) * bu[IDX(i, j, k)];
  if (i == d.nx - 1) acc += ac_coef_u(m, d, d.nx, j, k) * bu[IDX(d.nx, j, k)];
  acc -= ac_coef_u(m, d, i + 1, j, k) * bu[IDX(i + 1, j, k)];
  if (i == 0) acc -= ac_coef_u(m, d, 0, j, k) * bu[IDX(0, j, k)];
  acc += ac_coef_v(m, d, i, j, k) * bv[IDX(i, j, k)];
  if (j == d.ny - 1) acc += ac_coef_v(m, d, i, d.ny, k) * bv[IDX(i, d.ny, k)];
  acc -= ac_coef_v(m, d, i, j + 1, k) * bv[IDX(i, j + 1, k)];
  if (j == 0) acc -= ac_coef_v(m, d, i, 0, k) * bv[IDX(i, 0, k)];
  if (with_w) {
    acc += ac_coef_w(m, d, i, j, k) * bw[IDX(i, j, k)];
    if (k == d.nz - 1) acc += ac_coef_w(m, d, i, j, d.nz) * bw[IDX(i, j, d.nz)];
    acc -= ac_coef_w(m, d, i, j, k + 1) * bw[IDX(i, j, k + 1)];
    if (k == 0) acc -= ac_coef_w(m, d, i, j, 0) * bw[IDX(i, j, 0)];
  }
  bpi[IDX(i, j, k)] += dtau * acc;
}

// phase 1 transposed: faces
__global__ void k_fbad_vel(Dims d, Metric m, const double* __restrict__ brho, const double* __restrict__ bpi,
                           double* __restrict__ bu, double* __restrict__ bv, double* __restrict__ bw, double dtau) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i > d.nx || j > d.ny || k > d.nz) return;
  const double* r0 = m.rho0;
  auto Z = [&](int ci, int cj, int ck) {
    const size_t c = IDX(ci, cj, ck);
    return brho[c] + (kRd / kCv) * (m.pi0[c] / dmax(m.rho0[c], 1e-8)) * bpi[c];
  };
  if (j < d.ny && k < d.nz) {  // u face i: east face of cell i-1, west face of cell i
    double acc = 0.0;
    if (i >= 1) {
      const int c = i - 1;
      acc -= 0.5 * (R3(r0, d, c, j, k) + R3(r0, d, imin(c + 1, d.nx - 1), j, k)) / m.dx * Z(c, j, k);
    }
    if (i < d.nx) acc += 0.5 * (R3(r0, d, imax(i - 1, 0), j, k) + R3(r0, d, i, j, k)) / m.dx * Z(i, j, k);
    bu[IDX(i, j, k)] += dtau * acc;
  }
  if (i < d.nx && k < d.nz) {  // v face j
    double acc = 0.0;
    if (j >= 1) {
      const int c = j - 1;
      acc -= 0.5 * (R3(r0, d, i, c, k) + R3(r0, d, i, imin(c + 1, d.ny - 1), k)) / m.dy * Z(i, c, k);
    }
    if (j < d.ny) acc += 0.5 * (R3(r0, d, i, imax(j - 1, 0), k) + R3(r0, d, i, j, k)) / m.dy * Z(i, j, k);
    bv[IDX(i, j, k)] += dtau * acc;
  }
  if (i < d.nx && j < d.ny) {  // w face k: top face of cell k-1, bottom face of cell k
    double acc = 0.0;
    if (k >= 1) {
      const int c = k - 1;
      const double dz = dmax(dzeta(m, d, c) * scale_at(m, d, i, j), 1.0);
      acc -= 0.5 * (R3(r0, d, i, j, c) + R3(r0, d, i, j, imin(c + 1, d.nz - 1))) / dz * Z(i, j, c);
    }
    if (k < d.nz) {
      const double dz = dmax(dzeta(m, d, k) * scale_at(m, d, i, j), 1.0);
      acc += 0.5 * (R3(r0, d, i, j, imax(k - 1, 0)) + R3(r0, d, i, j, k)) / dz * Z(i, j, k);
    }
    bw[IDX(i, j, k)] += dtau * acc;
  }
}


// ---- adjoint of the consistent HEVI substep (k_chevi_column + k_uv_backward)
// With the gradient taken of pi itself (pgf_perturbation = 0) the substep is
// linear in (u, v, w, rho, pi): wt = w - dtau (1-b) cp theta0_f d(pi)/dz on
// interior faces; per cell pstar = pi + dtau kappa (Dh + (1-b) dv(w) + b dv(wt))
// and the column system A x = pstar (A from the reference state only);
// wn = wt - dtau b cp theta0_f dx/dz; rho += dtau (Dh + (1-b) dv(w) + b dv(wn));
// pi = x; w = wn; then u, v take the horizontal gradient of the new pi. The
// adjoint runs these in reverse: the horizontal gradient transposed (cells
// gather from their faces, k_fbad_pi without w), one thread per column for the
// vertical part (the column system transposed: A^T y = bar_x by the Thomas
// recurrence on the swapped off-diagonals), and the horizontal divergence
// Dh transposed (faces gather from their two cells).
__global__ void k_hevi_ad_column(Dims d, Metric m, Flags fl, double* __restrict__ bw, const double* __restrict__ brho,
                                 double* __restrict__ bpi, double* __restrict__ bdh, double* __restrict__ scratch,
                                 double dtau, unsigned* err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= d.nx || j >= d.ny) return;
  const int nz = d.nz;
  const double b = fl.hevi_beta, ob = 1.0 - b;
  const size_t col = (size_t)j * d.nx + i;
  double* ya = scratch + col * (5 * (size_t)nz + 2);  // nz: bar_x, then y
  double* cpr = ya + nz;                              // nz: Thomas c'
  double* bwn = cpr + nz;                             // nz+1: bar_wn, then bar_wt
  double* dvo = bwn + nz + 1;                         // nz: bar_dv_old
  const double sc = m.scale[col];
  auto rf = [&](int k) { return 0.5 * (R3(m.rho0, d, i, j, imax(k - 1, 0)) + R3(m.rho0, d, i, j, imin(k, nz - 1))); };
  auto tf = [&](int k) { return 0.5 * (R3(m.th0, d, i, j, imax(k - 1, 0)) + R3(m.th0, d, i, j, imin(k, nz - 1))); };
  auto dzf = [&](int k) { return dmax(m.dzeta[imin(k, nz - 1)] * sc, 1.0); };
  auto dzc = [&](int k) { return dmax(m.dzeta[k] * sc, 1.0); };
  auto kap = [&](int k) { return (kRd / kCv) * (R3(m.pi0, d, i, j, k) / dmax(R3(m.rho0, d, i, j, k), 1e-8)); };
  // the column matrix of k_chevi_column: row k = (a_k, bb_k, c_k)
  auto row = [&](int k, double& a, double& bb, double& c) {
    const double ck = (dtau * b) * (dtau * b) * kap(k) / dzc(k);
    const double Tk = (k == 0) ? 0.0 : rf(k) * kCp * tf(k) / dzf(k);
    const double Tk1 = (k + 1 == nz) ? 0.0 : rf(k + 1) * kCp * tf(k + 1) / dzf(k + 1);
    a = -ck * Tk;
    c = -ck * Tk1;
    bb = 1.0 + ck * (Tk + Tk1);
  };
  // rho = rho + dtau (Dh + ob dv_old + b dv_new): bar_dv_new = dtau b bar_rho
  // wn feeds dv_new of the cells below and above each face, and w_out
  for (int k = 0; k <= nz; ++k) {
    double g = bw[IDX(i, j, k)];
    if (k < nz) g += rf(k) / dzc(k) * (dtau * b * brho[IDX(i, j, k)]);
    if (k >= 1) g -= rf(k) / dzc(k - 1) * (dtau * b * brho[IDX(i, j, k - 1)]);
    bwn[k] = g;
  }
  // wn = wt - cb_k (x_k - x_{k-1}) on interior faces; x = pi_out
  for (int k = 0; k < nz; ++k) ya[k] = bpi[IDX(i, j, k)];
  for (int k = 1; k < nz; ++k) {
    const double cb = dtau * b * kCp * tf(k) / dzf(k);
    ya[k] -= cb * bwn[k];
    ya[k - 1] += cb * bwn[k];
  }
  // A^T y = bar_x: row k of A^T has (c_{k-1}, bb_k, a_{k+1})
  double yprev = 0.0, cprev = 0.0;
  for (int k = 0; k < nz; ++k) {
    double a, bb, c, a1 = 0.0, bb1, c1;
    row(k, a, bb, c);
    double cm = 0.0;
    if (k > 0) {
      double a0, bb0, c0;
      row(k - 1, a0, bb0, c0);
      cm = c0;  // A^T sub-diagonal
    }
    if (k + 1 < nz) row(k + 1, a1, bb1, c1);
    const double denom = (k == 0) ? bb : bb - cm * cprev;
    if (fabs(denom) < 1e-300) { atomicOr(err, (unsigned)kErrSingular); return; }
    yprev = (k == 0) ? ya[k] / denom : (ya[k] - cm * yprev) / denom;
    cprev = (k + 1 < nz) ? a1 / denom : 0.0;
    cpr[k] = cprev;
    ya[k] = yprev;
  }
  for (int k = nz - 1; k-- > 0;) ya[k] -= cpr[k] * ya[k + 1];
  // pstar = pi + dtau kappa (Dh + ob dv_old + b dv_t)
  for (int k = 0; k < nz; ++k) {
    const double y = ya[k], kp = dtau * kap(k) * y;
    bdh[IDX(i, j, k)] = dtau * brho[IDX(i, j, k)] + kp;
    dvo[k] = dtau * ob * brho[IDX(i, j, k)] + ob * kp;
    cpr[k] = b * kp;  // bar_dv_t
  }
  // bar_wt: from wn (identity) and dv_t
  for (int k = 0; k <= nz; ++k) {
    double g = bwn[k];
    if (k < nz) g += rf(k) / dzc(k) * cpr[k];
    if (k >= 1) g -= rf(k) / dzc(k - 1) * cpr[k - 1];
    bwn[k] = g;
  }
  // bar_w: from wt (identity) and dv_old
  for (int k = 0; k <= nz; ++k) {
    double g = bwn[k];
    if (k < nz) g += rf(k) / dzc(k) * dvo[k];
    if (k >= 1) g -= rf(k) / dzc(k - 1) * dvo[k - 1];
    bw[IDX(i, j, k)] = g;
  }
  // bar_pi of the input: pstar's pi (y) and wt's gradient, wt(k) = w - ce_k (pi_k - pi_{k-1});
  // the output pi is x itself, whose bar went into y
  for (int k = 0; k < nz; ++k) {
    double g = ya[k];
    if (k >= 1) g -= dtau * ob * kCp * tf(k) / dzf(k) * bwn[k];
    if (k + 1 < nz) g += dtau * ob * kCp * tf(k + 1) / dzf(k + 1) * bwn[k + 1];
    bpi[IDX(i, j, k)] = g;
  }
}

// The forward substep copies the column solve's whole w, rho, pi outputs back,
// whose ghost column i = nx and ghost row j = ny it never writes (zeros): those
// outputs do not depend on the input, so their bars do not reach it
__global__ void k_hevi_ad_ghost(Dims d, double* __restrict__ bw, double* __restrict__ brho, double* __restrict__ bpi) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i > d.nx || j > d.ny || k > d.nz || (i < d.nx && j < d.ny)) return;
  const size_t c = IDX(i, j, k);
  bw[c] = 0.0;
  if (k < d.nz) {
    brho[c] = 0.0;
    bpi[c] = 0.0;
  }
}

// Dh = -(fx/dx + fy/dy) transposed: each u / v face gathers from its two cells
__global__ void k_dh_ad(Dims d, Metric m, const double* __restrict__ bdh, double* __restrict__ bu,
                        double* __restrict__ bv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i > d.nx || j > d.ny || k >= d.nz) return;
  const double* r0 = m.rho0;
  if (j < d.ny) {
    double acc = 0.0;
    if (i >= 1) {
      const int c = i - 1;
      acc -= 0.5 * (R3(r0, d, c, j, k) + R3(r0, d, imin(c + 1, d.nx - 1), j, k)) / m.dx * bdh[IDX(c, j, k)];
    }
    if (i < d.nx) acc += 0.5 * (R3(r0, d, imax(i - 1, 0), j, k) + R3(r0, d, i, j, k)) / m.dx * bdh[IDX(i, j, k)];
    bu[IDX(i, j, k)] += acc;
  }
  if (i < d.nx) {
    double acc = 0.0;
    if (j >= 1) {
      const int c = j - 1;
      acc -= 0.5 * (R3(r0, d, i, c, k) + R3(r0, d, i, imin(c + 1, d.ny - 1), k)) / m.dy * bdh[IDX(i, c, k)];
    }
    if (j < d.ny) acc += 0.5 * (R3(r0, d, i, imax(j - 1, 0), k) + R3(r0, d, i, j, k)) / m.dy * bdh[IDX(i, j, k)];
    bv[IDX(i, j, k)] += acc;
  }
}
}  // namespace

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
static dim3 grid3(const Dims& d, int ni, int nj, int nk, dim3 blk) {
  return dim3((ni + blk.x - 1) / blk.x, (nj + blk.y - 1) / blk.y, nk);
}
static const dim3 kBlk(32, 4, 1);

static CS to_cs(double* const* f) {
  CS s;
  for (int q = 0; q < NSPECIES; ++q) s.f[q] = f[q];
  return s;
}
static MS to_ms(double* const* f) {
  MS s;
  for (int q = 0; q < NSPECIES; ++q) s.f[q] = f[q];
  return s;
}

void FP64_FN(fp64_slow_tendency)(const Dims& d, const Metric& m, const Flags& fl, double* const* st, double* const* tend,
                        double* lap_scratch, double* face_scratch, cudaStream_t stream) {
  const CS s = to_cs(st);
  k_tend_u<<<grid3(d, d.nx + 1, d.ny, d.nz, kBlk), kBlk, 0, stream>>>(d, m, fl, s, tend[U]);
  k_tend_v<<<grid3(d, d.nx, d.ny + 1, d.nz, kBlk), kBlk, 0, stream>>>(d, m, fl, s, tend[V]);
  k_tend_w<<<grid3(d, d.nx, d.ny, d.nz + 1, kBlk), kBlk, 0, stream>>>(d, m, fl, s, tend[W]);
  const double* lapf = nullptr;
  if (fl.div_damp > 0.0 && fl.div_order > 2) {
    k_lap<<<grid3(d, d.nx, d.ny, d.nz, kBlk), kBlk, 0, stream>>>(d, m, st[PI], lap_scratch);
    lapf = lap_scratch;
  }
  k_tend_cells<<<grid3(d, d.nx, d.ny, d.nz, kBlk), kBlk, 0, stream>>>(d, m, fl, s, to_ms(tend), lapf);
  if (fl.weno_scalars) {
    const size_t nf = d.plane * (size_t)(d.nz + 1);
    double* fx = face_scratch;
    double* fy = fx + nf;
    double* fz = fy + nf;
    const int last = fl.moist ? QG : QV;
    for (int q = THETA; q <= last; ++q) {
      if (q == PI) continue;
      k_weno_faces<<<grid3(d, d.nx + 1, d.ny + 1, d.nz + 1, kBlk), kBlk, 0, stream>>>(d, s, q, fx, fy, fz);
      k_weno_cells<<<grid3(d, d.nx, d.ny, d.nz, kBlk), kBlk, 0, stream>>>(d, m, fl, s, q, fx, fy, fz, tend[q]);
    }
  }
}

void FP64_FN(fp64_stage_update)(const Dims& d, double* const* s0, double* const* tend, double a, double* const* out,
                       cudaStream_t stream) {
  for (int q = 0; q < NSPECIES; ++q) {
    const int ni = d.nx + (q == U), nj = d.ny + (q == V), nk = d.nz + (q == W);
    k_axpy_field<<<grid3(d, ni, nj, nk, kBlk), kBlk, 0, stream>>>(d, ni, nj, nk, s0[q], tend[q], a, out[q]);
  }
}

void FP64_FN(fp64_fb_substep_ad)(const Dims& d, const Metric& m, double* const* bar, double dtau, cudaStream_t stream) {
  k_fbad_pi<<<grid3(d, d.nx, d.ny, d.nz, kBlk), kBlk, 0, stream>>>(d, m, bar[U], bar[V], bar[W], bar[PI], dtau, 1);
  k_fbad_vel<<<grid3(d, d.nx + 1, d.ny + 1, d.nz + 1, kBlk), kBlk, 0, stream>>>(d, m, bar[RHO], bar[PI], bar[U], bar[V],
                                                                               bar[W], dtau);
}

void FP64_FN(fp64_hevi_substep_ad)(const Dims& d, const Metric& m, const Flags& fl, double* const* bar, double* bdh,
                                   double* scratch, double dtau, unsigned* err, cudaStream_t stream) {
  k_fbad_pi<<<grid3(d, d.nx, d.ny, d.nz, kBlk), kBlk, 0, stream>>>(d, m, bar[U], bar[V], bar[W], bar[PI], dtau, 0);
  k_hevi_ad_column<<<dim3((d.nx + 31) / 32, (d.ny + 3) / 4), dim3(32, 4), 0, stream>>>(d, m, fl, bar[W], bar[RHO],
                                                                                      bar[PI], bdh, scratch, dtau,
                                                                                      err);
  k_dh_ad<<<grid3(d, d.nx + 1, d.ny + 1, d.nz, kBlk), kBlk, 0, stream>>>(d, m, bdh, bar[U], bar[V]);
  k_hevi_ad_ghost<<<grid3(d, d.nx + 1, d.ny + 1, d.nz + 1, kBlk), kBlk, 0, stream>>>(d, bar[W], bar[RHO], bar[PI]);
}

void FP64_FN(fp64_fb_substep)(const Dims& d, const Metric& m, const Flags& fl, double* const* st, double dtau,
                     cudaStream_t stream) {
  const CS s = to_cs(st);
  k_fb_mass<<<grid3(d, d.nx, d.ny, d.nz, kBlk), kBlk, 0, stream>>>(d, m, s, st[RHO], st[PI], dtau);
  k_fb_mom<<<grid3(d, d.nx + 1, d.ny + 1, d.nz + 1, kBlk), kBlk, 0, stream>>>(d, m, fl, s, st[U], st[V], st[W], dtau);
}

void FP64_FN(fp64_ref_hevi_substep)(const Dims& d, const Metric& m, double* const* st, double dtau, const double* ta,
                           const double* tb, const double* tc, double* scratch, unsigned* err, cudaStream_t stream) {
  const CS s = to_cs(st);
  double* drho = scratch;
  double* colscr = scratch + d.plane * d.nz;
  k_rhevi_mass<<<grid3(d, d.nx, d.ny, d.nz, kBlk), kBlk, 0, stream>>>(d, m, s, drho);
  k_rhevi_apply<<<grid3(d, d.nx, d.ny, d.nz, kBlk), kBlk, 0, stream>>>(d, m, drho, st[RHO], st[PI], dtau);
  const dim3 b2(32, 4);
  k_rhevi_column<<<dim3((d.nx + 31) / 32, (d.ny + 3) / 4), b2, 0, stream>>>(d, ta, tb, tc, st[PI], colscr, err);
  k_rhevi_mom<<<grid3(d, d.nx + 1, d.ny + 1, d.nz + 1, kBlk), kBlk, 0, stream>>>(d, m, s, st[U], st[V], st[W], dtau);
}

void FP64_FN(fp64_cons_hevi_substep)(const Dims& d, const Metric& m, const Flags& fl, double* const* st, double* const* tmp,
                            double* scratch, double dtau, unsigned* err, cudaStream_t stream) {
  // column solve reads the old state, writes w/rho/pi into tmp, copied back
  const CS s = to_cs(st);
  const dim3 b2(32, 4);
  k_chevi_column<<<dim3((d.nx + 31) / 32, (d.ny + 3) / 4), b2, 0, stream>>>(d, m, fl, s, tmp[W], tmp[RHO], tmp[PI],
                                                                             scratch, dtau, err);
  const size_t n_w = d.plane * (d.nz + 1), n_c = d.plane * d.nz;
  cudaMemcpyAsync(st[W], tmp[W], n_w * sizeof(double), cudaMemcpyDeviceToDevice, stream);
  cudaMemcpyAsync(st[RHO], tmp[RHO], n_c * sizeof(double), cudaMemcpyDeviceToDevice, stream);
  cudaMemcpyAsync(st[PI], tmp[PI], n_c * sizeof(double), cudaMemcpyDeviceToDevice, stream);
  k_uv_backward<<<grid3(d, d.nx + 1, d.ny + 1, d.nz, kBlk), kBlk, 0, stream>>>(d, m, fl, s, st[U], st[V], dtau);
}

void FP64_FN(fp64_sponge)(const Dims& d, const Metric& m, double* const* st, int kmin, double dt, cudaStream_t stream) {
  if (kmin > d.nz) return;
  k_sponge<<<grid3(d, d.nx + 1, d.ny + 1, d.nz + 1 - kmin, kBlk), kBlk, 0, stream>>>(d, m, to_ms(st), kmin, dt);
}

void FP64_FN(fp64_nonfinite)(const Dims& d, double* const* st, unsigned* err, cudaStream_t stream) {
  k_nonfinite<<<grid3(d, d.nx + 1, d.ny + 1, d.nz + 1, kBlk), kBlk, 0, stream>>>(d, to_cs(st), err);
}

}  // namespace vgb
