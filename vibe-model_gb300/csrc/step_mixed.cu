// vibe-model_gb300/csrc/step_mixed.cu
//
// Mixed-precision dynamics step: the state is FP64 in HBM; tendencies,
// reconstructions and the acoustic substeps are computed in FP32 from an
// FP32 working copy held in perturbation form (u, v, w, rho' = rho - rho0,
// theta' = theta - theta0, pi' = pi - pi0, q); FP64 is used only where the
// state is updated (s = s0 + dt*R per stage, and the acoustic increment of
// each stage folded back into the FP64 state) and for the sponge.
//
// Why: on GB300 every FP64 instruction, including an f64<->f32 conversion,
// issues at ~2 per clock per SM against 128 FP32 FMAs; an FP64 update per
// substep would make the step FP64-issue bound. Working in perturbation
// form keeps FP32 free of the cancellation a total Exner function or
// potential temperature would suffer (|pi'| ~ 1e-4 of pi).
//
// Requires a horizontally uniform reference state on flat terrain (all
// coefficients are per-level tables) and the stable composition
// (pi' pressure gradient, fast terms integrated once by the substeps).
#include "step_kernels.cuh"

namespace vgb {
namespace {

struct CS64 {
  const double* __restrict__ f[NSPECIES];
};
struct MS64 {
  double* __restrict__ f[NSPECIES];
};

#define IX(i, j, k) (d.idx((i), (j), (k)))
#define WI(q, i, j, k) (win.f[q][IX(i, j, k)])
#define WC(q, i, j, k) (win.f[q][IX(iclamp((i), 0, d.nx - 1), iclamp((j), 0, d.ny - 1), iclamp((k), 0, d.nz - 1))])

// WENO5 face reconstruction + local Lax-Friedrichs flux in FP32
// (advection.cpp:62-98,151-156), with the weights normalised by a single
// division: a_k = d_k / s_k^2 -> numerator and denominator scaled by
// (s0 s1 s2)^2.
__device__ __forceinline__ float weno_face_f(float qm2, float qm1, float q0, float q1, float q2, float vel) {
  const float eps = 1e-6f;
  const float v0 = (2.f * qm2 - 7.f * qm1 + 11.f * q0) * (1.f / 6.f);
  const float v1 = (-qm1 + 5.f * q0 + 2.f * q1) * (1.f / 6.f);
  const float v2 = (2.f * q0 + 5.f * q1 - q2) * (1.f / 6.f);
  const float e0 = qm2 - 2.f * qm1 + q0, f0 = qm2 - 4.f * qm1 + 3.f * q0;
  const float e1 = qm1 - 2.f * q0 + q1, f1 = qm1 - q1;
  const float e2 = q0 - 2.f * q1 + q2, f2 = 3.f * q0 - 4.f * q1 + q2;
  const float s0 = eps + (13.f / 12.f) * (e0 * e0) + 0.25f * (f0 * f0);
  const float s1 = eps + (13.f / 12.f) * (e1 * e1) + 0.25f * (f1 * f1);
  const float s2 = eps + (13.f / 12.f) * (e2 * e2) + 0.25f * (f2 * f2);
  const float p01 = s0 * s1, p02 = s0 * s2, p12 = s1 * s2;
  const float w0 = 0.1f * (p12 * p12), w1 = 0.6f * (p02 * p02), w2 = 0.3f * (p01 * p01);
  const float ql = (w0 * v0 + w1 * v1 + w2 * v2) / (w0 + w1 + w2);
  const float u0 = (2.f * q2 - 7.f * q1 + 11.f * q0) * (1.f / 6.f);
  const float u1 = (-q1 + 5.f * q0 + 2.f * qm1) * (1.f / 6.f);
  const float u2 = (2.f * q0 + 5.f * qm1 - qm2) * (1.f / 6.f);
  const float g0e = q2 - 2.f * q1 + q0, g0f = q2 - 4.f * q1 + 3.f * q0;
  const float g1e = q1 - 2.f * q0 + qm1, g1f = q1 - qm1;
  const float g2e = q0 - 2.f * qm1 + qm2, g2f = 3.f * q0 - 4.f * qm1 + qm2;
  const float t0 = eps + (13.f / 12.f) * (g0e * g0e) + 0.25f * (g0f * g0f);
  const float t1 = eps + (13.f / 12.f) * (g1e * g1e) + 0.25f * (g1f * g1f);
  const float t2 = eps + (13.f / 12.f) * (g2e * g2e) + 0.25f * (g2f * g2f);
  const float r01 = t0 * t1, r02 = t0 * t2, r12 = t1 * t2;
  const float c0 = 0.1f * (r12 * r12), c1 = 0.6f * (r02 * r02), c2 = 0.3f * (r01 * r01);
  const float qr = (c0 * u0 + c1 * u1 + c2 * u2) / (c0 + c1 + c2);
  const float alpha = fmaxr(fabsf(vel), 1e-3f);
  return 0.5f * (vel * (ql + qr) - alpha * (qr - ql));
}

__device__ __forceinline__ float gradc(float m3, float m2, float m1, float p1, float p2, float p3, float inv, int order) {
  switch (order) {
    case 4: return (m2 - 8.f * m1 + 8.f * p1 - p2) * (inv * (1.f / 12.f));
    case 6: return (-m3 + 9.f * m2 - 45.f * m1 + 45.f * p1 - 9.f * p2 + p3) * (inv * (1.f / 60.f));
    default: return (p1 - m1) * (0.5f * inv);
  }
}

// scalar tendency of species q at cell (i,j,k); shift_theta: q is theta'
__device__ float scalar_tend(const Dims& d, const Tab& t, const Flags& fl, const WS& win, int q, int i, int j, int k,
                             bool is_theta) {
  const float qc = WI(q, i, j, k);
  const float* sh = t.t0d + 6 * k;  // theta0(clamp(k+m)) - theta0(k), m=-3..2
  auto zq = [&](int m) {          // vertical stencil value shifted by theta0(k)
    const float v = WC(q, i, j, k + m);
    return is_theta ? v + sh[m + 3] : v;
  };
  const float u_w = WI(U, i, j, k), u_e = WI(U, i + 1, j, k);
  const float v_s = WI(V, i, j, k), v_n = WI(V, i, j + 1, k);
  const float w_b = WI(W, i, j, k), w_t = WI(W, i, j, k + 1);
  const float idz = t.idza[k];
  if (fl.weno_scalars) {
    const float xm3 = WC(q, i - 3, j, k), xm2 = WC(q, i - 2, j, k), xm1 = WC(q, i - 1, j, k);
    const float xp1 = WC(q, i + 1, j, k), xp2 = WC(q, i + 2, j, k);
    const float ym3 = WC(q, i, j - 3, k), ym2 = WC(q, i, j - 2, k), ym1 = WC(q, i, j - 1, k);
    const float yp1 = WC(q, i, j + 1, k), yp2 = WC(q, i, j + 2, k);
    const float fe = weno_face_f(xm2, xm1, qc, xp1, xp2, u_e);
    const float fw = weno_face_f(xm3, xm2, xm1, qc, xp1, u_w);
    const float fn = weno_face_f(ym2, ym1, qc, yp1, yp2, v_n);
    const float fs = weno_face_f(ym3, ym2, ym1, qc, yp1, v_s);
    float ft = 0.f, fb = 0.f;
    const bool vert = (k + 2 < d.nz || k >= 2);
    const float zc = is_theta ? qc : qc;  // shift is 0 at m = 0
    if (vert) {
      const float zm3 = zq(-3), zm2 = zq(-2), zm1 = zq(-1), zp1 = zq(1), zp2 = zq(2);
      ft = weno_face_f(zm2, zm1, zc, zp1, zp2, w_t);
      fb = weno_face_f(zm3, zm2, zm1, zc, zp1, w_b);
    }
    float r = -(fe - fw) * t.dx_inv - (fn - fs) * t.dy_inv - (ft - fb) * idz;
    float div = (u_e - u_w) * t.dx_inv + (v_n - v_s) * t.dy_inv;
    if (vert) div += (w_t - w_b) * idz;
    // flux form of (q'+c): -dF(q')/dx - c*div; advective form adds (q'+c)*div
    if (fl.weno_advective) r += qc * div;
    else if (is_theta) r -= t.t0c[k] * div;
    return r;
  }
  const float ua = 0.5f * (u_w + u_e), va = 0.5f * (v_s + v_n), wa = 0.5f * (w_b + w_t);
  const float gx = gradc(WC(q, i - 3, j, k), WC(q, i - 2, j, k), WC(q, i - 1, j, k), WC(q, i + 1, j, k),
                         WC(q, i + 2, j, k), WC(q, i + 3, j, k), t.dx_inv, fl.advection);
  const float gy = gradc(WC(q, i, j - 3, k), WC(q, i, j - 2, k), WC(q, i, j - 1, k), WC(q, i, j + 1, k),
                         WC(q, i, j + 2, k), WC(q, i, j + 3, k), t.dy_inv, fl.advection);
  const float gz = (zq(1) - zq(-1)) * (0.5f * idz);
  return -(ua * gx + va * gy + wa * gz);
}

template <bool kFP64Out>
__global__ void __launch_bounds__(128) k_mx_stage(Dims d, Tab t, Flags fl, WS win, WS w0, WS wout, CS64 s0, MS64 ss,
                                                  float dts, double dtd, unsigned* err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i > d.nx || j > d.ny || k > d.nz) return;
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const size_t c = IX(i, j, k);
  bool bad = false;
  auto emit = [&](int q, float r) {
    const float o = (w0.f[q] != nullptr) ? w0.f[q][c] + dts * r : r;  // no base: raw tendency
    wout.f[q][c] = o;
    bad |= !isfinite(o);
    if (kFP64Out) ss.f[q][c] = s0.f[q][c] + dtd * (double)r;
  };
  const float cp = (float)kCp;
  if (j < ny && k < nz) {  // u face
    const int ip = imin(i, nx - 1), im = imax(i - 1, 0);
    const int jp1 = imin(j + 1, ny - 1), jm1 = imax(j - 1, 0);
    const float uc = 0.5f * (WI(U, im, j, k) + WI(U, ip, j, k));
    const float ux = (WI(U, ip, j, k) - WI(U, im, j, k)) * t.dx_inv;
    const float uy = (WI(U, ip, jp1, k) - WI(U, ip, jm1, k)) * (0.5f * t.dy_inv);
    const float uz = (WI(U, ip, j, imin(k + 1, nz - 1)) - WI(U, ip, j, imax(k - 1, 0))) * (0.5f * t.idza[k]);
    const float vc = 0.25f * (WI(V, im, jm1, k) + WI(V, ip, jm1, k) + WI(V, im, j, k) + WI(V, ip, j, k));
    const float wc = 0.5f * (WI(W, ip, j, k) + WI(W, ip, j, imin(k + 1, nz - 1)));
    float r = -(uc * ux + vc * uy + wc * uz);
    if (fl.coriolis) r += (fl.coriolis == 2 ? t.f0 + t.beta * (((float)j + 0.5f) * t.dy - 0.5f * (float)ny * t.dy) : t.f0) * vc;
    r -= cp * (0.5f * (WI(THETA, im, j, k) + WI(THETA, ip, j, k))) * (WI(PI, ip, j, k) - WI(PI, im, j, k)) * t.dx_inv;
    emit(U, r);
  }
  if (i < nx && k < nz) {  // v face
    const int jp = imin(j, ny - 1), jm = imax(j - 1, 0);
    const int ip1 = imin(i + 1, nx - 1), im1 = imax(i - 1, 0);
    const float vc = 0.5f * (WI(V, i, jm, k) + WI(V, i, jp, k));
    const float vy = (WI(V, i, jp, k) - WI(V, i, jm, k)) * t.dy_inv;
    const float vx = (WI(V, ip1, jp, k) - WI(V, im1, jp, k)) * (0.5f * t.dx_inv);
    const float vz = (WI(V, i, jp, imin(k + 1, nz - 1)) - WI(V, i, jp, imax(k - 1, 0))) * (0.5f * t.idza[k]);
    const float uc = 0.25f * (WI(U, im1, jm, k) + WI(U, i, jm, k) + WI(U, im1, jp, k) + WI(U, i, jp, k));
    const float wc = 0.5f * (WI(W, i, jp, k) + WI(W, i, jp, imin(k + 1, nz - 1)));
    float r = -(uc * vx + vc * vy + wc * vz);
    if (fl.coriolis) r -= (fl.coriolis == 2 ? t.f0 + t.beta * (((float)j + 0.5f) * t.dy - 0.5f * (float)ny * t.dy) : t.f0) * uc;
    r -= cp * (0.5f * (WI(THETA, i, jm, k) + WI(THETA, i, jp, k))) * (WI(PI, i, jp, k) - WI(PI, i, jm, k)) * t.dy_inv;
    emit(V, r);
  }
  if (i < nx && j < ny) {  // w face
    const int kc = imin(k, nz - 1), km = imax(k - 1, 0);
    const int ip1 = imin(i + 1, nx - 1), im1 = imax(i - 1, 0);
    const int jp1 = imin(j + 1, ny - 1), jm1 = imax(j - 1, 0);
    const float wc = 0.5f * (WI(W, i, j, kc) + WI(W, i, j, k));
    const float wz = (WI(W, i, j, k) - WI(W, i, j, km)) * t.idza[kc];
    const float wx = (WI(W, ip1, j, k) - WI(W, im1, j, k)) * (0.5f * t.dx_inv);
    const float wy = (WI(W, i, jp1, k) - WI(W, i, jm1, k)) * (0.5f * t.dy_inv);
    const float uc = 0.5f * (WI(U, i, j, kc) + WI(U, i + 1, j, kc));
    const float vc = 0.5f * (WI(V, i, j, kc) + WI(V, i, j + 1, kc));
    float r = -(uc * wx + vc * wy + wc * wz);
    r -= cp * (0.5f * (WI(THETA, i, j, km) + WI(THETA, i, j, kc))) * (WI(PI, i, j, kc) - WI(PI, i, j, km)) * t.idzw[k];
    float qcond = 0.f;
    if (fl.moist) qcond = WI(QC, i, j, kc) + WI(QR, i, j, kc) + WI(QI, i, j, kc) + WI(QS, i, j, kc) + WI(QG, i, j, kc);
    r += (float)kG * (WI(THETA, i, j, kc) * t.th0inv[kc] + (float)kBuoyMoist * WI(QV, i, j, kc) - qcond);
    emit(W, r);
  }
  if (i < nx && j < ny && k < nz) {  // cells
    {
      const float rc = WI(RHO, i, j, k);
      const float fx = WI(U, i + 1, j, k) * 0.5f * (rc + WI(RHO, i + 1, j, k)) -
                       WI(U, i, j, k) * 0.5f * (WI(RHO, imax(i - 1, 0), j, k) + rc);
      const float fy = WI(V, i, j + 1, k) * 0.5f * (rc + WI(RHO, i, j + 1, k)) -
                       WI(V, i, j, k) * 0.5f * (WI(RHO, i, imax(j - 1, 0), k) + rc);
      const float fz = WI(W, i, j, k + 1) * 0.5f * (rc + WI(RHO, i, j, imin(k + 1, nz - 1))) -
                       WI(W, i, j, k) * 0.5f * (WI(RHO, i, j, imax(k - 1, 0)) + rc);
      emit(RHO, -(fx * t.dx_inv + fy * t.dy_inv + fz * t.idzc[k]));
    }
    {
      float r = 0.f;
      if (fl.div_damp > 0.0) {
        const float pc = WI(PI, i, j, k);
        const float lap = (WC(PI, i + 1, j, k) - 2.f * pc + WC(PI, i - 1, j, k)) * (t.dx_inv * t.dx_inv) +
                          (WC(PI, i, j + 1, k) - 2.f * pc + WC(PI, i, j - 1, k)) * (t.dy_inv * t.dy_inv);
        r = -(float)fl.div_damp * lap;
      }
      emit(PI, r);
    }
    // inactive moisture species (moist off) keep their values in every
    // buffer: zero tendency, so they are neither read nor rewritten here
    const int last = fl.moist ? QG : QV;
    for (int q = THETA; q <= last; ++q) {
      if (q == PI) continue;
      float r = scalar_tend(d, t, fl, win, q, i, j, k, q == THETA);
      if (q >= QV && WI(q, i, j, k) <= 0.f && r < 0.f) r = 0.f;
      emit(q, r);
    }
  }
  if (bad) atomicOr(err, (unsigned)kErrNonFinite);
}

// ---- explicit forward-backward substep in FP32 (runge_kutta.cpp:65-75) --
__global__ void k_mx_fb_mass(Dims d, Tab t, WS win, WS wout, float dtau) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= d.nx || j >= d.ny || k >= d.nz) return;
  const size_t c = IX(i, j, k);
  const float r0 = t.r0c[k];
  const float drho = -(r0 * ((WI(U, i + 1, j, k) - WI(U, i, j, k)) * t.dx_inv +
                             (WI(V, i, j + 1, k) - WI(V, i, j, k)) * t.dy_inv) +
                       (WI(W, i, j, k + 1) * t.rfz[k + 1] - WI(W, i, j, k) * t.rfz[k]) * t.idzc[k]);
  wout.f[RHO][c] = win.f[RHO][c] + dtau * drho;
  wout.f[PI][c] = win.f[PI][c] + dtau * (t.kap[k] * drho);
}
// momentum backward with the new pi' (read from wout)
__global__ void k_mx_fb_mom(Dims d, Tab t, WS win, WS wout, float dtau, int do_w) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i > d.nx || j > d.ny || k > d.nz) return;
  const size_t c = IX(i, j, k);
  const float* __restrict__ pn = wout.f[PI];
  const float cp = (float)kCp;
  if (j < d.ny && k < d.nz) {
    const int ip = imin(i, d.nx - 1), im = imax(i - 1, 0);
    wout.f[U][c] = win.f[U][c] + dtau * (-cp * t.t0c[k] * (pn[IX(ip, j, k)] - pn[IX(im, j, k)]) * t.dx_inv);
  }
  if (i < d.nx && k < d.nz) {
    const int jp = imin(j, d.ny - 1), jm = imax(j - 1, 0);
    wout.f[V][c] = win.f[V][c] + dtau * (-cp * t.t0c[k] * (pn[IX(i, jp, k)] - pn[IX(i, jm, k)]) * t.dy_inv);
  }
  if (do_w && i < d.nx && j < d.ny) {
    const int kc = imin(k, d.nz - 1), km = imax(k - 1, 0);
    wout.f[W][c] = win.f[W][c] + dtau * (-cp * t.tfz[k] * (pn[IX(i, j, kc)] - pn[IX(i, j, km)]) * t.idzw[k]);
  }
}

// ---- consistent vertically implicit substep in FP32 ---------------------
// One thread per column; the LU factors of the (column-independent)
// tridiagonal matrix come in lu = [a(k), c'(k), 1/den(k)] x nz.
// Per-thread scratch in shared memory: dp, S = Dh + (1-b) Dv_old, wt.
__global__ void k_mx_hevi_col(Dims d, Tab t, Flags fl, WS win, WS wout, float dtau, const float* __restrict__ lu) {
  extern __shared__ float sm[];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int nz = d.nz;
  const int tid = threadIdx.y * blockDim.x + threadIdx.x, nt = blockDim.x * blockDim.y;
  float* s_dp = sm;                   // nz * nt
  float* s_S = sm + (size_t)nz * nt;  // nz * nt
  float* s_wt = s_S + (size_t)nz * nt; // (nz+1) * nt
  if (i >= d.nx || j >= d.ny) return;
  const float b = (float)fl.hevi_beta, ob = 1.f - b;
  const float cp = (float)kCp;
  const float* __restrict__ la = lu;
  const float* __restrict__ lc = lu + nz;
  const float* __restrict__ li = lu + 2 * nz;
  // explicit part of w at face k: wt = w - dtau*(1-b)*cp*tf*G(pi'_old)
  float p_k = WI(PI, i, j, 0);
  float wt_k = WI(W, i, j, 0);  // face 0: no pressure gradient
  s_wt[tid] = wt_k;
  float w_k = wt_k;
  float dp_prev = 0.f;
  for (int k = 0; k < nz; ++k) {
    const float w_k1 = WI(W, i, j, k + 1);
    float wt_k1 = w_k1, p_k1 = 0.f;
    if (k + 1 < nz) {
      p_k1 = WI(PI, i, j, k + 1);
      wt_k1 = w_k1 - dtau * ob * cp * t.tfz[k + 1] * (p_k1 - p_k) * t.idzw[k + 1];
    }
    s_wt[(size_t)(k + 1) * nt + tid] = wt_k1;
    const float r0 = t.r0c[k];
    const float Dh = -(r0 * ((WI(U, i + 1, j, k) - WI(U, i, j, k)) * t.dx_inv + (WI(V, i, j + 1, k) - WI(V, i, j, k)) * t.dy_inv));
    const float rk = t.rfz[k], rk1 = t.rfz[k + 1];
    const float dv_old = -(rk1 * w_k1 - rk * w_k) * t.idzc[k];
    const float dv_t = -(rk1 * wt_k1 - rk * wt_k) * t.idzc[k];
    const float S = Dh + ob * dv_old;
    const float rhs = p_k + dtau * t.kap[k] * (S + b * dv_t);
    const float dpk = (k == 0) ? rhs * li[0] : (rhs - la[k] * dp_prev) * li[k];
    s_dp[(size_t)k * nt + tid] = dpk;
    s_S[(size_t)k * nt + tid] = S;
    dp_prev = dpk;
    w_k = w_k1;
    wt_k = wt_k1;
    p_k = p_k1;
  }
  // back substitution with a one-level lag: x(k) = pi'_new(k);
  // wn(k+1) needs x(k), x(k+1); rho'(k+1) needs wn(k+2), wn(k+1).
  float x_up = s_dp[(size_t)(nz - 1) * nt + tid];  // x(nz-1)
  float wn_up = s_wt[(size_t)nz * nt + tid];       // wn(nz) = wt(nz)
  wout.f[W][IX(i, j, nz)] = wn_up;
  for (int k = nz - 2; k >= -1; --k) {
    // x(k) (k >= 0), then finalise level k+1
    float x_k = 0.f, wn_k1;
    if (k >= 0) {
      x_k = s_dp[(size_t)k * nt + tid] - lc[k] * x_up;
      wn_k1 = s_wt[(size_t)(k + 1) * nt + tid] - dtau * b * cp * t.tfz[k + 1] * (x_up - x_k) * t.idzw[k + 1];
    } else {
      wn_k1 = s_wt[tid];  // face 0
    }
    const int kk = k + 1;  // finalise cell kk with faces kk, kk+1
    const float dv_new = -(t.rfz[kk + 1] * wn_up - t.rfz[kk] * wn_k1) * t.idzc[kk];
    const size_t ck = IX(i, j, kk);
    wout.f[RHO][ck] = win.f[RHO][ck] + dtau * (s_S[(size_t)kk * nt + tid] + b * dv_new);
    wout.f[PI][ck] = x_up;
    wout.f[W][ck] = wn_k1;
    x_up = x_k;
    wn_up = wn_k1;
  }
}

// ---- finish: fold the last stage's acoustic increments into the FP64
// state, apply the sponge (damping.cpp:76-140) in FP64 and to the FP32
// working copy, which becomes the next step's s0 working copy.
__global__ void k_mx_finish(Dims d, Tab t, Flags fl, WS wfin, WS wst, WS w0, MS64 ss, unsigned* err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i > d.nx || j > d.ny || k > d.nz) return;
  const size_t c = IX(i, j, k);
  const int kc = imin(k, d.nz - 1);
  const double wd = t.spwd[k];
  const float wf = t.spw[k];
  bool bad = false;
  auto face = [&](int q) {
    const double v = wd * (ss.f[q][c] + (double)(wfin.f[q][c] - wst.f[q][c]));
    ss.f[q][c] = v;
    w0.f[q][c] = wf * wfin.f[q][c];
    bad |= !isfinite(v);
  };
  if (j < d.ny && k < d.nz) face(U);
  if (i < d.nx && k < d.nz) face(V);
  if (i < d.nx && j < d.ny) face(W);
  if (i < d.nx && j < d.ny && k < d.nz) {
    const double sdt = t.spdt[k];
    {
      const double v = wd * ((ss.f[RHO][c] + (double)(wfin.f[RHO][c] - wst.f[RHO][c])) + sdt * t.r0d[kc]);
      ss.f[RHO][c] = v;
      w0.f[RHO][c] = wf * wfin.f[RHO][c];
      bad |= !isfinite(v);
    }
    {
      const double v = wd * ((ss.f[PI][c] + (double)(wfin.f[PI][c] - wst.f[PI][c])) + sdt * t.p0d[kc]);
      ss.f[PI][c] = v;
      w0.f[PI][c] = wf * wfin.f[PI][c];
      bad |= !isfinite(v);
    }
    if (wd != 1.0) ss.f[THETA][c] = wd * (ss.f[THETA][c] + sdt * t.t0dd[kc]);
    w0.f[THETA][c] = wf * wst.f[THETA][c];
    bad |= !isfinite(ss.f[THETA][c]);
    const int last = fl.moist ? QG : QV;
    for (int q = QV; q <= last; ++q) {
      w0.f[q][c] = wst.f[q][c];
      bad |= !isfinite(ss.f[q][c]);
    }
  }
  if (bad) atomicOr(err, (unsigned)kErrNonFinite);
}

// FP32 field (device layout) -> FP64 FieldT storage (zeros outside the box)
__global__ void k_mx_unpack_f32(Dims d, int nsx, int nsy, int nsz, int ni, int nj, int nk, const float* __restrict__ src,
                                double* __restrict__ dst) {
  const size_t n = (size_t)nsx * nsy * nsz;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const int ii = (int)(e % nsx) - 4, jj = (int)((e / nsx) % nsy) - 4, kk = (int)(e / ((size_t)nsx * nsy)) - 4;
    double v = 0.0;
    if (ii >= 0 && ii < ni && jj >= 0 && jj < nj && kk >= 0 && kk < nk) v = (double)src[d.idx(ii, jj, kk)];
    dst[e] = v;
  }
}

// FP64 state -> FP32 working copy in perturbation form, incl. ghosts.
__global__ void k_mx_to_working(Dims d, Tab t, CS64 s, WS w) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i > d.nx || j > d.ny || k > d.nz) return;
  const size_t c = IX(i, j, k);
  if (j < d.ny && k < d.nz) w.f[U][c] = (float)s.f[U][c];
  if (i < d.nx && k < d.nz) w.f[V][c] = (float)s.f[V][c];
  if (i < d.nx && j < d.ny) w.f[W][c] = (float)s.f[W][c];
  if (k < d.nz) {  // cells incl. the ghost column/row
    w.f[RHO][c] = (float)(s.f[RHO][c] - t.r0d[k]);
    w.f[THETA][c] = (float)(s.f[THETA][c] - t.t0dd[k]);
    w.f[PI][c] = (float)(s.f[PI][c] - t.p0d[k]);
    for (int q = QV; q < NSPECIES; ++q) w.f[q][c] = (float)s.f[q][c];
  }
}

}  // namespace

static dim3 g3(int ni, int nj, int nk, dim3 b) { return dim3((ni + b.x - 1) / b.x, (nj + b.y - 1) / b.y, nk); }

static CS64 cs64(double* const* f) {
  CS64 s;
  for (int q = 0; q < NSPECIES; ++q) s.f[q] = f ? f[q] : nullptr;
  return s;
}
static MS64 ms64(double* const* f) {
  MS64 s;
  for (int q = 0; q < NSPECIES; ++q) s.f[q] = f ? f[q] : nullptr;
  return s;
}

void mixed_stage(const Dims& d, const Tab& t, const Flags& fl, const WS& win, const WS& w0, const WS& wout,
                 double* const* s0, double* const* ss, double dt_stage, bool write_fp64, unsigned* err,
                 cudaStream_t stream) {
  const dim3 b(32, 4);
  const dim3 g = g3(d.nx + 1, d.ny + 1, d.nz + 1, b);
  if (write_fp64)
    k_mx_stage<true><<<g, b, 0, stream>>>(d, t, fl, win, w0, wout, cs64(s0), ms64(ss), (float)dt_stage, dt_stage, err);
  else
    k_mx_stage<false><<<g, b, 0, stream>>>(d, t, fl, win, w0, wout, cs64(nullptr), ms64(nullptr), (float)dt_stage,
                                           dt_stage, err);
}

void mixed_fb_substep(const Dims& d, const Tab& t, const Flags& fl, const WS& win, const WS& wout, float dtau,
                      cudaStream_t stream) {
  const dim3 b(32, 4);
  k_mx_fb_mass<<<g3(d.nx, d.ny, d.nz, b), b, 0, stream>>>(d, t, win, wout, dtau);
  k_mx_fb_mom<<<g3(d.nx + 1, d.ny + 1, d.nz + 1, b), b, 0, stream>>>(d, t, win, wout, dtau, 1);
}

void mixed_hevi_column(const Dims& d, const Tab& t, const Flags& fl, const WS& win, const WS& wout, float dtau,
                       const float* lu, cudaStream_t stream) {
  const dim3 bc(32, 2);
  const size_t smem = (size_t)(3 * d.nz + 1) * bc.x * bc.y * sizeof(float);
  static size_t smem_set = 0;  // opt in above 48 KB once per size
  if (smem > 48 * 1024 && smem > smem_set) {
    cudaFuncSetAttribute(k_mx_hevi_col, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    smem_set = smem;
  }
  k_mx_hevi_col<<<dim3((d.nx + bc.x - 1) / bc.x, (d.ny + bc.y - 1) / bc.y), bc, smem, stream>>>(d, t, fl, win, wout,
                                                                                               dtau, lu);
}

void mixed_uv_backward(const Dims& d, const Tab& t, const WS& win, const WS& wout, float dtau, cudaStream_t stream) {
  const dim3 b(32, 4);
  k_mx_fb_mom<<<g3(d.nx + 1, d.ny + 1, d.nz, b), b, 0, stream>>>(d, t, win, wout, dtau, 0);
}

void mixed_hevi_substep(const Dims& d, const Tab& t, const Flags& fl, const WS& win, const WS& wout, float dtau,
                        const float* lu, unsigned* err, cudaStream_t stream) {
  (void)err;
  mixed_hevi_column(d, t, fl, win, wout, dtau, lu, stream);
  mixed_uv_backward(d, t, win, wout, dtau, stream);
}

void mixed_finish(const Dims& d, const Tab& t, const Flags& fl, const WS& wfin, const WS& wst, const WS& w0,
                  double* const* ss, double dt, int kmin, unsigned* err, cudaStream_t stream) {
  (void)dt; (void)kmin;
  const dim3 b(32, 4);
  k_mx_finish<<<g3(d.nx + 1, d.ny + 1, d.nz + 1, b), b, 0, stream>>>(d, t, fl, wfin, wst, w0, ms64(ss), err);
}

void mixed_unpack_f32(const Dims& d, int nsx, int nsy, int nsz, int ni, int nj, int nk, const float* src, double* dst,
                      cudaStream_t stream) {
  k_mx_unpack_f32<<<1024, 256, 0, stream>>>(d, nsx, nsy, nsz, ni, nj, nk, src, dst);
}

void mixed_to_working(const Dims& d, const Tab& t, double* const* s, const WS& w, cudaStream_t stream) {
  const dim3 b(32, 4);
  k_mx_to_working<<<g3(d.nx + 1, d.ny + 1, d.nz + 1, b), b, 0, stream>>>(d, t, cs64(s), w);
}

}  // namespace vgb
