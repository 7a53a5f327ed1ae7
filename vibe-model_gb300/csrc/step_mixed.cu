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
#include <cmath>
#include <cstdlib>
#include <map>
#include <mutex>
#include <tuple>

#include <cuda.h>
#include <cudaTypedefs.h>
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
// (advection.cpp:62-98,151-156), organised for FP32 throughput; the
// arithmetic is the reference's up to rounding:
//  * the right-biased reconstruction of (qm2..q2) is the left-biased one of
//    the reversed stencil (q2..qm2), whose smoothness indicators are the same
//    three values in reverse order -- they are computed once;
//  * with alpha = max(|vel|, 1e-3) the flux 0.5*(vel*(ql+qr) - alpha*(qr-ql))
//    is vel*ql for vel >= 1e-3 and vel*qr for vel <= -1e-3, so one
//    reconstruction on the upwind-ordered stencil suffices there; only lanes
//    with |vel| < 1e-3 evaluate the second one;
//  * the weights a_k = d_k/s_k^2 are normalised with one division:
//    numerator and denominator scaled by (s0 s1 s2)^2, all terms positive
//    and far inside the FP32 range (s_k in [1e-6, ~1e4]).
__device__ __forceinline__ float weno_left(float qm2, float qm1, float q0, float q1, float q2, float s0, float s1,
                                           float s2) {
  const float v0 = (2.f * qm2 - 7.f * qm1 + 11.f * q0) * (1.f / 6.f);
  const float v1 = (-qm1 + 5.f * q0 + 2.f * q1) * (1.f / 6.f);
  const float v2 = (2.f * q0 + 5.f * q1 - q2) * (1.f / 6.f);
  const float p01 = s0 * s1, p02 = s0 * s2, p12 = s1 * s2;
  const float w0 = 0.1f * (p12 * p12), w1 = 0.6f * (p02 * p02), w2 = 0.3f * (p01 * p01);
  return __fdividef(w0 * v0 + w1 * v1 + w2 * v2, w0 + w1 + w2);
}
__device__ __forceinline__ float weno_face_f(float qm2, float qm1, float q0, float q1, float q2, float vel) {
  const float eps = 1e-6f;
  const float e0 = qm2 - 2.f * qm1 + q0, f0 = qm2 - 4.f * qm1 + 3.f * q0;
  const float e1 = qm1 - 2.f * q0 + q1, f1 = qm1 - q1;
  const float e2 = q0 - 2.f * q1 + q2, f2 = 3.f * q0 - 4.f * q1 + q2;
  const float s0 = eps + (13.f / 12.f) * (e0 * e0) + 0.25f * (f0 * f0);
  const float s1 = eps + (13.f / 12.f) * (e1 * e1) + 0.25f * (f1 * f1);
  const float s2 = eps + (13.f / 12.f) * (e2 * e2) + 0.25f * (f2 * f2);
  const bool up = vel >= 0.f;  // upwind-ordered stencil (no divergence)
  const float a0 = up ? qm2 : q2, a1 = up ? qm1 : q1, a3 = up ? q1 : qm1, a4 = up ? q2 : qm2;
  const float t0 = up ? s0 : s2, t2 = up ? s2 : s0;
  const float rec = weno_left(a0, a1, q0, a3, a4, t0, s1, t2);
  if (fabsf(vel) >= 1e-3f) return vel * rec;
  const float oth = weno_left(a4, a3, q0, a1, a0, t2, s1, t0);  // the other side
  const float ql = up ? rec : oth, qr = up ? oth : rec;
  return 0.5f * (vel * (ql + qr) - 1e-3f * (qr - ql));
}

// ---- theta' and qv side by side: packed FP32 pairs ----
// The stage kernel reconstructs theta' and qv at the same faces with the
// same velocity, so their WENO5 arithmetic runs on f32x2 pairs (low:
// theta', high: qv): one add/mul/fma.rn.f32x2 does both species' operation,
// each lane IEEE-rounded as the scalar instruction would be.
struct F2 {
  unsigned long long r;
};
__device__ __forceinline__ F2 mk2(float a, float b) {
  F2 o;
  asm("mov.b64 %0, {%1, %2};" : "=l"(o.r) : "f"(a), "f"(b));
  return o;
}
__device__ __forceinline__ F2 dup2(float a) { return mk2(a, a); }
__device__ __forceinline__ void un2(F2 x, float& a, float& b) { asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(x.r)); }
__device__ __forceinline__ F2 add2(F2 a, F2 b) {
  F2 o;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(o.r) : "l"(a.r), "l"(b.r));
  return o;
}
__device__ __forceinline__ F2 sub2(F2 a, F2 b) {
  F2 o;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(o.r) : "l"(a.r), "l"(b.r));
  return o;
}
__device__ __forceinline__ F2 mul2(F2 a, F2 b) {
  F2 o;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(o.r) : "l"(a.r), "l"(b.r));
  return o;
}
__device__ __forceinline__ F2 fma2(F2 a, F2 b, F2 c) {
  F2 o;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(o.r) : "l"(a.r), "l"(b.r), "l"(c.r));
  return o;
}
__device__ __forceinline__ F2 sel2(bool p, F2 a, F2 b) { return p ? a : b; }

// WENO5 left-biased reconstruction of the stencil a0..a4 (centre a2) with
// smoothness indicators s0..s2, as weno_left; the candidates are formed at
// 6x and the 1/6 folded into the normalisation
__device__ __forceinline__ F2 weno_left2(F2 a0, F2 a1, F2 a2, F2 a3, F2 a4, F2 s0, F2 s1, F2 s2) {
  const F2 V0 = fma2(dup2(11.f), a2, fma2(dup2(-7.f), a1, add2(a0, a0)));
  const F2 V1 = fma2(dup2(5.f), a2, sub2(add2(a3, a3), a1));
  const F2 V2 = sub2(fma2(dup2(5.f), a3, add2(a2, a2)), a4);
  const F2 p01 = mul2(s0, s1), p02 = mul2(s0, s2), p12 = mul2(s1, s2);
  const F2 w0 = mul2(dup2(0.1f), mul2(p12, p12)), w1 = mul2(dup2(0.6f), mul2(p02, p02));
  const F2 w2 = mul2(dup2(0.3f), mul2(p01, p01));
  const F2 num = fma2(w2, V2, fma2(w1, V1, mul2(w0, V0)));
  float d0, d1;
  un2(mul2(dup2(6.f), add2(add2(w0, w1), w2)), d0, d1);
  float i0, i1;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(i0) : "f"(d0));
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(i1) : "f"(d1));
  return mul2(num, mk2(i0, i1));
}
// WENO5 face flux of a pair (local Lax-Friedrichs, as weno_face_f) from the
// stencil in upwind order: qm2 qm1 q0 q1 q2 for vel >= 0, its mirror image
// q2 q1 q0 qm1 qm2 for vel < 0 (centre q0 either way). The smoothness
// indicators of the mirrored stencil are the original ones in reverse
// order, so the caller's choice of load addresses replaces the selects.
__device__ __forceinline__ F2 weno_flux2(F2 a0, F2 a1, F2 a2, F2 a3, F2 a4, float vel) {
  const F2 eps = dup2(1e-6f), c1312 = dup2(13.f / 12.f), q25 = dup2(0.25f), m2 = dup2(-2.f), m4 = dup2(-4.f),
           c3 = dup2(3.f);
  const F2 e0 = add2(fma2(m2, a1, a0), a2), f0 = fma2(c3, a2, fma2(m4, a1, a0));
  const F2 e1 = add2(fma2(m2, a2, a1), a3), f1 = sub2(a1, a3);
  const F2 e2 = add2(fma2(m2, a3, a2), a4), f2 = fma2(m4, a3, fma2(c3, a2, a4));
  const F2 s0 = fma2(q25, mul2(f0, f0), fma2(c1312, mul2(e0, e0), eps));
  const F2 s1 = fma2(q25, mul2(f1, f1), fma2(c1312, mul2(e1, e1), eps));
  const F2 s2 = fma2(q25, mul2(f2, f2), fma2(c1312, mul2(e2, e2), eps));
  const F2 rec = weno_left2(a0, a1, a2, a3, a4, s0, s1, s2);
  if (fabsf(vel) >= 1e-3f) return mul2(dup2(vel), rec);
  const F2 oth = weno_left2(a4, a3, a2, a1, a0, s2, s1, s0);  // the other side
  const bool up = vel >= 0.f;
  const F2 ql = sel2(up, rec, oth), qr = sel2(up, oth, rec);
  return mul2(dup2(0.5f), sub2(mul2(dup2(vel), add2(ql, qr)), mul2(dup2(1e-3f), sub2(qr, ql))));
}
// the pair's flux through a vertical face from the column's values
// qm2..q2 in bottom-to-top order (the face between q0 and q1)
__device__ __forceinline__ F2 weno_vflux2(F2 qm2, F2 qm1, F2 q0, F2 q1, F2 q2, float vel) {
  const bool up = vel >= 0.f;
  return weno_flux2(sel2(up, qm2, q2), sel2(up, qm1, q1), q0, sel2(up, q1, qm1), sel2(up, q2, qm2), vel);
}

__device__ __forceinline__ float gradc(float m3, float m2, float m1, float p1, float p2, float p3, float inv, int order) {
  switch (order) {
    case 4: return (m2 - 8.f * m1 + 8.f * p1 - p2) * (inv * (1.f / 12.f));
    case 6: return (-m3 + 9.f * m2 - 45.f * m1 + 45.f * p1 - 9.f * p2 + p3) * (inv * (1.f / 60.f));
    default: return (p1 - m1) * (0.5f * inv);
  }
}

// ---- RK stage kernel: slow tendency + s = s0 + dt*R ------------------------
// 2.5-D: a block owns 32 x 8 columns and marches up a chunk of levels
// (grid z = chunk). Each level's planes of theta', qv, u, v, w, pi', rho' are
// brought into shared memory by TMA (cp.async.bulk.tensor, one box per field
// with the halo its stencils need: 3 rows for the scalar WENO / high-order
// stencils, 1 row for the others; every box is 40 columns wide starting 4
// columns left of the block, keeping the TMA x coordinate 16-byte aligned),
// double-buffered: the next level's boxes are in flight, tracked by an
// mbarrier, while the current level computes. Elements outside a field's
// index range arrive as zeros; blocks at the domain edge then overwrite them
// with the reference's clamped values (clamp_at, field.hpp:91-96), so a tile
// read at an unclamped offset returns the clamped value. The level boxes
// form a ring of three slots: while level k is computed, the boxes of level
// k+1 are resident too (the u, v, w, rho' values one level up that the
// vertical differences and the vertical mass flux need come from there) and
// those of level k+2 are in flight. Each thread keeps its own column's
// vertical neighbours in registers: theta' and qv over k-3..k+3 for the
// vertical WENO, whose flux through the top face of level k is carried to
// level k+1 as its bottom flux (one WENO evaluation per vertical face), and
// u, v, w, pi', rho' at k-1. Horizontal WENO fluxes are computed once per
// face into shared memory. When the stage's base state is its input (the
// first stage) the base values are read from the boxes too.
// kSpec: the composition the bench times (WENO5 scalars in advective form,
// dry, no Coriolis, no divergence damping) compiled with those flags fixed.
constexpr int TX = 32, TY = 8;
constexpr int NT = TX * TY;
constexpr int TW = 40;                   // box width (floats), all fields
constexpr int XO = 4;                    // local column of global i0
constexpr int R3 = TY + 6, R1 = TY + 2;  // box rows: halo 3 / halo 1
constexpr int SZ3 = 576, SZ1 = 416;      // box sizes padded to 128 B
constexpr int kBuf = 2 * SZ3 + 5 * SZ1;  // floats per level buffer
enum StageTile { TT = 0, TQ, TU, TV, TWF, TP, TR, NTILE };
__host__ __device__ constexpr int tile_off(int b) { return b < 2 ? b * SZ3 : 2 * SZ3 + (b - 2) * SZ1; }
constexpr unsigned kLevelBytes = (2 * R3 * TW + 5 * R1 * TW) * 4;
constexpr long long kSpinLimit = 1ll << 24;  // bounded mbarrier waits

struct StageMaps {
  CUtensorMap m[NTILE];
  int xmax[NTILE], ymax[NTILE];
};

// TMA-fed column kernel: a block owns 64 x 4 columns (two per thread); per
// level one box per field, 72 floats wide from i0-4 (16-byte aligned x):
// w, u, rho rows j0..j0+3, v rows j0..j0+4, pi' rows j0-1..j0+4
constexpr int CW = 72, CX = 4;
constexpr int kColBoxes = 5;  // w, pi', u, v, rho'
constexpr int kColRows[kColBoxes] = {4, 6, 4, 5, 4};
// box offsets in a level slot (floats, 128-byte aligned)
constexpr int kOffW = 0, kOffP = 288, kOffU = 736, kOffV = 1024, kOffR = 1408;
constexpr int kColSlot = 1696;                                  // floats per level slot (6784 B)
constexpr unsigned kColLevelBytes = (4 + 6 + 4 + 5 + 4) * CW * 4;
constexpr int kColRing = 4;
// backward sweep: per level the parked w, rho' and pi' (one level lower) of
// the block's own 64 x 4 columns, 64-float boxes at i0
constexpr int kBackBoxes = 3, BW = 64;
constexpr int kBOffW = 0, kBOffR = 256, kBOffP = 512;
constexpr unsigned kBackLevelBytes = 3 * BW * 4 * 4;
struct ColumnMaps {
  CUtensorMap m[kColBoxes];
  CUtensorMap back[kBackBoxes];  // w, rho', pi' of the output
};

// plain loader with the TMA box geometry (moisture species beyond qv)
__device__ __forceinline__ void load_box3(float* __restrict__ dst, const float* __restrict__ plane, int P, int i0,
                                          int j0, int xmax, int ymax) {
  for (int e = threadIdx.y * TX + threadIdx.x; e < R3 * TW; e += NT) {
    const int ty = e / TW, tx = e - ty * TW;
    const int gi = iclamp(i0 - XO + tx, 0, xmax), gj = iclamp(j0 - 3 + ty, 0, ymax);
    dst[e] = plane[gj * P + gi];
  }
}

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long* b, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* b, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* b, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* b, unsigned parity) {
  for (long long it = 0; it < kSpinLimit; ++it)
    if (mbar_try_wait(b, parity)) return true;
  return false;
}
__device__ __forceinline__ void tma_load_3d(float* dst, const CUtensorMap* map, int x, int y, int z,
                                            unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
      ::"r"(smem_u32(dst)), "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

// one level's seven boxes into buffer `buf` (called by one thread)
__device__ __forceinline__ void issue_level(const StageMaps& M, float* buf, unsigned long long* bar, int i0, int j0,
                                            int k, int nz) {
  const int kc = imin(k, nz - 1);
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  mbar_expect_tx(bar, kLevelBytes);
  tma_load_3d(buf + tile_off(TT), &M.m[TT], i0 - XO, j0 - 3, kc, bar);
  tma_load_3d(buf + tile_off(TQ), &M.m[TQ], i0 - XO, j0 - 3, kc, bar);
  tma_load_3d(buf + tile_off(TU), &M.m[TU], i0 - XO, j0 - 1, kc, bar);
  tma_load_3d(buf + tile_off(TV), &M.m[TV], i0 - XO, j0 - 1, kc, bar);
  tma_load_3d(buf + tile_off(TWF), &M.m[TWF], i0 - XO, j0 - 1, k, bar);
  tma_load_3d(buf + tile_off(TP), &M.m[TP], i0 - XO, j0 - 1, kc, bar);
  tma_load_3d(buf + tile_off(TR), &M.m[TR], i0 - XO, j0 - 1, kc, bar);
}

// replace out-of-range box elements by the clamped ones: columns first, then
// whole rows (so corners get clamp(x) and clamp(y))
__device__ void fix_box(float* t, int rows, int halo, int i0, int j0, int xmax, int ymax, int tid) {
  const int x0 = i0 - XO, y0 = j0 - halo;
  const int lxlo = imax(-x0, 0), lxhi = imin(xmax - x0, TW - 1);
  const int lylo = imax(-y0, 0), lyhi = imin(ymax - y0, rows - 1);
  if (lxlo > 0 || lxhi < TW - 1)
    for (int e = tid; e < rows * TW; e += NT) {
      const int r = e / TW, c = e - r * TW;
      if (c < lxlo) t[e] = t[r * TW + lxlo];
      else if (c > lxhi) t[e] = t[r * TW + lxhi];
    }
  __syncthreads();
  if (lylo > 0 || lyhi < rows - 1)
    for (int e = tid; e < rows * TW; e += NT) {
      const int r = e / TW, c = e - r * TW;
      if (r < lylo) t[e] = t[lylo * TW + c];
      else if (r > lyhi) t[e] = t[lyhi * TW + c];
    }
}

// kRaw: also write the tendency R itself (the last stage: the finish kernel
// forms the FP64 state from it)
constexpr int kStageRing = 3;  // level slots: k, k+1 resident, k+2 in flight

template <bool kRaw, bool kSpec>
__device__ __forceinline__ void stage_body(const Dims& d, const Tab& t, const Flags& fl, const StageMaps& M,
                                           const WS& win, const WS& w0, const WS& wout, const WS& rout, float dts,
                                           int kchunk, unsigned* err, int bx, int by, int bz) {
  __shared__ __align__(128) float sbuf[kStageRing][kBuf];
  __shared__ __align__(128) float sQm[R3 * TW], sQm2[R3 * TW];  // a pair of moisture species beyond qv (plain loads)
  __shared__ float sFx[2][TY * (TX + 1)], sFy[2][(TY + 1) * TX];  // theta' / qv (or a moisture pair)
  __shared__ __align__(8) unsigned long long sbar[kStageRing];
  // the flags, fixed at compile time for the kSpec composition
  const bool f_weno = kSpec || fl.weno_scalars, f_adv = kSpec || fl.weno_advective;
  const bool f_moist = !kSpec && fl.moist, f_dd = !kSpec && fl.div_damp > 0.0;
  const int f_cor = kSpec ? 0 : fl.coriolis;
  const int nx = d.nx, ny = d.ny, nz = d.nz, P = d.P;
  const unsigned pl = (unsigned)d.plane;  // a field has < 2^32 elements (checked when the model is made)
  const int i0 = bx * TX, j0 = by * TY;
  const int kb = bz * kchunk;
  const int klast = (kb + kchunk >= nz) ? nz : kb + kchunk - 1;  // the top chunk also owns face nz
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
  const int i = i0 + tx, j = j0 + ty;
  const bool in_box = i <= nx && j <= ny;
  const bool cell = i < nx && j < ny;
  const float cp = (float)kCp;
  const int o1 = (ty + 1) * TW + (tx + XO), o3 = (ty + 3) * TW + (tx + XO);  // own point in the boxes
  const int dim = (i > 0) ? -1 : 0;     // im - i, im = max(i-1, 0)
  const int ipu = imin(i, nx - 1) - i;  // ip - i on u faces (-1 at i = nx)
  const int jpv = imin(j, ny - 1) - j;  // jp - j on v faces (-1 at j = ny)
  const int djm = (j > 0) ? -1 : 0;     // jm - j
  const unsigned colc = (unsigned)(imin(j, ny) * P + imin(i, nx));
  const bool edge = (i0 - XO < 0) || (j0 - 3 < 0) || (i0 - XO + TW > nx - 1) || (j0 + TY + 3 > ny - 1);
  // levels kb..ktop are read: every level of the chunk, and the one above
  // its last cell level (capped at the top face nz); level L sits in slot
  // (L - kb) % kStageRing, whose mbarrier phase is ((L - kb) / kStageRing) & 1
  const int ktop = (klast < nz) ? klast + 1 : nz;
  int hi = imin(kb + 1, ktop);  // highest level issued
  if (tid == 0) {
    for (int sl = 0; sl < kStageRing; ++sl) mbar_init(&sbar[sl], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    for (int L = kb; L <= hi; ++L) issue_level(M, sbuf[L - kb], &sbar[L - kb], i0, j0, L, nz);
  }
  // bounded wait for level L by one thread, released to the block by the
  // barrier; on a timeout thread 0 drains every copy still in flight
  auto level_ready = [&](int L) -> bool {
    const int lev = L - kb;
    const bool arrived =
        (tid != 0) || mbar_wait_bounded(&sbar[lev % kStageRing], (unsigned)(lev / kStageRing) & 1u);
    if (__syncthreads_or(!arrived)) {
      if (tid == 0) {
        atomicOr(err, (unsigned)kErrWaitTimeout);
        for (int l = L; l <= hi; ++l)
          mbar_wait_bounded(&sbar[(l - kb) % kStageRing], (unsigned)((l - kb) / kStageRing) & 1u);
      }
      return false;
    }
    return true;
  };
  // edge blocks: out-of-range box elements become the clamped ones
  auto fix_level = [&](float* buf) {
    fix_box(buf + tile_off(TT), R3, 3, i0, j0, M.xmax[TT], M.ymax[TT], tid);
    fix_box(buf + tile_off(TQ), R3, 3, i0, j0, M.xmax[TQ], M.ymax[TQ], tid);
    for (int b = TU; b < NTILE; ++b) fix_box(buf + tile_off(b), R1, 1, i0, j0, M.xmax[b], M.ymax[b], tid);
    __syncthreads();
  };
  // vertical registers of the own column
  float wT[7], wQ[7];
  float wprev = 0.f, pprev = 0.f, rprev = 0.f, uprev = 0.f, vprev = 0.f;
  if (cell) {
#pragma unroll
    for (int m = 0; m < 7; ++m) {
      const unsigned o = (unsigned)iclamp(kb + m - 3, 0, nz - 1) * pl + colc;
      wT[m] = win.f[THETA][o];
      wQ[m] = win.f[QV][o];
    }
    const unsigned o = (unsigned)imax(kb - 1, 0) * pl + colc;
    wprev = win.f[W][o];
    pprev = win.f[PI][o];
    rprev = win.f[RHO][o];
  }
  // u, v of the level below the chunk at the own faces (k = 0: the level itself)
  if (kb > 0 && in_box) {
    const unsigned o = (unsigned)(kb - 1) * pl;
    if (j < ny) uprev = win.f[U][o + (unsigned)(j * P + (i + ipu))];
    if (i < nx) vprev = win.f[V][o + (unsigned)((j + jpv) * P + i)];
  }
  const bool has_base = w0.f[U] != nullptr;
  const bool base_in = has_base && w0.f[U] == win.f[U];  // first stage: the base state is the input
  float fcT = 0.f, fcQ = 0.f;  // carried vertical WENO fluxes (top face of the level below)
  // the sum of every value written: non-finite iff one of them is (the
  // values are perturbations, far from overflowing a sum)
  float fsum = 0.f;
  if (!level_ready(kb)) return;
  if (edge) fix_level(sbuf[0]);
  int cur = 0;  // ring slot of level k (k - kb mod kStageRing, rotated)
  for (int k = kb; k <= klast; ++k) {
    const int nxt = (cur + 1 == kStageRing) ? 0 : cur + 1, nn = (nxt + 1 == kStageRing) ? 0 : nxt + 1;
    const bool cells_here = k < nz;  // uniform across the block
    const int kc = imin(k, nz - 1);
    // This level's global loads (the base state the stage adds its tendency
    // to, when it is not the input), issued before the wait for the next
    // level's boxes so that their latencies overlap it and one another.
    const unsigned c = (unsigned)k * pl + colc;
    const bool do_u = cells_here && in_box && j < ny, do_v = cells_here && in_box && i < nx;
    float bU = 0.f, bV = 0.f, bW = 0.f, bR = 0.f, bP = 0.f, bT = 0.f, bQ = 0.f;
    if (has_base && !base_in) {
      if (do_u) bU = w0.f[U][c];
      if (do_v) bV = w0.f[V][c];
      if (cell) {
        bW = w0.f[W][c];
        if (cells_here) {
          bR = w0.f[RHO][c];
          bP = w0.f[PI][c];
          bT = w0.f[THETA][c];
          bQ = w0.f[QV][c];
        }
      }
    }
    if (k + 1 <= ktop) {
      if (!level_ready(k + 1)) break;
      if (edge) fix_level(sbuf[nxt]);
    }
    // past that barrier every thread is done with level k-1 (its values of
    // the level below live in registers), so its slot takes level k+2
    if (tid == 0 && k + 2 <= ktop)
      issue_level(M, sbuf[nn], &sbar[nn], i0, j0, k + 2, nz);
    if (k + 2 <= ktop) hi = k + 2;
    float* const buf = sbuf[cur];
    const float* const sT = buf + tile_off(TT);
    const float* const sQ = buf + tile_off(TQ);
    const float* const sU = buf + tile_off(TU);
    const float* const sV = buf + tile_off(TV);
    const float* const sW = buf + tile_off(TWF);
    const float* const sP = buf + tile_off(TP);
    const float* const sR = buf + tile_off(TR);
    const float* const nb = sbuf[nxt];  // level k+1 (k < nz)
    const float* const nU = nb + tile_off(TU);
    const float* const nV = nb + tile_off(TV);
    const float* const nW = nb + tile_off(TWF);
    const float* const nR = nb + tile_off(TR);
    // the level's vertical neighbours: u, v at kp1 = min(k+1, nz-1) and at
    // km = max(k-1, 0), w at face kp1 beside the u / v faces, w at face k+1
    // and rho' at kp1 in the own column
    const float* const wkp1 = (k + 1 < nz) ? nW : sW;  // face kp1
    const float gu_p = nU[o1 + ipu], gu_m = (k > 0) ? uprev : sU[o1 + ipu];
    const float gw_u = wkp1[o1 + ipu];
    const float gv_p = nV[o1 + jpv * TW], gv_m = (k > 0) ? vprev : sV[o1 + jpv * TW];
    const float gw_v = wkp1[o1 + jpv * TW];
    const float g_wt = nW[o1], g_rk = nR[o1];
    if (base_in) {
      bU = sU[o1];
      bV = sV[o1];
      bW = sW[o1];
      bR = sR[o1];
      bP = sP[o1];
      bT = sT[o3];
      bQ = sQ[o3];
    }
    // base value of q at this point: preloaded for the dynamic fields
    auto base_of = [&](int q) -> float {
      switch (q) {
        case U: return bU;
        case V: return bV;
        case W: return bW;
        case RHO: return bR;
        case PI: return bP;
        case THETA: return bT;
        case QV: return bQ;
        default: return w0.f[q][c];
      }
    };
    auto emit = [&](int q, float r) {
      const float o = has_base ? base_of(q) + dts * r : r;  // no base: raw tendency
      wout.f[q][c] = o;
      fsum += o;
      if (kRaw) rout.f[q][c] = r;
    };
    if (do_u) {  // u face (i, j, k)
      const float ump = sU[o1 + ipu], umm = sU[o1 + dim];
      const float uc = 0.5f * (umm + ump);
      const float ux = (ump - umm) * t.dx_inv;
      const float uy = (sU[o1 + ipu + TW] - sU[o1 + ipu - TW]) * (0.5f * t.dy_inv);
      const float uz = (gu_p - gu_m) * (0.5f * t.idza[k]);
      const float vc = 0.25f * (sV[o1 + dim - TW] + sV[o1 + ipu - TW] + sV[o1 + dim] + sV[o1 + ipu]);
      const float wc = 0.5f * (sW[o1 + ipu] + gw_u);
      float r = -(uc * ux + vc * uy + wc * uz);
      if (f_cor) r += (f_cor == 2 ? t.f0 + t.beta * (((float)j + 0.5f) * t.dy - 0.5f * (float)ny * t.dy) : t.f0) * vc;
      r -= cp * (0.5f * (sT[o3 + dim] + sT[o3 + ipu])) * (sP[o1 + ipu] - sP[o1 + dim]) * t.dx_inv;
      emit(U, r);
    }
    if (do_v) {  // v face (i, j, k)
      const int dp1 = jpv * TW, dm1 = djm * TW;
      const float vpp = sV[o1 + dp1], vmm = sV[o1 + dm1];
      const float vc = 0.5f * (vmm + vpp);
      const float vy = (vpp - vmm) * t.dy_inv;
      const float vx = (sV[o1 + dp1 + 1] - sV[o1 + dp1 - 1]) * (0.5f * t.dx_inv);
      const float vz = (gv_p - gv_m) * (0.5f * t.idza[k]);
      const float uc = 0.25f * (sU[o1 + dim + dm1] + sU[o1 + dm1] + sU[o1 + dim + dp1] + sU[o1 + dp1]);
      const float wc = 0.5f * (sW[o1 + dp1] + gw_v);
      float r = -(uc * vx + vc * vy + wc * vz);
      if (f_cor) r -= (f_cor == 2 ? t.f0 + t.beta * (((float)j + 0.5f) * t.dy - 0.5f * (float)ny * t.dy) : t.f0) * uc;
      r -= cp * (0.5f * (sT[o3 + djm * TW] + sT[o3 + jpv * TW])) * (sP[o1 + dp1] - sP[o1 + dm1]) * t.dy_inv;
      emit(V, r);
    }
    // w face (i, j, k), k = 0..nz; at k = nz the boxes other than w hold level nz-1 = kc
    const float wk = sW[o1];
    if (cell) {
      const float wkc = cells_here ? wk : wprev;
      const float wc = 0.5f * (wkc + wk);
      const float wz = (wk - wprev) * t.idza[kc];
      const float wx = (sW[o1 + 1] - sW[o1 - 1]) * (0.5f * t.dx_inv);
      const float wy = (sW[o1 + TW] - sW[o1 - TW]) * (0.5f * t.dy_inv);
      const float uc = 0.5f * (sU[o1] + sU[o1 + 1]);
      const float vc = 0.5f * (sV[o1] + sV[o1 + TW]);
      float r = -(uc * wx + vc * wy + wc * wz);
      const float thc = sT[o3], pic = sP[o1];
      const float thm = wT[2];  // theta'(max(k-1, 0))
      const float pim = (k == 0) ? pic : pprev;
      r -= cp * (0.5f * (thm + thc)) * (pic - pim) * t.idzw[k];
      float qcond = 0.f, qvc = wQ[3];  // qv(kc)
      if (f_moist) {
        const unsigned ckc = (unsigned)kc * pl + colc;
        qcond = win.f[QC][ckc] + win.f[QR][ckc] + win.f[QI][ckc] + win.f[QS][ckc] + win.f[QG][ckc];
      }
      r += (float)kG * (thc * t.th0inv[kc] + (float)kBuoyMoist * qvc - qcond);
      emit(W, r);
    }
    if (!cells_here) break;
    const float wt = g_wt;  // w at face k+1
    if (cell) {  // mass and pi
      const float rc = sR[o1];
      const float fx = sU[o1 + 1] * 0.5f * (rc + sR[o1 + 1]) - sU[o1] * 0.5f * (sR[o1 - 1] + rc);
      const float fy = sV[o1 + TW] * 0.5f * (rc + sR[o1 + TW]) - sV[o1] * 0.5f * (sR[o1 - TW] + rc);
      const float rkp = g_rk;
      const float fz = wt * 0.5f * (rc + rkp) - wk * 0.5f * (rprev + rc);
      emit(RHO, -(fx * t.dx_inv + fy * t.dy_inv + fz * t.idzc[k]));
      float r = 0.f;
      if (f_dd) {
        const float pc = sP[o1];
        const float lap = (sP[o1 + 1] - 2.f * pc + sP[o1 - 1]) * (t.dx_inv * t.dx_inv) +
                          (sP[o1 + TW] - 2.f * pc + sP[o1 - TW]) * (t.dy_inv * t.dy_inv);
        r = -(float)fl.div_damp * lap;
      }
      emit(PI, r);
    }
    // ---- scalars ----
    const float idz = t.idza[k];
    const bool vert = (k + 2 < nz || k >= 2);
    const float* sh = t.t0d + 6 * k;  // theta0(clamp(k+m)) - theta0(k), m = -3..2
    const float divh = (sU[o1 + 1] - sU[o1]) * t.dx_inv + (sV[o1 + TW] - sV[o1]) * t.dy_inv;
    // A species' box at level k is Q. With WENO its horizontal face fluxes
    // are first computed into sFx[slot] / sFy[slot] by all threads
    // (hflux for one species, hflux_pair for two as an f32x2 pair: slots 0
    // and 1), and after one barrier `scalar` reads them with the vertical
    // face fluxes; theta' and qv share that barrier, as do the two species of
    // a moisture pair.
    auto hflux = [&](const float* Q, int slot) {
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        const int t_ = tid + e * NT;
        if (t_ < TY * (TX + 1)) {
          const int fr = t_ / (TX + 1), ff = t_ - fr * (TX + 1);
          float F = 0.f;
          if (i0 + ff <= nx && j0 + fr < ny) {
            const float* qq = Q + (fr + 3) * TW + ff + XO;  // cell i0+ff, the face's right cell
            F = weno_face_f(qq[-3], qq[-2], qq[-1], qq[0], qq[1], sU[(fr + 1) * TW + ff + XO]);
          }
          sFx[slot][t_] = F;
        }
        if (t_ < (TY + 1) * TX) {
          const int fg = t_ / TX, fcl = t_ - fg * TX;
          float G = 0.f;
          if (j0 + fg <= ny && i0 + fcl < nx) {
            const float* qq = Q + (fg + 3) * TW + fcl + XO;
            G = weno_face_f(qq[-3 * TW], qq[-2 * TW], qq[-TW], qq[0], qq[TW], sV[(fg + 1) * TW + fcl + XO]);
          }
          sFy[slot][t_] = G;
        }
      }
    };
    // theta' and qv together: every face of the tile, TY (TX+1) x faces and
    // (TY+1) TX y faces, reconstructs both species as one f32x2 pair (same
    // face velocity, same stencil addresses in the two boxes), the stencil
    // loaded in upwind order by choosing the addresses; x and y faces share
    // one code path with the stencil stride chosen per face. Same face values
    // as hflux up to rounding.
    auto hflux_pair = [&](const float* A, const float* B) {  // species A and B (theta', qv or a moisture pair)
      // one x and one y face pair per thread: its cell's left and lower
      // faces; the top row's y faces go to warp 0 and the right column's x
      // faces to lanes 0..7 of warp 1 as a third (no warp diverges on it)
      auto face = [&](int off, int st, float vel, bool valid, float* d0, float* d1) {
        const int sp = vel >= 0.f ? st : -st;  // upwind order
        const F2 a0 = mk2(A[off - 2 * sp], B[off - 2 * sp]), a1 = mk2(A[off - sp], B[off - sp]);
        const F2 a2 = mk2(A[off], B[off]), a3 = mk2(A[off + sp], B[off + sp]);
        const F2 a4 = mk2(A[off + 2 * sp], B[off + 2 * sp]);
        float Ft, Fq;
        un2(weno_flux2(a0, a1, a2, a3, a4, vel), Ft, Fq);
        *d0 = valid ? Ft : 0.f;
        *d1 = valid ? Fq : 0.f;
      };
      // x face (i0+tx, j0+ty): cells i-1 (centre) .. in row ty
      face(o3 - 1, 1, sU[o1], i <= nx && j < ny, &sFx[0][ty * (TX + 1) + tx], &sFx[1][ty * (TX + 1) + tx]);
      // y face (i0+tx, j0+ty): cells j-1 (centre) .. in column tx
      face(o3 - TW, TW, sV[o1], j <= ny && i < nx, &sFy[0][ty * TX + tx], &sFy[1][ty * TX + tx]);
      if (tid < TX) {  // y face (i0+c, j0+TY)
        const int c = tid, bo = (TY + 3) * TW + c + XO;
        face(bo - TW, TW, sV[(TY + 1) * TW + c + XO], j0 + TY <= ny && i0 + c < nx, &sFy[0][TY * TX + c],
             &sFy[1][TY * TX + c]);
      } else if (tid < TX + TY) {  // x face (i0+TX, j0+f)
        const int f = tid - TX, bo = (f + 3) * TW + TX + XO;
        face(bo - 1, 1, sU[(f + 1) * TW + TX + XO], i0 + TX <= nx && j0 + f < ny, &sFx[0][f * (TX + 1) + TX],
             &sFx[1][f * (TX + 1) + TX]);
      }
    };
    // species q's tendency from its horizontal face fluxes (slot) and its
    // vertical ones: ft through the top face, fb through the bottom face
    // (WENO), or the column values z2 = q(k-1), z4 = q(k+1) (central)
    auto scalar = [&](int q, const float* Q, int slot, float ft, float fb, float z2, float z4) {
      float r = 0.f;
      const float qc = Q[o3];
      if (f_weno) {
        if (cell) {
          const float fe = sFx[slot][ty * (TX + 1) + tx + 1], fw = sFx[slot][ty * (TX + 1) + tx];
          const float fn = sFy[slot][(ty + 1) * TX + tx], fs = sFy[slot][ty * TX + tx];
          r = -(fe - fw) * t.dx_inv - (fn - fs) * t.dy_inv;
          float div = divh;
          if (vert) {
            r -= (ft - fb) * idz;
            div += (wt - wk) * idz;
          }
          if (f_adv) r += qc * div;
          else if (q == THETA) r -= t.t0c[k] * div;
        }
      } else if (cell) {
        const float ua = 0.5f * (sU[o1] + sU[o1 + 1]), va = 0.5f * (sV[o1] + sV[o1 + TW]);
        const float wa = 0.5f * (wk + wt);
        const float* qq = Q + o3;
        const float gx = gradc(qq[-3], qq[-2], qq[-1], qq[1], qq[2], qq[3], t.dx_inv, fl.advection);
        const float gy = gradc(qq[-3 * TW], qq[-2 * TW], qq[-TW], qq[TW], qq[2 * TW], qq[3 * TW], t.dy_inv, fl.advection);
        r = -(ua * gx + va * gy + wa * (z4 - z2) * (0.5f * idz));
      }
      if (cell) {
        if (q >= QV && qc <= 0.f && r < 0.f) r = 0.f;
        emit(q, r);
      }
    };
    // theta' is advected as theta - theta0(k): the carried flux of level
    // k-1 was formed with theta0(k-1) subtracted, and a WENO flux of q + s
    // is the flux of q plus w*s, so it is corrected by
    // w*(theta0(k-1) - theta0(k)) = -w*(theta0(k) - theta0(k-1)).
    const float tshift = (k > 0) ? -t.t0d[6 * (k - 1) + 4] : 0.f;
    float ftT = 0.f, fbT = 0.f, ftQ = 0.f, fbQ = 0.f;  // vertical face fluxes of theta' and qv
    if (f_weno) {
      hflux_pair(sT, sQ);
      if (cell) {  // the top face's pair, carried up as the next level's bottom face
        const F2 z1 = mk2(wT[1] + sh[1], wQ[1]), z2 = mk2(wT[2] + sh[2], wQ[2]);
        const F2 z4 = mk2(wT[4] + sh[4], wQ[4]), z5 = mk2(wT[5] + sh[5], wQ[5]);
        const F2 qc = mk2(sT[o3], sQ[o3]);
        un2(weno_vflux2(z1, z2, qc, z4, z5, wt), ftT, ftQ);
        if (k > kb) {
          fbT = fcT + wk * tshift;
          fbQ = fcQ;
        } else {
          un2(weno_vflux2(mk2(wT[0] + sh[0], wQ[0]), z1, z2, qc, z4, wk), fbT, fbQ);
        }
        fcT = ftT;
        fcQ = ftQ;
      }
      __syncthreads();
    }
    scalar(THETA, sT, 0, ftT, fbT, wT[2] + sh[2], wT[4] + sh[4]);
    scalar(QV, sQ, 1, ftQ, fbQ, wQ[2], wQ[4]);
    if (f_moist) {
      // the moisture species in pairs (qc qr, qi qs, and qg with itself),
      // each pair's faces reconstructed as one f32x2 pair like theta' and qv
      for (int qa = QC; qa <= QG; qa += 2) {
        const int qb = (qa + 1 <= QG) ? qa + 1 : qa;
        __syncthreads();  // sQm, sQm2 and the flux slots are no longer read
        load_box3(sQm, win.f[qa] + (unsigned)k * pl, P, i0, j0, nx - 1, ny - 1);
        if (qb != qa) load_box3(sQm2, win.f[qb] + (unsigned)k * pl, P, i0, j0, nx - 1, ny - 1);
        __syncthreads();
        const float* const QB = (qb != qa) ? sQm2 : sQm;
        if (f_weno) {
          hflux_pair(sQm, QB);
          __syncthreads();
        }
        float za[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, zb[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        float fta = 0.f, fba = 0.f, ftb = 0.f, fbb = 0.f;
        if (cell) {
#pragma unroll
          for (int m = 0; m < 6; ++m) {
            const unsigned o = (unsigned)iclamp(k + m - 3, 0, nz - 1) * pl + colc;
            za[m] = win.f[qa][o];
            zb[m] = win.f[qb][o];
          }
          if (f_weno) {
            const F2 z1 = mk2(za[1], zb[1]), z2 = mk2(za[2], zb[2]), z4 = mk2(za[4], zb[4]);
            const F2 qc2 = mk2(sQm[o3], QB[o3]);
            un2(weno_vflux2(z1, z2, qc2, z4, mk2(za[5], zb[5]), wt), fta, ftb);
            un2(weno_vflux2(mk2(za[0], zb[0]), z1, z2, qc2, z4, wk), fba, fbb);
          }
        }
        scalar(qa, sQm, 0, fta, fba, za[2], za[4]);
        if (qb != qa) scalar(qb, QB, 1, ftb, fbb, zb[2], zb[4]);
      }
    }
    // slide the column registers up one level
    if (cell) {
#pragma unroll
      for (int m = 0; m < 6; ++m) {
        wT[m] = wT[m + 1];
        wQ[m] = wQ[m + 1];
      }
      const unsigned o = (unsigned)imin(k + 4, nz - 1) * pl + colc;
      wT[6] = win.f[THETA][o];
      wQ[6] = win.f[QV][o];
      wprev = wk;
      pprev = sP[o1];
      rprev = sR[o1];
    }
    uprev = sU[o1 + ipu];
    vprev = sV[o1 + jpv * TW];
    cur = nxt;
  }
  if (!isfinite(fsum)) atomicOr(err, (unsigned)kErrNonFinite);
}

template <bool kRaw, bool kSpec>
__global__ void __launch_bounds__(NT, 3) k_mx_stage(const __grid_constant__ Dims d, const __grid_constant__ Tab t,
                                                    const __grid_constant__ Flags fl,
                                                    const __grid_constant__ StageMaps M,
                                                    const __grid_constant__ WS win, const __grid_constant__ WS w0,
                                                    const __grid_constant__ WS wout, const __grid_constant__ WS rout,
                                                    float dts, int kchunk, unsigned* err) {
  stage_body<kRaw, kSpec>(d, t, fl, M, win, w0, wout, rout, dts, kchunk, err, blockIdx.x, blockIdx.y, blockIdx.z);
}

// the flag set kSpec compiles in: WENO5 scalars in advective form, dry, no
// Coriolis, no divergence damping
bool stage_spec(const Flags& fl) {
  return fl.weno_scalars && fl.weno_advective && !fl.moist && fl.coriolis == 0 && !(fl.div_damp > 0.0);
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
__device__ __forceinline__ void fb_mom_body(const Dims& d, const Tab& t, const WS& win, const WS& wout, float dtau,
                                            int do_w, int bx, int by, int bz) {
  const int i = bx * blockDim.x + threadIdx.x;
  const int j = by * blockDim.y + threadIdx.y;
  const int k = bz;
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
// One thread per column, 32 x 4 columns per block. The tridiagonal matrix is
// the same for every column, so its LU factors come precomputed in
// lu = [a(k), c'(k), 1/den(k)] x nz. Only the forward-elimination values
// dp(k) are kept on chip (one float per level and column in shared memory:
// 40 KB per block at nz = 80, so 5 blocks -- 20 warps -- fit an SM); the
// backward sweep re-derives the explicit terms from the same inputs, which
// the forward sweep has just pulled through L2.
__global__ void k_mx_fb_mom(const __grid_constant__ Dims d, const __grid_constant__ Tab t,
                            const __grid_constant__ WS win, const __grid_constant__ WS wout, float dtau, int do_w) {
  fb_mom_body(d, t, win, wout, dtau, do_w, blockIdx.x, blockIdx.y, blockIdx.z);
}

// apply_uv: the u/v backward update of the previous substep is applied here,
// on the fly, from this substep's input pi' (the previous substep's result):
// u(i) += dtau (-cp theta0(k) (pi'(ip) - pi'(im)) / dx) with the clamped
// neighbours ip = min(i, nx-1), im = max(i-1, 0) (runge_kutta.cpp:65-75
// backward half); the updated u, v enter this substep's divergence and are
// written to the output. After the last substep of a stage one u/v kernel
// applies the final update in place. cdx = -cp dtau / dx, cdy likewise.
// Per-grid launch choices set by the autotuner (vibe_gb300_autotune): the
// stage kernel's levels per block and the column kernel variant. Every
// variant computes the same update; results differ only by FP32 rounding
// (each variant's own FMA contraction, the stage kernel's recomputed
// vertical fluxes at level-chunk starts).
struct TuneKey {
  int nx, ny, nz;
  bool operator<(const TuneKey& o) const {
    return nx != o.nx ? nx < o.nx : (ny != o.ny ? ny < o.ny : nz < o.nz);
  }
};
std::mutex g_tune_mu;
std::map<TuneKey, MixedTune> g_tune;

bool tune_of(const Dims& d, MixedTune* t) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  auto it = g_tune.find(TuneKey{d.nx, d.ny, d.nz});
  if (it == g_tune.end()) return false;
  *t = it->second;
  return true;
}

constexpr int kDefaultHeviRing = 4;  // single-domain column kernel: 0 = register ring
constexpr int kDefaultHeviPar = 0;   // levels per thread of the level-split column kernel (0 = off)
constexpr int kDefaultHeviTwo = 2;   // ring depth of the two-columns-per-thread kernel (0 = off)
constexpr bool kDefaultHeviTma = true;  // TMA-fed two-column kernel (VIBE_GB300_HEVI_TMA=0 turns it off; candidate 4)
constexpr bool kDefaultHeviDefer = true;  // ... with the w/rho' corrections deferred to the reader (candidate 5)
constexpr int kBatchTwoRing = 2;     // work-list column kernel of groups: the single-domain default

// 4-byte asynchronous global -> shared copies (sm_80+ cp.async), grouped
__device__ __forceinline__ void cp_async4(float* smem, const float* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

template <int kPF, int kRing>
__device__ __forceinline__ void hevi_body(const Dims& d, const Tab& t, const Flags& fl, const WS& win, const WS& wout,
                                          float dtau, const float* __restrict__ lu, int apply_uv, float cdx,
                                          float cdy, int bx, int by) {
  // per-level tables in shared memory; the forward sweep parks its per-level
  // results in the thread's own column of the output arrays (wt on the w
  // faces, dp on pi', the explicit source S on rho'), where the backward
  // sweep reads them back (from L2) and overwrites them with the final values
  extern __shared__ float s_tab[];
  const int nz = d.nz;
  float* s_tfz = s_tab;                    // nz+1
  float* s_idzw = s_tfz + (nz + 1);        // nz+1
  float* s_rfz = s_idzw + (nz + 1);        // nz+1
  float* s_idzc = s_rfz + (nz + 1);        // nz
  float* s_kap = s_idzc + nz;              // nz
  float* s_la = s_kap + nz;                // nz
  float* s_lc = s_la + nz;                 // nz
  float* s_li = s_lc + nz;                 // nz
  float* s_r0 = s_li + nz;                 // nz
  float* s_t0 = s_r0 + nz;                 // nz
  const int tid = threadIdx.y * blockDim.x + threadIdx.x;
  for (int e = tid; e <= nz; e += 128) {
    s_tfz[e] = t.tfz[e];
    s_idzw[e] = t.idzw[e];
    s_rfz[e] = t.rfz[e];
    if (e < nz) {
      s_idzc[e] = t.idzc[e];
      s_kap[e] = t.kap[e];
      s_la[e] = lu[e];
      s_lc[e] = lu[nz + e];
      s_li[e] = lu[2 * nz + e];
      s_r0[e] = t.r0c[e];
      s_t0[e] = t.t0c[e];
    }
  }
  __syncthreads();
  const int i = bx * blockDim.x + threadIdx.x;
  const int j = by * blockDim.y + threadIdx.y;
  if (i >= d.nx || j >= d.ny) return;
  const float b = (float)fl.hevi_beta, ob = 1.f - b;
  const float cpf = (float)kCp;
  const size_t col = (size_t)j * d.P + i;
  const size_t pl = d.plane;
  const float* __restrict__ U0 = win.f[U] + col;
  const float* __restrict__ V0 = win.f[V] + col;
  const float* __restrict__ W0 = win.f[W] + col;
  const float* __restrict__ P0 = win.f[PI] + col;
  const float* __restrict__ R0 = win.f[RHO] + col;
  float* __restrict__ Wo = wout.f[W] + col;
  float* __restrict__ Po = wout.f[PI] + col;
  float* __restrict__ Ro = wout.f[RHO] + col;
  float* __restrict__ Uo = wout.f[U] + col;
  float* __restrict__ Vo = wout.f[V] + col;
  const size_t vn = d.P;  // v(j+1) offset
  const float dxi = t.dx_inv, dyi = t.dy_inv;
  // clamped neighbour offsets of pi' (0 where the clamp lands on the column)
  const int ow = (i > 0) ? -1 : 0, oe = (i + 1 < d.nx) ? 1 : 0;
  const long long os = (j > 0) ? -(long long)vn : 0, on = (j + 1 < d.ny) ? (long long)vn : 0;
  const bool last_i = (i == d.nx - 1), last_j = (j == d.ny - 1);
  // Forward-sweep loads run ahead of their use: with kRing > 0 as 4-byte
  // cp.async copies into a per-thread shared-memory ring kRing levels deep
  // (no registers held, one commit group per level, wait_group kRing-1 before
  // a level is read; each thread reads only its own slots), else in a
  // register ring kPF levels deep.
  float fw[kPF], fp[kPF], fu0[kPF], fu1[kPF], fv0[kPF], fv1[kPF];
  float fpw[kPF], fpe[kPF], fps[kPF], fpn[kPF], fr[kPF];
  float* ring = s_t0 + nz;  // kRing x 11 x 128 floats after the tables
  auto rs = [&](int slot, int f) -> float* { return ring + ((size_t)slot * 11 + f) * 128 + tid; };
  auto issueF = [&](int L) {  // level L -> slot L % kRing
    const int slot = L % (kRing > 0 ? kRing : 1);
    const size_t o = (size_t)L * pl, o1 = o + pl;
    cp_async4(rs(slot, 0), W0 + o1);
    if (L + 1 < nz) cp_async4(rs(slot, 1), P0 + o1);
    else *rs(slot, 1) = 0.f;
    cp_async4(rs(slot, 2), U0 + o);
    cp_async4(rs(slot, 3), U0 + o + 1);
    cp_async4(rs(slot, 4), V0 + o);
    cp_async4(rs(slot, 5), V0 + o + vn);
    cp_async4(rs(slot, 10), R0 + o);
    if (apply_uv) {
      cp_async4(rs(slot, 6), P0 + o + ow);
      cp_async4(rs(slot, 7), P0 + o + oe);
      cp_async4(rs(slot, 8), P0 + o + os);
      cp_async4(rs(slot, 9), P0 + o + on);
    }
  };
  auto loadF = [&](int L, int q) {
    const size_t o = (size_t)L * pl, o1 = o + pl;
    fw[q] = W0[o1];
    fp[q] = (L + 1 < nz) ? P0[o1] : 0.f;
    fu0[q] = U0[o];
    fu1[q] = U0[o + 1];
    fv0[q] = V0[o];
    fv1[q] = V0[o + vn];
    fr[q] = R0[o];
    if (apply_uv) {
      fpw[q] = P0[o + ow];
      fpe[q] = P0[o + oe];
      fps[q] = P0[o + os];
      fpn[q] = P0[o + on];
    }
  };
  if (kRing > 0) {
    for (int L = 0; L < kRing; ++L) {
      if (L < nz) issueF(L);
      cp_async_commit();
    }
  } else {
#pragma unroll
    for (int q = 0; q < kPF; ++q)
      if (q < nz) loadF(q, q);
  }
  float p_k = P0[0];
  float w_k = W0[0];
  float wt_k = w_k;  // face 0: no pressure gradient
  Wo[0] = w_k;
  float dp_prev = 0.f;
  for (int k0 = 0; k0 < nz; k0 += kPF) {
#pragma unroll
    for (int q = 0; q < kPF; ++q) {
      const int k = k0 + q;
      if (k < nz) {
        float w_k1, pf1, u0, u1, v0, v1, r0_, pw_ = 0.f, pe_ = 0.f, ps_ = 0.f, pn_ = 0.f;
        if (kRing > 0) {
          cp_async_wait<(kRing > 0 ? kRing - 1 : 0)>();
          const int slot = k % (kRing > 0 ? kRing : 1);
          w_k1 = *rs(slot, 0);
          pf1 = *rs(slot, 1);
          u0 = *rs(slot, 2);
          u1 = *rs(slot, 3);
          v0 = *rs(slot, 4);
          v1 = *rs(slot, 5);
          r0_ = *rs(slot, 10);
          if (apply_uv) {
            pw_ = *rs(slot, 6);
            pe_ = *rs(slot, 7);
            ps_ = *rs(slot, 8);
            pn_ = *rs(slot, 9);
          }
        } else {
          w_k1 = fw[q];
          pf1 = fp[q];
          u0 = fu0[q];
          u1 = fu1[q];
          v0 = fv0[q];
          v1 = fv1[q];
          r0_ = fr[q];
          if (apply_uv) {
            pw_ = fpw[q];
            pe_ = fpe[q];
            ps_ = fps[q];
            pn_ = fpn[q];
          }
        }
        float wt_k1 = w_k1, p_k1 = 0.f;
        if (k + 1 < nz) {
          p_k1 = pf1;
          wt_k1 = w_k1 - dtau * ob * cpf * s_tfz[k + 1] * (p_k1 - p_k) * s_idzw[k + 1];
        }
        if (apply_uv) {
          const float tx_ = s_t0[k] * cdx, ty_ = s_t0[k] * cdy;
          u0 += tx_ * (p_k - pw_);
          u1 += tx_ * (pe_ - p_k);
          v0 += ty_ * (p_k - ps_);
          v1 += ty_ * (pn_ - p_k);
        }
        const float Dh = -(s_r0[k] * ((u1 - u0) * dxi + (v1 - v0) * dyi));
        if (kRing == 0 && k + kPF < nz) loadF(k + kPF, q);
        {
          const size_t o = (size_t)k * pl;
          Uo[o] = u0;
          Vo[o] = v0;
          if (last_i) Uo[o + 1] = u1;  // face nx (zero clamped gradient)
          if (last_j) Vo[o + vn] = v1;
        }
        const float rk = s_rfz[k], rk1 = s_rfz[k + 1], idz = s_idzc[k];
        const float dv_old = -(rk1 * w_k1 - rk * w_k) * idz;
        const float dv_t = -(rk1 * wt_k1 - rk * wt_k) * idz;
        const float S = Dh + ob * dv_old;
        const float rhs = p_k + dtau * s_kap[k] * (S + b * dv_t);
        const float dpk = (k == 0) ? rhs * s_li[0] : (rhs - s_la[k] * dp_prev) * s_li[k];
        const size_t o = (size_t)k * pl;
        Po[o] = dpk;
        Ro[o] = r0_ + dtau * S;  // rho' less the implicit part, added in the backward sweep
        Wo[o + pl] = wt_k1;  // face k+1 (face nz: w_old(nz), already final)
        if (kRing > 0) {
          // refill the slot only now that every value read from it has been used
          if (k + kRing < nz) issueF(k + kRing);
          cp_async_commit();
        }
        dp_prev = dpk;
        w_k = w_k1;
        wt_k = wt_k1;
        p_k = p_k1;
      }
    }
  }
  // ---- backward sweep: x(k) = dp(k) - c'(k) x(k+1); after x(k) is known, face
  // k+1 (needs x(k), x(k+1)) and cell k+1 (needs faces k+1, k+2) are final.
  if (kRing > 0) cp_async_wait<0>();
  constexpr int kB = kRing > 0 ? 4 : kPF;  // backward loads in flight (L2 hits)
  float bdp[kB], bwt[kB], bS[kB];
  auto loadB = [&](int kk, int q) {  // inputs of step kk (cell/face kk), parked by the forward sweep
    const size_t o = (size_t)kk * pl;
    bdp[q] = (kk >= 1) ? Po[o - pl] : 0.f;  // dp(kk-1)
    bwt[q] = Wo[o];                          // wt(kk)
    bS[q] = Ro[o];                           // rho'_old(kk) + dtau S(kk)
  };
#pragma unroll
  for (int q = 0; q < kB; ++q)
    if (nz - 1 - q >= 0) loadB(nz - 1 - q, q);
  float x_up = dp_prev;  // x(nz-1) = dp(nz-1)
  float wn_up = Wo[(size_t)nz * pl];
  for (int kk0 = nz - 1; kk0 >= 0; kk0 -= kB) {
#pragma unroll
    for (int q = 0; q < kB; ++q) {
      const int kk = kk0 - q;  // face kk and cell kk are finalised here
      if (kk >= 0) {
        const int k = kk - 1;
        const size_t okk = (size_t)kk * pl;
        float x_k = 0.f, wn_kk = bwt[q];
        if (k >= 0) {
          x_k = bdp[q] - s_lc[k] * x_up;
          wn_kk = bwt[q] - dtau * b * cpf * s_tfz[kk] * (x_up - x_k) * s_idzw[kk];
        }
        const float dv_new = -(s_rfz[kk + 1] * wn_up - s_rfz[kk] * wn_kk) * s_idzc[kk];
        const float rnew = bS[q] + dtau * b * dv_new;
        if (kk - kB >= 0) loadB(kk - kB, q);
        Ro[okk] = rnew;
        Po[okk] = x_up;
        Wo[okk] = wn_kk;
        x_up = x_k;
        wn_up = wn_kk;
      }
    }
  }
}

// Finite test of an FP64 value on its exponent bits (integer pipe; the FP64
// pipe, which bounds the finish kernel, is left to the arithmetic).
__device__ __forceinline__ bool finite64(double v) { return (__double2hiint(v) & 0x7ff00000) != 0x7ff00000; }

// Exact FP32 -> FP64 widening on the integer pipe (IEEE 754 binary32 ->
// binary64: rebias the exponent by 1023 - 127 = 896 and move the 23 fraction
// bits to the top of the 52; a subnormal m * 2^-149 with leading bit p becomes
// the normal 2^(p-149) (1 + frac), exponent field p + 874; zeros keep their
// sign; inf and NaN keep exponent 0x7ff and their fraction). GB300's FP64
// pipe, where the hardware conversion issues, runs at 1/64 of the FP32 rate;
// these integer operations run at full rate.
__device__ __forceinline__ double widen(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned s = u & 0x80000000u, e = (u >> 23) & 0xffu;
  unsigned m = u & 0x7fffffu, ex = e + 896u;
  if (e == 0xffu) ex = 0x7ffu;
  if (e == 0u) {
    if (m == 0u) {
      ex = 0u;
    } else {
      const int p = 31 - __clz((int)m);  // 0..22
      ex = (unsigned)(p + 874);
      m = (m << (23 - p)) & 0x7fffffu;
    }
  }
  return __hiloint2double((int)(s | (ex << 20) | (m >> 3)), (int)(m << 29));
}

// ---- finish: fold the last stage's acoustic increments into the FP64
// state, apply the sponge (damping.cpp:76-140) in FP64 and to the FP32
// working copy, which becomes the next step's s0 working copy.
// S1 = sponge(S0 + (double)(dt R3 + (W_final - W_stage3))) for the acoustic
// fields, S0 + (double)(dt R3) for theta and q (sponge on theta): the stage-3
// tendency and the acoustic increment of its substeps are summed in FP32 and
// added to the FP64 state with one conversion and one FP64 add per field.
// rin == nullptr: no tendency (single-substep entry points, S1 == S0).
// Also writes the next step's FP32 working copy W0.
// uv_dtau != 0: the last substep's u/v backward update (fb_mom_body, u and
// v) is applied here on the fly instead of by its own in-place launch
// The deferred corrections of a kDefer column kernel's w and rho' (see
// hevi_tma_body below), for 1 <= k <= nz-1 with cb = dtau beta cp:
//   w(k) = w~(k) - cb tfz(k) (pi'(k) - pi'(k-1)) idzw(k)   (faces 0, nz: w = w~)
// and with db = dtau beta, from the corrected w(k), w(k+1):
//   rho'(k) = rho~(k) - db (rfz(k+1) w(k+1) - rfz(k) w(k)) idzc(k)
__device__ __forceinline__ float defer_fix_w(const Tab& t, int nz, float cb, float wt, float pk, float pkm, int k) {
  return (k >= 1 && k < nz) ? wt - cb * t.tfz[k] * (pk - pkm) * t.idzw[k] : wt;
}
__device__ __forceinline__ float defer_fix_rho(const Tab& t, float db, float rt, float wk, float wk1, int k) {
  return rt + db * (-(t.rfz[k + 1] * wk1 - t.rfz[k] * wk) * t.idzc[k]);
}

// defer: wfin is a kDefer column kernel's output; its w and rho' get their
// corrections (with dtau = uv_dtau) on the fly
__device__ __forceinline__ void finish_body(const Dims& d, const Tab& t, const Flags& fl, const WS& wfin,
                                            const WS& wst, const WS& w0, const WS& rin, float dtf, const CS64& s0,
                                            const MS64& s1, unsigned* err, int bx, int by, int bz,
                                            float uv_dtau = 0.f, bool defer = false) {
  const int i = bx * blockDim.x + threadIdx.x;
  const int j = by * blockDim.y + threadIdx.y;
  const int k = bz;
  if (i > d.nx || j > d.ny || k > d.nz) return;
  const size_t c = IX(i, j, k);
  const int kc = imin(k, d.nz - 1);
  const double wd = t.spwd[k];
  const float wf = t.spw[k];
  const double sdt = (k < d.nz) ? t.spdt[k] : 0.0;
  // below the sponge layers (weight exactly 1, relaxation exactly 0; uniform
  // over the block, whose level is blockIdx.z) the sponge leaves every value
  // unchanged, so only the FP64 additions remain
  const bool plain = __double_as_longlong(wd) == 0x3ff0000000000000ll && __double_as_longlong(sdt) == 0ll;
  bool bad = false;
  auto incr = [&](int q) { return rin.f[q] ? dtf * rin.f[q][c] : 0.f; };
  const float cb = uv_dtau * (float)fl.hevi_beta * (float)kCp, db = uv_dtau * (float)fl.hevi_beta;
  auto w_at = [&](int kf) {  // w at face kf of this column, corrected when deferred
    const float wt = wfin.f[W][IX(i, j, kf)];
    if (!defer || kf < 1 || kf >= d.nz) return wt;
    return defer_fix_w(t, d.nz, cb, wt, wfin.f[PI][IX(i, j, kf)], wfin.f[PI][IX(i, j, kf - 1)], kf);
  };
  auto face = [&](int q) {
    float wv = (q == W) ? w_at(k) : wfin.f[q][c];
    if (uv_dtau != 0.f && q != W) {  // as fb_mom_body: k < nz and the face's clamped pi' neighbours
      const float* __restrict__ pn = wfin.f[PI];
      const float cp = (float)kCp;
      if (q == U) {
        const int ip = imin(i, d.nx - 1), im = imax(i - 1, 0);
        wv = wv + uv_dtau * (-cp * t.t0c[k] * (pn[IX(ip, j, k)] - pn[IX(im, j, k)]) * t.dx_inv);
      } else {
        const int jp = imin(j, d.ny - 1), jm = imax(j - 1, 0);
        wv = wv + uv_dtau * (-cp * t.t0c[k] * (pn[IX(i, jp, k)] - pn[IX(i, jm, k)]) * t.dy_inv);
      }
    }
    const double a = s0.f[q][c] + widen(incr(q) + (wv - wst.f[q][c]));
    const double v = plain ? a : wd * a;
    s1.f[q][c] = v;
    w0.f[q][c] = wf * wv;
    bad |= !finite64(v);
  };
  if (j < d.ny && k < d.nz) face(U);
  if (i < d.nx && k < d.nz) face(V);
  if (i < d.nx && j < d.ny) {
    if (fl.w_rigid && (k == 0 || k == d.nz)) {
      s1.f[W][c] = 0.0;
      w0.f[W][c] = 0.f;
    } else {
      face(W);
    }
  }
  if (i < d.nx && j < d.ny && k < d.nz) {
    {
      float wv = wfin.f[RHO][c];
      if (defer) wv = defer_fix_rho(t, db, wv, w_at(k), w_at(k + 1), k);
      const double a = s0.f[RHO][c] + widen(incr(RHO) + (wv - wst.f[RHO][c]));
      const double v = plain ? a : wd * (a + sdt * t.r0d[kc]);
      s1.f[RHO][c] = v;
      w0.f[RHO][c] = wf * wv;
      bad |= !finite64(v);
    }
    {
      const float wv = wfin.f[PI][c];
      const double a = s0.f[PI][c] + widen(incr(PI) + (wv - wst.f[PI][c]));
      const double v = plain ? a : wd * (a + sdt * t.p0d[kc]);
      s1.f[PI][c] = v;
      w0.f[PI][c] = wf * wv;
      bad |= !finite64(v);
    }
    {
      double v = s0.f[THETA][c] + widen(incr(THETA));
      if (!plain) v = wd * (v + sdt * t.t0dd[kc]);
      s1.f[THETA][c] = v;
      w0.f[THETA][c] = wf * wst.f[THETA][c];
      bad |= !finite64(v);
    }
    const int last = fl.moist ? QG : QV;
    for (int q = QV; q <= last; ++q) {
      const double v = s0.f[q][c] + widen(incr(q));
      s1.f[q][c] = v;
      w0.f[q][c] = wst.f[q][c];
      bad |= !finite64(v);
    }
  }
  if (bad) atomicOr(err, (unsigned)kErrNonFinite);
}

// FP32 field (device layout) -> FP64 FieldT storage (zeros outside the box)
__global__ void k_mx_finish(const __grid_constant__ Dims d, const __grid_constant__ Tab t,
                            const __grid_constant__ Flags fl, const __grid_constant__ WS wfin,
                            const __grid_constant__ WS wst, const __grid_constant__ WS w0,
                            const __grid_constant__ WS rin, float dtf, const __grid_constant__ CS64 s0,
                            const __grid_constant__ MS64 s1, unsigned* err, float uv_dtau, int defer) {
  finish_body(d, t, fl, wfin, wst, w0, rin, dtf, s0, s1, err, blockIdx.x, blockIdx.y, blockIdx.z, uv_dtau,
              defer != 0);
}

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
__device__ __forceinline__ void to_working_point(const Dims& d, const Tab& t, const CS64& s, const WS& w, int i,
                                                 int j, int k) {
  const size_t c = IX(i, j, k);
  if (j < d.ny && k < d.nz) w.f[U][c] = (float)s.f[U][c];
  if (i < d.nx && k < d.nz) w.f[V][c] = (float)s.f[V][c];
  if (i < d.nx && j < d.ny) w.f[W][c] = (float)s.f[W][c];
  if (k < d.nz) {  // cells incl. the ghost column/row
    w.f[RHO][c] = (float)(s.f[RHO][c] - t.r0d[k]);
    w.f[THETA][c] = (float)(s.f[THETA][c] - t.t0dd[k]);
    w.f[PI][c] = (float)(s.f[PI][c] - t.p0d[k]);
    for (int q = QV; q < NSPECIES; ++q)
      if (w.f[q]) w.f[q][c] = (float)s.f[q][c];  // species without a target are not prognostic
  }
}
__device__ __forceinline__ void to_working_body(const Dims& d, const Tab& t, const CS64& s, const WS& w, int bx,
                                                int by, int bz) {
  const int i = bx * blockDim.x + threadIdx.x;
  const int j = by * blockDim.y + threadIdx.y;
  const int k = bz;
  if (i > d.nx || j > d.ny || k > d.nz) return;
  to_working_point(d, t, s, w, i, j, k);
}
__global__ void k_mx_to_working(const __grid_constant__ Dims d, const __grid_constant__ Tab t,
                                const __grid_constant__ CS64 s, const __grid_constant__ WS w) {
  to_working_body(d, t, s, w, blockIdx.x, blockIdx.y, blockIdx.z);
}
// the columns of a box [ia, ib) x [ja, jb)
__global__ void k_mx_to_working_region(const __grid_constant__ Dims d, const __grid_constant__ Tab t,
                                       const __grid_constant__ CS64 s, const __grid_constant__ WS w, int ia, int ja,
                                       int ib, int jb) {
  const int i = ia + blockIdx.x * blockDim.x + threadIdx.x;
  const int j = ja + blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= ib || j >= jb || k > d.nz) return;
  to_working_point(d, t, s, w, i, j, k);
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

// Levels per block of the stage kernel: the columns' blocks times the level
// chunks should fill whole waves of resident blocks (a block's chunk is long,
// so a partial last wave idles the rest of the GPU). Chunks of at least 8
// levels keep the per-chunk start-up (column registers, one extra vertical
// flux per species) small.
// VIBE_GB300_STAGE_LEVELS=<n> overrides the choice (levels per block).
static int stage_kchunk(const Dims& d, bool fp64_out) {
  MixedTune tn;
  if (tune_of(d, &tn) && tn.stage_levels > 0) return imin(tn.stage_levels, d.nz);
  if (const char* e = std::getenv("VIBE_GB300_STAGE_LEVELS")) {
    const int v = std::atoi(e);
    if (v > 0) return imin(v, d.nz);
  }
  static int resident[2] = {0, 0};
  int& res = resident[fp64_out ? 1 : 0];
  if (res == 0) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (fp64_out)
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mx_stage<true, false>, NT, 0);
    else
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mx_stage<false, false>, NT, 0);
    res = imax(1, sms * per_sm);
  }
  const long cols = (long)((d.nx + TX) / TX) * ((d.ny + TY) / TY);
  int best = d.nz;
  double best_eff = -1.0;
  for (int nch = 1; nch <= 16; ++nch) {
    const int kc = (d.nz + nch - 1) / nch;
    if (kc < 8 && nch > 1) break;
    const int n = (d.nz + kc - 1) / kc;
    const double waves = (double)(cols * n) / res;
    const double eff = waves / std::ceil(waves) - 0.004 * n;  // small cost per chunk
    if (eff > best_eff) { best_eff = eff; best = kc; }
  }
  return best;
}

// TMA descriptors of the stage kernel's boxes, one per (field, box shape),
// cached for the life of the process (buffers live as long as their model;
// the key includes the shape, so a reused address with other sizes gets its
// own descriptor).
namespace {
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
std::mutex g_map_mu;
std::map<std::tuple<const void*, int, int, int, int, size_t, int>, CUtensorMap> g_maps;

bool encode_fn() {
  if (g_encode) return true;
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q{};
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess || !fn)
    return false;
  g_encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
  return true;
}

bool box_map(const float* base, int xext, int yext, int zext, int P, size_t plane, int rows, CUtensorMap* out,
             int width = TW) {
  const auto key = std::make_tuple((const void*)base, xext, yext, zext, P, plane, rows * 1024 + width);
  std::lock_guard<std::mutex> lk(g_map_mu);
  auto it = g_maps.find(key);
  if (it != g_maps.end()) {
    *out = it->second;
    return true;
  }
  if (!encode_fn()) return false;
  CUtensorMap m;
  const cuuint64_t dims[3] = {(cuuint64_t)xext, (cuuint64_t)yext, (cuuint64_t)zext};
  const cuuint64_t strides[2] = {(cuuint64_t)P * sizeof(float), (cuuint64_t)plane * sizeof(float)};
  const cuuint32_t box[3] = {(cuuint32_t)width, (cuuint32_t)rows, 1};
  const cuuint32_t es[3] = {1, 1, 1};
  if (g_encode(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, (void*)base, dims, strides, box, es,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return false;
  g_maps.emplace(key, m);
  *out = m;
  return true;
}

bool stage_maps(const Dims& d, const WS& win, StageMaps& M) {
  struct Spec { int q, xe, ye, ze, rows; };
  const Spec sp[NTILE] = {{THETA, d.nx, d.ny, d.nz, R3},     {QV, d.nx, d.ny, d.nz, R3},
                          {U, d.nx + 1, d.ny, d.nz, R1},     {V, d.nx, d.ny + 1, d.nz, R1},
                          {W, d.nx, d.ny, d.nz + 1, R1},     {PI, d.nx, d.ny, d.nz, R1},
                          {RHO, d.nx + 1, d.ny + 1, d.nz, R1}};
  for (int b = 0; b < NTILE; ++b) {
    if (!box_map(win.f[sp[b].q], sp[b].xe, sp[b].ye, sp[b].ze, d.P, d.plane, sp[b].rows, &M.m[b])) return false;
    M.xmax[b] = sp[b].xe - 1;
    M.ymax[b] = sp[b].ye - 1;
  }
  return true;
}

// boxes of the TMA-fed column kernel: every field over the whole padded
// allocation (P x (ny+1) x (nz+1)), so only the left edge and the rows outside
// 0..ny arrive as zeros (the kernel never uses them)
bool column_maps(const Dims& d, const WS& win, const WS& wout, ColumnMaps& C) {
  const int q[kColBoxes] = {W, PI, U, V, RHO};
  for (int b = 0; b < kColBoxes; ++b)
    if (!box_map(win.f[q[b]], d.P, d.ny + 1, d.nz + 1, d.P, d.plane, kColRows[b], &C.m[b], CW)) return false;
  const int qb[kBackBoxes] = {W, RHO, PI};
  for (int b = 0; b < kBackBoxes; ++b)
    if (!box_map(wout.f[qb[b]], d.P, d.ny + 1, d.nz + 1, d.P, d.plane, 4, &C.back[b], BW)) return false;
  return true;
}
}  // namespace

int mixed_stage(const Dims& d, const Tab& t, const Flags& fl, const WS& win, const WS& w0, const WS& wout,
                const WS* rout, double dt_stage, unsigned* err, cudaStream_t stream) {
  StageMaps M;
  if (!stage_maps(d, win, M)) return -1;
  const dim3 b(TX, TY);
  const bool raw = rout != nullptr;
  const int kchunk = stage_kchunk(d, raw);
  const dim3 g((d.nx + TX) / TX, (d.ny + TY) / TY, (d.nz + kchunk - 1) / kchunk);
  const bool spec = stage_spec(fl);
  if (raw && spec)
    k_mx_stage<true, true><<<g, b, 0, stream>>>(d, t, fl, M, win, w0, wout, *rout, (float)dt_stage, kchunk, err);
  else if (raw)
    k_mx_stage<true, false><<<g, b, 0, stream>>>(d, t, fl, M, win, w0, wout, *rout, (float)dt_stage, kchunk, err);
  else if (spec)
    k_mx_stage<false, true><<<g, b, 0, stream>>>(d, t, fl, M, win, w0, wout, wout, (float)dt_stage, kchunk, err);
  else
    k_mx_stage<false, false><<<g, b, 0, stream>>>(d, t, fl, M, win, w0, wout, wout, (float)dt_stage, kchunk, err);
  return 0;
}

// ---- adjoint of the FP32 forward-backward substep (k_mx_fb_mass, then
// fb_mom_body with w): the transposed momentum phase (each cell gathers the
// pressure-gradient coefficients of its faces, uniform per level) and then
// the transposed mass phase (each face gathers the divergence of its two
// cells, with Z = bar_rho' + kappa bar_pi'); in place on the bars.
__global__ void k_mxad_pi(Dims d, Tab t, WS bar, float dtau, int with_w) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= d.nx || j >= d.ny || k >= d.nz) return;
  const float cp = (float)kCp;
  const float* bu = bar.f[U];
  const float* bv = bar.f[V];
  const float* bw = bar.f[W];
  const float cu = -cp * t.t0c[k] * t.dx_inv, cv = -cp * t.t0c[k] * t.dy_inv;
  float acc = cu * (bu[IX(i, j, k)] - bu[IX(i + 1, j, k)]);
  if (i == d.nx - 1) acc += cu * bu[IX(d.nx, j, k)];
  if (i == 0) acc -= cu * bu[IX(0, j, k)];
  acc += cv * (bv[IX(i, j, k)] - bv[IX(i, j + 1, k)]);
  if (j == d.ny - 1) acc += cv * bv[IX(i, d.ny, k)];
  if (j == 0) acc -= cv * bv[IX(i, 0, k)];
  // w faces: face f uses pi'(min(f, nz-1)) - pi'(max(f-1, 0)) with -cp tfz(f) idzw(f)
  auto cw = [&](int f) { return -cp * t.tfz[f] * t.idzw[f]; };
  if (with_w) {
    acc += cw(k) * bw[IX(i, j, k)] - cw(k + 1) * bw[IX(i, j, k + 1)];
    if (k == d.nz - 1) acc += cw(d.nz) * bw[IX(i, j, d.nz)];
    if (k == 0) acc -= cw(0) * bw[IX(i, j, 0)];
  }
  bar.f[PI][IX(i, j, k)] += dtau * acc;
}

__global__ void k_mxad_vel(Dims d, Tab t, WS bar, float dtau) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i > d.nx || j > d.ny || k > d.nz) return;
  auto Z = [&](int ci, int cj, int ck) {
    const size_t c = IX(ci, cj, ck);
    return bar.f[RHO][c] + t.kap[ck] * bar.f[PI][c];
  };
  if (j < d.ny && k < d.nz) {
    const float r = t.r0c[k] * t.dx_inv;
    float acc = 0.f;
    if (i >= 1) acc -= r * Z(i - 1, j, k);
    if (i < d.nx) acc += r * Z(i, j, k);
    bar.f[U][IX(i, j, k)] += dtau * acc;
  }
  if (i < d.nx && k < d.nz) {
    const float r = t.r0c[k] * t.dy_inv;
    float acc = 0.f;
    if (j >= 1) acc -= r * Z(i, j - 1, k);
    if (j < d.ny) acc += r * Z(i, j, k);
    bar.f[V][IX(i, j, k)] += dtau * acc;
  }
  if (i < d.nx && j < d.ny) {
    float acc = 0.f;
    if (k >= 1) acc -= t.rfz[k] * t.idzc[k - 1] * Z(i, j, k - 1);
    if (k < d.nz) acc += t.rfz[k] * t.idzc[k] * Z(i, j, k);
    bar.f[W][IX(i, j, k)] += dtau * acc;
  }
}

// adjoint of one standalone FP32 HEVI substep (the column kernel without a
// pending u/v update, then the in-place u/v update): the u/v gradient
// transposed, the column transposed (the steps of hevi2_body in reverse; the
// column system A = L U, with L = (la sub, 1/li diagonal) and U = (1, lc
// super), transposed as U^T z = bar_x forward and L^T y = z backward), and the
// horizontal divergence transposed
__global__ void k_mxad_hevi_column(Dims d, Tab t, Flags fl, const float* __restrict__ lu, WS bar,
                                   float* __restrict__ bdh, float* __restrict__ scratch, float dtau) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= d.nx || j >= d.ny) return;
  const int nz = d.nz;
  const float b = (float)fl.hevi_beta, ob = 1.f - b, cp = (float)kCp;
  const float* la = lu;
  const float* lc = lu + nz;
  const float* li = lu + 2 * nz;
  float* bw = bar.f[W];
  const float* brho = bar.f[RHO];
  float* bpi = bar.f[PI];
  const size_t col = (size_t)j * d.nx + i;
  float* ya = scratch + col * (4 * (size_t)nz + 2);  // nz
  float* bwn = ya + nz;                              // nz+1
  float* dvo = bwn + nz + 1;                         // nz
  float* dvt = dvo + nz;                             // nz
  auto rho_bar = [&](int k) { return brho[IX(i, j, k)]; };
  for (int k = 0; k <= nz; ++k) {  // wn: w_out and dv_new of the cells around face k
    float g = bw[IX(i, j, k)];
    if (k < nz) g += t.rfz[k] * t.idzc[k] * (dtau * b * rho_bar(k));
    if (k >= 1) g -= t.rfz[k] * t.idzc[k - 1] * (dtau * b * rho_bar(k - 1));
    bwn[k] = g;
  }
  for (int k = 0; k < nz; ++k) ya[k] = bpi[IX(i, j, k)];  // pi_out = x
  for (int k = 1; k < nz; ++k) {  // wn = wt - cb_k (x_k - x_{k-1})
    const float cb = dtau * b * cp * t.tfz[k] * t.idzw[k];
    ya[k] -= cb * bwn[k];
    ya[k - 1] += cb * bwn[k];
  }
  for (int k = 1; k < nz; ++k) ya[k] -= lc[k - 1] * ya[k - 1];           // U^T z = bar_x
  ya[nz - 1] *= li[nz - 1];                                              // L^T y = z
  for (int k = nz - 2; k >= 0; --k) ya[k] = (ya[k] - la[k + 1] * ya[k + 1]) * li[k];
  for (int k = 0; k < nz; ++k) {  // rhs = pi + dtau kappa (Dh + ob dv_old + b dv_t); rho += dtau (Dh + ob dv_old)
    const float kp = dtau * t.kap[k] * ya[k];
    bdh[IX(i, j, k)] = dtau * rho_bar(k) + kp;
    dvo[k] = dtau * ob * rho_bar(k) + ob * kp;
    dvt[k] = b * kp;
  }
  for (int k = 0; k <= nz; ++k) {  // bar_wt
    float g = bwn[k];
    if (k < nz) g += t.rfz[k] * t.idzc[k] * dvt[k];
    if (k >= 1) g -= t.rfz[k] * t.idzc[k - 1] * dvt[k - 1];
    bwn[k] = g;
  }
  for (int k = 0; k <= nz; ++k) {  // bar_w: wt's identity and dv_old
    float g = bwn[k];
    if (k < nz) g += t.rfz[k] * t.idzc[k] * dvo[k];
    if (k >= 1) g -= t.rfz[k] * t.idzc[k - 1] * dvo[k - 1];
    bw[IX(i, j, k)] = g;
  }
  for (int k = 0; k < nz; ++k) {  // bar_pi: rhs's pi and wt's gradient
    float g = ya[k];
    if (k >= 1) g -= dtau * ob * cp * t.tfz[k] * t.idzw[k] * bwn[k];
    if (k + 1 < nz) g += dtau * ob * cp * t.tfz[k + 1] * t.idzw[k + 1] * bwn[k + 1];
    bpi[IX(i, j, k)] = g;
  }
}

__global__ void k_mxad_dh(Dims d, Tab t, const float* __restrict__ bdh, WS bar) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i > d.nx || j > d.ny || k >= d.nz) return;
  if (j < d.ny) {
    const float r = t.r0c[k] * t.dx_inv;
    float acc = 0.f;
    if (i >= 1) acc -= r * bdh[IX(i - 1, j, k)];
    if (i < d.nx) acc += r * bdh[IX(i, j, k)];
    bar.f[U][IX(i, j, k)] += acc;
  }
  if (i < d.nx) {
    const float r = t.r0c[k] * t.dy_inv;
    float acc = 0.f;
    if (j >= 1) acc -= r * bdh[IX(i, j - 1, k)];
    if (j < d.ny) acc += r * bdh[IX(i, j, k)];
    bar.f[V][IX(i, j, k)] += acc;
  }
}

void mixed_hevi_substep_ad(const Dims& d, const Tab& t, const Flags& fl, const WS& bar, const float* lu, float* bdh,
                           float* scratch, float dtau, cudaStream_t stream) {
  const dim3 b(32, 4);
  k_mxad_pi<<<g3(d.nx, d.ny, d.nz, b), b, 0, stream>>>(d, t, bar, dtau, 0);
  k_mxad_hevi_column<<<dim3((d.nx + 31) / 32, (d.ny + 3) / 4), b, 0, stream>>>(d, t, fl, lu, bar, bdh, scratch,
                                                                                dtau);
  k_mxad_dh<<<g3(d.nx + 1, d.ny + 1, d.nz, b), b, 0, stream>>>(d, t, bdh, bar);
}

void mixed_fb_substep_ad(const Dims& d, const Tab& t, const WS& bar, float dtau, cudaStream_t stream) {
  const dim3 b(32, 4);
  k_mxad_pi<<<g3(d.nx, d.ny, d.nz, b), b, 0, stream>>>(d, t, bar, dtau, 1);
  k_mxad_vel<<<g3(d.nx + 1, d.ny + 1, d.nz + 1, b), b, 0, stream>>>(d, t, bar, dtau);
}

void mixed_fb_substep(const Dims& d, const Tab& t, const Flags& fl, const WS& win, const WS& wout, float dtau,
                      cudaStream_t stream) {
  const dim3 b(32, 4);
  k_mx_fb_mass<<<g3(d.nx, d.ny, d.nz, b), b, 0, stream>>>(d, t, win, wout, dtau);
  k_mx_fb_mom<<<g3(d.nx + 1, d.ny + 1, d.nz + 1, b), b, 0, stream>>>(d, t, win, wout, dtau, 1);
}

__device__ __forceinline__ void cp_async8(float* smem, const float* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem) : "memory");
}

// ---- the HEVI column update for two adjacent columns per thread ----------
// Same arithmetic per column and level as hevi_body; a thread owns columns i
// and i+1 (i even, so every row access is one aligned 8-byte load or store of
// both columns) and carries two independent recurrences. Forward loads go
// through a kRing-deep cp.async ring (8-byte copies for the row pairs, 4-byte
// for the three single neighbours); the backward sweep reads the parked data
// (L2) four levels ahead in registers. With nx odd, the last thread of a row
// computes a second, ghost column (i + 1 = nx) from in-bounds ghost-line data
// and stores nothing of it.
template <int kRing>
__device__ __forceinline__ void hevi2_body(const Dims& d, const Tab& t, const Flags& fl, const WS& win,
                                           const WS& wout, float dtau, const float* __restrict__ lu, int apply_uv,
                                           float cdx, float cdy, int bx, int by) {
  extern __shared__ float s_tab[];
  const int nz = d.nz;
  float* s_tfz = s_tab;                    // nz+1
  float* s_idzw = s_tfz + (nz + 1);        // nz+1
  float* s_rfz = s_idzw + (nz + 1);        // nz+1
  float* s_idzc = s_rfz + (nz + 1);        // nz
  float* s_kap = s_idzc + nz;              // nz
  float* s_la = s_kap + nz;                // nz
  float* s_lc = s_la + nz;                 // nz
  float* s_li = s_lc + nz;                 // nz
  float* s_r0 = s_li + nz;                 // nz
  float* s_t0 = s_r0 + nz;                 // nz
  const int tid = threadIdx.y * blockDim.x + threadIdx.x;
  for (int e = tid; e <= nz; e += 128) {
    s_tfz[e] = t.tfz[e];
    s_idzw[e] = t.idzw[e];
    s_rfz[e] = t.rfz[e];
    if (e < nz) {
      s_idzc[e] = t.idzc[e];
      s_kap[e] = t.kap[e];
      s_la[e] = lu[e];
      s_lc[e] = lu[nz + e];
      s_li[e] = lu[2 * nz + e];
      s_r0[e] = t.r0c[e];
      s_t0[e] = t.t0c[e];
    }
  }
  __syncthreads();
  const int i = 2 * (bx * blockDim.x + threadIdx.x);
  const int j = by * blockDim.y + threadIdx.y;
  if (i >= d.nx || j >= d.ny) return;
  const bool two = i + 1 < d.nx;
  const float b = (float)fl.hevi_beta, ob = 1.f - b;
  const float cpf = (float)kCp;
  const size_t col = (size_t)j * d.P + i;
  const size_t pl = d.plane;
  const float* __restrict__ U0 = win.f[U] + col;
  const float* __restrict__ V0 = win.f[V] + col;
  const float* __restrict__ W0 = win.f[W] + col;
  const float* __restrict__ P0 = win.f[PI] + col;
  const float* __restrict__ R0 = win.f[RHO] + col;
  float* __restrict__ Wo = wout.f[W] + col;
  float* __restrict__ Po = wout.f[PI] + col;
  float* __restrict__ Ro = wout.f[RHO] + col;
  float* __restrict__ Uo = wout.f[U] + col;
  float* __restrict__ Vo = wout.f[V] + col;
  const size_t vn = d.P;
  const float dxi = t.dx_inv, dyi = t.dy_inv;
  // single neighbours: u(i+2) (u(i+1) when i+1 is the last face), pi'(i-1)
  // (clamped to i), pi'(i+2) (clamped to the last column); row pairs j-1, j+1
  // clamped to j
  const int ou2 = two ? 2 : 1;
  const int opw = (i > 0) ? -1 : 0;
  const int ope = (i + 2 < d.nx) ? 2 : (two ? 1 : 0);
  const long long os = (j > 0) ? -(long long)vn : 0, on = (j + 1 < d.ny) ? (long long)vn : 0;
  const bool last_j = (j == d.ny - 1);
  auto st2 = [&](float* p, float a, float c) {
    if (two) *reinterpret_cast<float2*>(p) = make_float2(a, c);
    else *p = a;
  };
  // ring: per slot 8 float2 fields (w, pi', u(i..i+1), v(j), v(j+1), rho',
  // pi'(j-1), pi'(j+1)) then 3 float fields (u(i+2), pi'(i-1), pi'(i+2))
  float* ring = s_tab + ((10 * (size_t)(nz + 1) + 3) & ~(size_t)3);
  auto r2 = [&](int slot, int f) -> float* { return ring + ((size_t)slot * 19 * 128) + ((size_t)f * 128 + tid) * 2; };
  auto r1 = [&](int slot, int f) -> float* {
    return ring + ((size_t)slot * 19 * 128) + 16 * 128 + (size_t)f * 128 + tid;
  };
  auto issue = [&](int L) {
    const int slot = L % kRing;
    const size_t o = (size_t)L * pl, o1 = o + pl;
    cp_async8(r2(slot, 0), W0 + o1);
    if (L + 1 < nz) cp_async8(r2(slot, 1), P0 + o1);
    else { r2(slot, 1)[0] = 0.f; r2(slot, 1)[1] = 0.f; }
    cp_async8(r2(slot, 2), U0 + o);
    cp_async8(r2(slot, 3), V0 + o);
    cp_async8(r2(slot, 4), V0 + o + vn);
    cp_async8(r2(slot, 5), R0 + o);
    cp_async4(r1(slot, 0), U0 + o + ou2);
    if (apply_uv) {
      cp_async8(r2(slot, 6), P0 + o + os);
      cp_async8(r2(slot, 7), P0 + o + on);
      cp_async4(r1(slot, 1), P0 + o + opw);
      cp_async4(r1(slot, 2), P0 + o + ope);
    }
  };
  for (int L = 0; L < kRing; ++L) {
    if (L < nz) issue(L);
    cp_async_commit();
  }
  float pk[2], wk[2], wtk[2], dpp[2] = {0.f, 0.f};
  {
    const float2 p0 = *reinterpret_cast<const float2*>(P0);
    const float2 w0 = *reinterpret_cast<const float2*>(W0);
    pk[0] = p0.x; pk[1] = p0.y;
    wk[0] = w0.x; wk[1] = w0.y;
    wtk[0] = wk[0]; wtk[1] = wk[1];  // face 0: no pressure gradient
    st2(Wo, wk[0], wk[1]);
  }
  for (int k = 0; k < nz; ++k) {
    cp_async_wait<kRing - 1>();
    const int slot = k % kRing;
    const float2 fw = *reinterpret_cast<const float2*>(r2(slot, 0));
    const float2 fp = *reinterpret_cast<const float2*>(r2(slot, 1));
    const float2 fu = *reinterpret_cast<const float2*>(r2(slot, 2));
    const float2 fv0 = *reinterpret_cast<const float2*>(r2(slot, 3));
    const float2 fv1 = *reinterpret_cast<const float2*>(r2(slot, 4));
    const float2 fr = *reinterpret_cast<const float2*>(r2(slot, 5));
    const float fu2 = *r1(slot, 0);
    float u0[2] = {fu.x, fu.y}, u1[2] = {fu.y, fu2};
    float v0[2] = {fv0.x, fv0.y}, v1[2] = {fv1.x, fv1.y};
    if (apply_uv) {
      const float2 fs = *reinterpret_cast<const float2*>(r2(slot, 6));
      const float2 fn = *reinterpret_cast<const float2*>(r2(slot, 7));
      const float fpw = *r1(slot, 1), fpe = *r1(slot, 2);
      const float tx_ = s_t0[k] * cdx, ty_ = s_t0[k] * cdy;
      // column i: west pi'(i-1), east pi'(i+1) (itself at the last column);
      // column i+1: west pi'(i), east pi'(i+2)
      const float peA = two ? pk[1] : pk[0];
      u0[0] += tx_ * (pk[0] - fpw);
      u1[0] += tx_ * (peA - pk[0]);
      u0[1] += tx_ * (pk[1] - pk[0]);
      u1[1] += tx_ * (fpe - pk[1]);
      v0[0] += ty_ * (pk[0] - fs.x);
      v1[0] += ty_ * (fn.x - pk[0]);
      v0[1] += ty_ * (pk[1] - fs.y);
      v1[1] += ty_ * (fn.y - pk[1]);
    }
    const size_t o = (size_t)k * pl;
    st2(Uo + o, u0[0], u0[1]);
    st2(Vo + o, v0[0], v0[1]);
    if (two) {
      if (i + 1 == d.nx - 1) Uo[o + 2] = u1[1];  // face nx
    } else {
      Uo[o + 1] = u1[0];
    }
    if (last_j) st2(Vo + o + vn, v1[0], v1[1]);
    const float wk1[2] = {fw.x, fw.y}, pk1in[2] = {fp.x, fp.y}, r0v[2] = {fr.x, fr.y};
    const float rk = s_rfz[k], rk1 = s_rfz[k + 1], idz = s_idzc[k];
    float dpk[2], rsv[2], wtk1[2], pk1[2];
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      wtk1[c] = wk1[c];
      pk1[c] = 0.f;
      if (k + 1 < nz) {
        pk1[c] = pk1in[c];
        wtk1[c] = wk1[c] - dtau * ob * cpf * s_tfz[k + 1] * (pk1[c] - pk[c]) * s_idzw[k + 1];
      }
      const float Dh = -(s_r0[k] * ((u1[c] - u0[c]) * dxi + (v1[c] - v0[c]) * dyi));
      const float dv_old = -(rk1 * wk1[c] - rk * wk[c]) * idz;
      const float dv_t = -(rk1 * wtk1[c] - rk * wtk[c]) * idz;
      const float S = Dh + ob * dv_old;
      const float rhs = pk[c] + dtau * s_kap[k] * (S + b * dv_t);
      dpk[c] = (k == 0) ? rhs * s_li[0] : (rhs - s_la[k] * dpp[c]) * s_li[k];
      rsv[c] = r0v[c] + dtau * S;
    }
    st2(Po + o, dpk[0], dpk[1]);
    st2(Ro + o, rsv[0], rsv[1]);
    st2(Wo + o + pl, wtk1[0], wtk1[1]);
    if (k + kRing < nz) issue(k + kRing);
    cp_async_commit();
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      dpp[c] = dpk[c];
      wk[c] = wk1[c];
      wtk[c] = wtk1[c];
      pk[c] = pk1[c];
    }
  }
  cp_async_wait<0>();
  // backward sweep (as hevi_body), both columns
  constexpr int kB = 4;
  float2 bdp[kB], bwt[kB], bS[kB];
  auto ld2 = [&](const float* p) -> float2 {
    if (two) return *reinterpret_cast<const float2*>(p);
    return make_float2(*p, 0.f);
  };
  auto loadB = [&](int kk, int q) {
    const size_t o = (size_t)kk * pl;
    bdp[q] = (kk >= 1) ? ld2(Po + o - pl) : make_float2(0.f, 0.f);
    bwt[q] = ld2(Wo + o);
    bS[q] = ld2(Ro + o);
  };
#pragma unroll
  for (int q = 0; q < kB; ++q)
    if (nz - 1 - q >= 0) loadB(nz - 1 - q, q);
  float xu[2] = {dpp[0], dpp[1]};
  float wu[2];
  {
    const float2 t2 = ld2(Wo + (size_t)nz * pl);
    wu[0] = t2.x;
    wu[1] = t2.y;
  }
  for (int kk0 = nz - 1; kk0 >= 0; kk0 -= kB) {
#pragma unroll
    for (int q = 0; q < kB; ++q) {
      const int kk = kk0 - q;
      if (kk >= 0) {
        const int k = kk - 1;
        const size_t okk = (size_t)kk * pl;
        const float bd[2] = {bdp[q].x, bdp[q].y}, bw[2] = {bwt[q].x, bwt[q].y}, bs[2] = {bS[q].x, bS[q].y};
        float xk[2], wkk[2], rn[2];
#pragma unroll
        for (int c = 0; c < 2; ++c) {
          xk[c] = 0.f;
          wkk[c] = bw[c];
          if (k >= 0) {
            xk[c] = bd[c] - s_lc[k] * xu[c];
            wkk[c] = bw[c] - dtau * b * cpf * s_tfz[kk] * (xu[c] - xk[c]) * s_idzw[kk];
          }
          const float dv_new = -(s_rfz[kk + 1] * wu[c] - s_rfz[kk] * wkk[c]) * s_idzc[kk];
          rn[c] = bs[c] + dtau * b * dv_new;
        }
        if (kk - kB >= 0) loadB(kk - kB, q);
        st2(Ro + okk, rn[0], rn[1]);
        st2(Po + okk, xu[0], xu[1]);
        st2(Wo + okk, wkk[0], wkk[1]);
#pragma unroll
        for (int c = 0; c < 2; ++c) {
          xu[c] = xk[c];
          wu[c] = wkk[c];
        }
      }
    }
  }
}

template <int kRing>
__global__ void __launch_bounds__(128, 7) k_mx_hevi_col2(const __grid_constant__ Dims d, const __grid_constant__ Tab t,
                                                          const __grid_constant__ Flags fl,
                                                          const __grid_constant__ WS win,
                                                          const __grid_constant__ WS wout, float dtau,
                                                          const float* __restrict__ lu, int apply_uv, float cdx,
                                                          float cdy) {
  hevi2_body<kRing>(d, t, fl, win, wout, dtau, lu, apply_uv, cdx, cdy, blockIdx.x, blockIdx.y);
}

// ---- the two-column HEVI update fed by TMA -------------------------------
// Same arithmetic per column and level as hevi2_body. The forward sweep's
// loads of a level (w and pi' of the level above, u, v, rho' and the pi'
// neighbours of the level) are five TMA boxes per block issued by one thread
// into a kColRing-deep ring of level slots tracked by mbarriers, instead of
// eleven per-thread cp.async copies; threads read their points from the
// boxes. At iteration k a thread needs the slots of levels k and k+1; after
// the block barrier of iteration k the slot of level k-1 is free and receives
// level k-1+kColRing. Neighbours outside the domain are never read: the
// clamped neighbour offsets of hevi2_body select in-range box points. Waits
// are bounded; a box that does not arrive sets kErrWaitTimeout, and the block
// waits (bounded) for its copies in flight before it returns.
// kDefer: the HEVI backward sweep updates pi' alone. w and rho' leave the
// kernel as their explicit parts w~ (= wt) and rho~ (= rho' + dtau S), and
// every reader applies the implicit corrections from the final pi' itself
// (defer_fix_w / defer_fix_rho). This kernel applies them to its own input
// when apply_uv is set (its input is then a deferred substep's output); the
// fix-up kernel after a stage's last substep (k_mx_fix) and the finish
// kernel apply them to the last one. The parked sweep data shrinks from
// w~, rho~ and the eliminated pi' to the eliminated pi' alone: 48 instead of
// 64 bytes of traffic per cell and substep.
template <bool kDefer>
__device__ __forceinline__ void hevi_tma_body(const Dims& d, const Tab& t, const Flags& fl, const ColumnMaps& C,
                                              const WS& win, const WS& wout, float dtau, const float* __restrict__ lu,
                                              int apply_uv, float cdx, float cdy, unsigned* err, int bx, int by) {
  extern __shared__ float s_dyn[];
  __shared__ __align__(8) unsigned long long bar[kColRing], bbar[kColRing];
  const int nz = d.nz;
  const unsigned sa = (unsigned)__cvta_generic_to_shared(s_dyn);
  float* ring = s_dyn + ((((sa + 127u) & ~127u) - sa) >> 2);
  float* s_tfz = ring + (size_t)kColRing * kColSlot;  // nz+1
  float* s_idzw = s_tfz + (nz + 1);                   // nz+1
  float* s_rfz = s_idzw + (nz + 1);                   // nz+1
  float* s_idzc = s_rfz + (nz + 1);                   // nz
  float* s_kap = s_idzc + nz;                         // nz
  float* s_la = s_kap + nz;                           // nz
  float* s_lc = s_la + nz;                            // nz
  float* s_li = s_lc + nz;                            // nz
  float* s_r0 = s_li + nz;                            // nz
  float* s_t0 = s_r0 + nz;                            // nz
  const int tid = threadIdx.y * blockDim.x + threadIdx.x;
  const int i0 = bx * 64, j0 = by * 4;
  auto issue = [&](int L) {  // one thread: level L (0..nz) into its slot
    float* s = ring + (size_t)(L % kColRing) * kColSlot;
    unsigned long long* b = &bar[L % kColRing];
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_expect_tx(b, kColLevelBytes);
    tma_load_3d(s + kOffW, &C.m[0], i0 - CX, j0, L, b);
    tma_load_3d(s + kOffP, &C.m[1], i0 - CX, j0 - 1, L, b);
    tma_load_3d(s + kOffU, &C.m[2], i0 - CX, j0, L, b);
    tma_load_3d(s + kOffV, &C.m[3], i0 - CX, j0, L, b);
    tma_load_3d(s + kOffR, &C.m[4], i0 - CX, j0, L, b);
  };
  if (tid == 0) {
    for (int s = 0; s < kColRing; ++s) {
      mbar_init(&bar[s], 1);
      mbar_init(&bbar[s], 1);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    for (int L = 0; L < kColRing && L <= nz; ++L) issue(L);
  }
  for (int e = tid; e <= nz; e += 128) {
    s_tfz[e] = t.tfz[e];
    s_idzw[e] = t.idzw[e];
    s_rfz[e] = t.rfz[e];
    if (e < nz) {
      s_idzc[e] = t.idzc[e];
      s_kap[e] = t.kap[e];
      s_la[e] = lu[e];
      s_lc[e] = lu[nz + e];
      s_li[e] = lu[2 * nz + e];
      s_r0[e] = t.r0c[e];
      s_t0[e] = t.t0c[e];
    }
  }
  __syncthreads();
  // bounded wait for level L by every thread; on a timeout thread 0 drains
  // the copies still in flight (levels L..hi) and the block returns
  int hi = imin(kColRing - 1, nz);  // highest level issued
  auto level_ready = [&](int L) -> bool {
    const bool ok = (tid != 0) || mbar_wait_bounded(&bar[L % kColRing], (unsigned)(L / kColRing) & 1u);
    if (__syncthreads_or(!ok)) {
      if (tid == 0) {
        atomicOr(err, (unsigned)kErrWaitTimeout);
        for (int l = L; l <= hi; ++l) mbar_wait_bounded(&bar[l % kColRing], (unsigned)(l / kColRing) & 1u);
      }
      return false;
    }
    return true;
  };
  const int i = i0 + 2 * threadIdx.x;
  const int j = j0 + threadIdx.y;
  const bool active = i < d.nx && j < d.ny;
  const bool two = i + 1 < d.nx;
  const float b = (float)fl.hevi_beta, ob = 1.f - b;
  const float cpf = (float)kCp;
  const size_t col = (size_t)imin(j, d.ny - 1) * d.P + imin(i, d.nx - 1);
  const size_t pl = d.plane;
  float* __restrict__ Wo = wout.f[W] + col;
  float* __restrict__ Po = wout.f[PI] + col;
  float* __restrict__ Ro = wout.f[RHO] + col;
  float* __restrict__ Uo = wout.f[U] + col;
  float* __restrict__ Vo = wout.f[V] + col;
  const size_t vn = d.P;
  const float dxi = t.dx_inv, dyi = t.dy_inv;
  // box-local offsets of the own points (row r, column c = CX + 2 tx)
  const int c0 = CX + 2 * threadIdx.x, r = threadIdx.y;
  const int oW = kOffW + r * CW + c0, oU = kOffU + r * CW + c0, oV = kOffV + r * CW + c0;
  const int oR = kOffR + r * CW + c0, oP = kOffP + (r + 1) * CW + c0;
  const int ou2 = two ? 2 : 1;
  const int opw = (i > 0) ? -1 : 0;
  const int ope = (i + 2 < d.nx) ? 2 : (two ? 1 : 0);
  const int ops = (j > 0) ? -CW : 0, opn = (j + 1 < d.ny) ? CW : 0;
  const bool last_j = (j == d.ny - 1);
  auto st2 = [&](float* p, float a, float c) {
    if (two) *reinterpret_cast<float2*>(p) = make_float2(a, c);
    else *p = a;
  };
  // L2 policies: the outputs stream out (the next substep reads them a whole
  // launch later), the parked pi' of the forward sweep is read back by this
  // block's backward sweep
  unsigned long long pol_first, pol_last;
  asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol_first));
  asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol_last));
  auto st2p = [&](float* p, float a, float c, unsigned long long pol) {
    if (two)
      asm volatile("st.global.L2::cache_hint.v2.f32 [%0], {%1, %2}, %3;" ::"l"(p), "f"(a), "f"(c), "l"(pol) : "memory");
    else
      asm volatile("st.global.L2::cache_hint.f32 [%0], %1, %2;" ::"l"(p), "f"(a), "l"(pol) : "memory");
  };
  if (!level_ready(0)) return;
  float pk[2], wk[2], wtk[2], dpp[2] = {0.f, 0.f};
  {
    const float2 p0 = *reinterpret_cast<const float2*>(ring + oP);
    const float2 w0 = *reinterpret_cast<const float2*>(ring + oW);
    pk[0] = p0.x; pk[1] = p0.y;
    wk[0] = w0.x; wk[1] = w0.y;
    wtk[0] = wk[0]; wtk[1] = wk[1];  // face 0: no pressure gradient
    if (active) st2(Wo, wk[0], wk[1]);
  }
  for (int k = 0; k < nz; ++k) {
    if (!level_ready(k + 1)) return;  // also: every thread is done with level k-1's slot
    if (tid == 0 && k >= 1 && k - 1 + kColRing <= nz) {
      issue(k - 1 + kColRing);
      hi = k - 1 + kColRing;
    }
    const float* s0 = ring + (size_t)(k % kColRing) * kColSlot;
    const float* s1 = ring + (size_t)((k + 1) % kColRing) * kColSlot;
    const float2 fw = *reinterpret_cast<const float2*>(s1 + oW);
    const float2 fp = *reinterpret_cast<const float2*>(s1 + oP);
    const float2 fu = *reinterpret_cast<const float2*>(s0 + oU);
    const float2 fv0 = *reinterpret_cast<const float2*>(s0 + oV);
    const float2 fv1 = *reinterpret_cast<const float2*>(s0 + oV + CW);
    const float2 fr = *reinterpret_cast<const float2*>(s0 + oR);
    const float fu2 = s0[oU + ou2];
    float u0[2] = {fu.x, fu.y}, u1[2] = {fu.y, fu2};
    float v0[2] = {fv0.x, fv0.y}, v1[2] = {fv1.x, fv1.y};
    if (apply_uv) {
      const float2 fs = *reinterpret_cast<const float2*>(s0 + oP + ops);
      const float2 fn = *reinterpret_cast<const float2*>(s0 + oP + opn);
      const float fpw = s0[oP + opw], fpe = s0[oP + ope];
      const float tx_ = s_t0[k] * cdx, ty_ = s_t0[k] * cdy;
      const float peA = two ? pk[1] : pk[0];
      u0[0] += tx_ * (pk[0] - fpw);
      u1[0] += tx_ * (peA - pk[0]);
      u0[1] += tx_ * (pk[1] - pk[0]);
      u1[1] += tx_ * (fpe - pk[1]);
      v0[0] += ty_ * (pk[0] - fs.x);
      v1[0] += ty_ * (fn.x - pk[0]);
      v0[1] += ty_ * (pk[1] - fs.y);
      v1[1] += ty_ * (fn.y - pk[1]);
    }
    const size_t o = (size_t)k * pl;
    float wk1[2] = {fw.x, fw.y}, r0v[2] = {fr.x, fr.y};
    const float pk1in[2] = {fp.x, fp.y};
    const float rk = s_rfz[k], rk1 = s_rfz[k + 1], idz = s_idzc[k];
    if (kDefer && apply_uv) {  // the input's deferred corrections (wk: corrected last iteration)
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        if (k + 1 < nz) wk1[c] = wk1[c] - dtau * b * cpf * s_tfz[k + 1] * (pk1in[c] - pk[c]) * s_idzw[k + 1];
        r0v[c] = r0v[c] + dtau * b * (-(rk1 * wk1[c] - rk * wk[c]) * idz);
      }
    }
    float dpk[2], rsv[2], wtk1[2], pk1[2];
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      wtk1[c] = wk1[c];
      pk1[c] = 0.f;
      if (k + 1 < nz) {
        pk1[c] = pk1in[c];
        wtk1[c] = wk1[c] - dtau * ob * cpf * s_tfz[k + 1] * (pk1[c] - pk[c]) * s_idzw[k + 1];
      }
      const float Dh = -(s_r0[k] * ((u1[c] - u0[c]) * dxi + (v1[c] - v0[c]) * dyi));
      const float dv_old = -(rk1 * wk1[c] - rk * wk[c]) * idz;
      const float dv_t = -(rk1 * wtk1[c] - rk * wtk[c]) * idz;
      const float S = Dh + ob * dv_old;
      const float rhs = pk[c] + dtau * s_kap[k] * (S + b * dv_t);
      dpk[c] = (k == 0) ? rhs * s_li[0] : (rhs - s_la[k] * dpp[c]) * s_li[k];
      rsv[c] = r0v[c] + dtau * S;
    }
    if (active) {
      st2p(Uo + o, u0[0], u0[1], pol_first);
      st2p(Vo + o, v0[0], v0[1], pol_first);
      if (two) {
        if (i + 1 == d.nx - 1) Uo[o + 2] = u1[1];  // face nx
      } else {
        Uo[o + 1] = u1[0];
      }
      if (last_j) st2(Vo + o + vn, v1[0], v1[1]);
      st2p(Po + o, dpk[0], dpk[1], pol_last);
      st2p(Ro + o, rsv[0], rsv[1], pol_first);
      st2p(Wo + o + pl, wtk1[0], wtk1[1], pol_first);
    }
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      dpp[c] = dpk[c];
      wk[c] = wk1[c];
      wtk[c] = wtk1[c];
      pk[c] = pk1[c];
    }
  }
  // backward sweep (as hevi2_body), the parked data of the block's columns
  // brought back by TMA: every thread's forward stores are made visible to
  // the async proxy before thread 0 issues the first box
  asm volatile("fence.proxy.async.global;" ::: "memory");
  __syncthreads();
  auto issue_b = [&](int n) {  // backward level n: face kk = nz-1-n (w, rho') and pi'(kk-1)
    const int kk = nz - 1 - n;
    float* s = ring + (size_t)(n % kColRing) * kColSlot;
    unsigned long long* bb = &bbar[n % kColRing];
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_expect_tx(bb, kDefer ? kBackLevelBytes / 3 : kBackLevelBytes);
    if (!kDefer) {
      tma_load_3d(s + kBOffW, &C.back[0], i0, j0, kk, bb);
      tma_load_3d(s + kBOffR, &C.back[1], i0, j0, kk, bb);
    }
    tma_load_3d(s + kBOffP, &C.back[2], i0, j0, imax(kk - 1, 0), bb);
  };
  int bhi = imin(kColRing, nz) - 1;
  if (tid == 0)
    for (int n = 0; n <= bhi; ++n) issue_b(n);
  auto back_ready = [&](int n) -> bool {
    const bool ok = (tid != 0) || mbar_wait_bounded(&bbar[n % kColRing], (unsigned)(n / kColRing) & 1u);
    if (__syncthreads_or(!ok)) {
      if (tid == 0) {
        atomicOr(err, (unsigned)kErrWaitTimeout);
        for (int l = n; l <= bhi; ++l) mbar_wait_bounded(&bbar[l % kColRing], (unsigned)(l / kColRing) & 1u);
      }
      return false;
    }
    return true;
  };
  const int obk = threadIdx.y * BW + 2 * threadIdx.x;
  float xu[2] = {dpp[0], dpp[1]};
  float wu[2] = {0.f, 0.f};
  if (!kDefer && active) {
    wu[0] = Wo[(size_t)nz * pl];
    if (two) wu[1] = Wo[(size_t)nz * pl + 1];
  }
  for (int n = 0; n < nz; ++n) {
    if (!back_ready(n)) return;  // also: every thread is done with level n-1's slot
    if (tid == 0 && n >= 1 && n - 1 + kColRing < nz) {
      issue_b(n - 1 + kColRing);
      bhi = n - 1 + kColRing;
    }
    const float* sb = ring + (size_t)(n % kColRing) * kColSlot;
    const int kk = nz - 1 - n, k = kk - 1;
    const float2 fd = *reinterpret_cast<const float2*>(sb + kBOffP + obk);
    if (kDefer) {
      float xk[2];
#pragma unroll
      for (int c = 0; c < 2; ++c) xk[c] = (k >= 0) ? (c == 0 ? fd.x : fd.y) - s_lc[k] * xu[c] : 0.f;
      if (active) st2p(Po + (size_t)kk * pl, xu[0], xu[1], pol_first);
      xu[0] = xk[0];
      xu[1] = xk[1];
      continue;
    }
    const float2 fw = *reinterpret_cast<const float2*>(sb + kBOffW + obk);
    const float2 fs = *reinterpret_cast<const float2*>(sb + kBOffR + obk);
    const float bd[2] = {fd.x, fd.y}, bw[2] = {fw.x, fw.y}, bs[2] = {fs.x, fs.y};
    float xk[2], wkk[2], rn[2];
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      xk[c] = 0.f;
      wkk[c] = bw[c];
      if (k >= 0) {
        xk[c] = bd[c] - s_lc[k] * xu[c];
        wkk[c] = bw[c] - dtau * b * cpf * s_tfz[kk] * (xu[c] - xk[c]) * s_idzw[kk];
      }
      const float dv_new = -(s_rfz[kk + 1] * wu[c] - s_rfz[kk] * wkk[c]) * s_idzc[kk];
      rn[c] = bs[c] + dtau * b * dv_new;
    }
    if (active) {
      const size_t okk = (size_t)kk * pl;
      st2(Ro + okk, rn[0], rn[1]);
      st2(Po + okk, xu[0], xu[1]);
      st2(Wo + okk, wkk[0], wkk[1]);
    }
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      xu[c] = xk[c];
      wu[c] = wkk[c];
    }
  }
}

__global__ void __launch_bounds__(128, 7) k_mx_hevi_tma(const __grid_constant__ Dims d, const __grid_constant__ Tab t,
                                                         const __grid_constant__ Flags fl,
                                                         const __grid_constant__ ColumnMaps C,
                                                         const __grid_constant__ WS win,
                                                         const __grid_constant__ WS wout, float dtau,
                                                         const float* __restrict__ lu, int apply_uv, float cdx,
                                                         float cdy, unsigned* err) {
  hevi_tma_body<false>(d, t, fl, C, win, wout, dtau, lu, apply_uv, cdx, cdy, err, blockIdx.x, blockIdx.y);
}
__global__ void __launch_bounds__(128, 7) k_mx_hevi_tmad(const __grid_constant__ Dims d, const __grid_constant__ Tab t,
                                                          const __grid_constant__ Flags fl,
                                                          const __grid_constant__ ColumnMaps C,
                                                          const __grid_constant__ WS win,
                                                          const __grid_constant__ WS wout, float dtau,
                                                          const float* __restrict__ lu, int apply_uv, float cdx,
                                                          float cdy, unsigned* err) {
  hevi_tma_body<true>(d, t, fl, C, win, wout, dtau, lu, apply_uv, cdx, cdy, err, blockIdx.x, blockIdx.y);
}

// After a stage's last substep of the kDefer column kernel: its u/v backward
// update (as fb_mom_body) and the w/rho' corrections, in place, in one
// launch: a thread owns a column position of the (nx+1) x (ny+1) face grid
// and marches up the levels, reading w~(k+1) (and correcting it) before it
// writes w(k+1), so no other thread's read races a write (pi' itself is not
// changed; the u/v updates read it across columns).
// Each thread marches two column positions, blockDim.x apart in i (so each
// load instruction stays coalesced), as two independent chains: half the
// threads, all resident at once at 512 x 512, twice the loads in flight each.
constexpr int kFixPos = 2;
__device__ __forceinline__ void fix_body(const Dims& d, const Tab& t, const Flags& fl, const WS& s, float dtau,
                                         int bx, int by) {
  const int i0 = bx * blockDim.x * kFixPos + threadIdx.x;
  const int j = by * blockDim.y + threadIdx.y;
  if (i0 > d.nx || j > d.ny) return;
  const int nz = d.nz;
  const float* __restrict__ pn = s.f[PI];
  float* __restrict__ su = s.f[U];
  float* __restrict__ sv = s.f[V];
  float* __restrict__ sw = s.f[W];
  float* __restrict__ sr = s.f[RHO];
  const float cp = (float)kCp, b = (float)fl.hevi_beta, cb = dtau * b * cp, db = dtau * b;
  const unsigned pl = (unsigned)d.plane, P = (unsigned)d.P;
  // per position (indices clamped into the grid; each is used only where it
  // is in range; 32-bit offsets: a field has < 2^32 elements, checked when
  // the model is made)
  bool du[kFixPos], dv[kFixPos], cell[kFixPos];
  unsigned cf[kFixPos], ue[kFixPos], uw[kFixPos], vn[kFixPos], vs[kFixPos], cc[kFixPos];
#pragma unroll
  for (int c = 0; c < kFixPos; ++c) {
    const int i = i0 + c * (int)blockDim.x;
    const bool in = i <= d.nx;
    du[c] = in && j < d.ny;
    dv[c] = in && i < d.nx;
    cell[c] = du[c] && dv[c];
    const int ii = imin(i, d.nx);
    const int ic = imin(ii, d.nx - 1), jc = imin(j, d.ny - 1);
    const int ip = ic, im = imax(ii - 1, 0), jp = jc, jm = imax(j - 1, 0);
    cf[c] = j * P + ii;                            // u face (j < ny), v face (i < nx)
    ue[c] = jc * P + ip, uw[c] = jc * P + im;      // pi' beside the u face
    vn[c] = jp * P + ic, vs[c] = jm * P + ic;      // pi' beside the v face
    cc[c] = jc * P + ic;                           // the cell (i, j) when cell
  }
  // a level's inputs, loaded one level ahead so that their latency overlaps
  // the level below's arithmetic and stores
  struct Lv {
    float uc, ue, uw, vc, vn, vs, rc, wn, pn;
  };
  auto load = [&](int k, int c) {
    const unsigned o = (unsigned)k * pl;
    Lv L = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (du[c]) {
      L.uc = su[cf[c] + o];
      L.ue = pn[ue[c] + o];
      L.uw = pn[uw[c] + o];
    }
    if (dv[c]) {
      L.vc = sv[cf[c] + o];
      L.vn = pn[vn[c] + o];
      L.vs = pn[vs[c] + o];
    }
    if (cell[c]) {
      L.rc = sr[cc[c] + o];
      L.wn = sw[cc[c] + o + pl];                     // w~(k+1) (w has nz+1 faces)
      if (k + 1 < nz) L.pn = pn[cc[c] + o + pl];     // pi'(k+1)
    }
    return L;
  };
  float pk[kFixPos], wk[kFixPos];  // pi'(k), w(k) (w(0) = w~(0))
  Lv cur[kFixPos];
#pragma unroll
  for (int c = 0; c < kFixPos; ++c) {
    pk[c] = cell[c] ? pn[cc[c]] : 0.f;
    wk[c] = cell[c] ? sw[cc[c]] : 0.f;
    cur[c] = load(0, c);
  }
  for (int k = 0; k < nz; ++k) {
    Lv nxt[kFixPos];
#pragma unroll
    for (int c = 0; c < kFixPos; ++c) nxt[c] = (k + 1 < nz) ? load(k + 1, c) : cur[c];
    const unsigned o = (unsigned)k * pl;
#pragma unroll
    for (int c = 0; c < kFixPos; ++c) {
      if (du[c]) su[cf[c] + o] = cur[c].uc + dtau * (-cp * t.t0c[k] * (cur[c].ue - cur[c].uw) * t.dx_inv);
      if (dv[c]) sv[cf[c] + o] = cur[c].vc + dtau * (-cp * t.t0c[k] * (cur[c].vn - cur[c].vs) * t.dy_inv);
      if (cell[c]) {
        const unsigned q = cc[c] + o;
        const float pk1 = cur[c].pn;
        const float wk1 = defer_fix_w(t, nz, cb, cur[c].wn, pk1, pk[c], k + 1);
        sr[q] = defer_fix_rho(t, db, cur[c].rc, wk[c], wk1, k);
        if (k >= 1) sw[q] = wk[c];  // faces 1 .. nz-1 (w(0) and w(nz) keep w~)
        wk[c] = wk1;
        pk[c] = pk1;
      }
      cur[c] = nxt[c];
    }
  }
}
__global__ void __launch_bounds__(128, 8) k_mx_fix(const __grid_constant__ Dims d, const __grid_constant__ Tab t,
                         const __grid_constant__ Flags fl, const __grid_constant__ WS s, float dtau) {
  fix_body(d, t, fl, s, dtau, blockIdx.x, blockIdx.y);
}

size_t hevi_tma_smem_bytes(int nz) {
  return 128 + ((size_t)kColRing * kColSlot + 10 * (size_t)(nz + 1)) * sizeof(float);
}

// ---- the same HEVI column update with the levels split over threads ------
// The column system's LU factors (la, lc, li) depend on the level only, so
// both recurrences, dp(k) = (rhs(k) - la(k) dp(k-1)) li(k) and
// x(k) = dp(k) - lc(k) x(k+1), split into chunks of kM levels: each thread
// solves its chunk with a zero carry and the chunks are joined by a scan of
// the carries, dp(k) = dpl(k) + G(k) dp(k0-1) with G(k) = prod_{l=k0..k}
// (-la(l) li(l)), and x(k) = xl(k) + H(k) x(k0+kM) with H(k) = prod_{l=k..
// k0+kM-1} (-lc(l)). A block is 32 consecutive columns (one warp per chunk,
// so every level's load is one 128-byte row) by C = ceil(nz/kM) chunks; every
// thread issues all the loads of its chunk at once and nothing is parked
// between sweeps. Same arithmetic per level as hevi_body; the carries change
// the rounding of the tridiagonal solve only.
template <int kM>
__device__ __forceinline__ void hevi_par_body(const Dims& d, const Tab& t, const Flags& fl, const WS& win,
                                              const WS& wout, float dtau, const float* __restrict__ lu,
                                              int apply_uv, float cdx, float cdy, int bx, int by) {
  extern __shared__ float s_tab[];
  const int nz = d.nz;
  const int C = blockDim.y;
  float* s_tfz = s_tab;                    // nz+1
  float* s_idzw = s_tfz + (nz + 1);        // nz+1
  float* s_rfz = s_idzw + (nz + 1);        // nz+1
  float* s_idzc = s_rfz + (nz + 1);        // nz
  float* s_kap = s_idzc + nz;              // nz
  float* s_la = s_kap + nz;                // nz
  float* s_lc = s_la + nz;                 // nz
  float* s_li = s_lc + nz;                 // nz
  float* s_r0 = s_li + nz;                 // nz
  float* s_t0 = s_r0 + nz;                 // nz
  float* s_a = s_t0 + nz;                  // C x 32: chunk result with zero carry
  float* s_g = s_a + C * 32;               // C x 32: its carry coefficient
  float* s_e = s_g + C * 32;               // (C+1) x 32: scanned carries
  float* s_x = s_e + (C + 1) * 32;         // C x 32: x at each chunk's top level
  const int tx = threadIdx.x, c = threadIdx.y;
  const int tid = c * 32 + tx, nthr = 32 * C;
  for (int e = tid; e <= nz; e += nthr) {
    s_tfz[e] = t.tfz[e];
    s_idzw[e] = t.idzw[e];
    s_rfz[e] = t.rfz[e];
    if (e < nz) {
      s_idzc[e] = t.idzc[e];
      s_kap[e] = t.kap[e];
      s_la[e] = lu[e];
      s_lc[e] = lu[nz + e];
      s_li[e] = lu[2 * nz + e];
      s_r0[e] = t.r0c[e];
      s_t0[e] = t.t0c[e];
    }
  }
  __syncthreads();
  const int i = bx * 32 + tx;
  const int j = by;
  const bool active = i < d.nx && j < d.ny;
  const int k0 = c * kM;
  const int kn = imin(kM, nz - k0);  // >= 1: C = ceil(nz / kM)
  const float b = (float)fl.hevi_beta, ob = 1.f - b;
  const float cpf = (float)kCp;
  const size_t pl = d.plane;
  const size_t col = active ? (size_t)j * d.P + i : 0;
  const float* __restrict__ U0 = win.f[U] + col;
  const float* __restrict__ V0 = win.f[V] + col;
  const float* __restrict__ W0 = win.f[W] + col;
  const float* __restrict__ P0 = win.f[PI] + col;
  const float* __restrict__ R0 = win.f[RHO] + col;
  float* __restrict__ Wo = wout.f[W] + col;
  float* __restrict__ Po = wout.f[PI] + col;
  float* __restrict__ Ro = wout.f[RHO] + col;
  float* __restrict__ Uo = wout.f[U] + col;
  float* __restrict__ Vo = wout.f[V] + col;
  const size_t vn = d.P;
  const float dxi = t.dx_inv, dyi = t.dy_inv;
  const int ow = (i > 0) ? -1 : 0, oe = (i + 1 < d.nx) ? 1 : 0;
  const long long os = (j > 0) ? -(long long)vn : 0, on = (j + 1 < d.ny) ? (long long)vn : 0;
  const bool last_i = (i == d.nx - 1), last_j = (j == d.ny - 1);

  float pv[kM + 2];  // p'(k0-1+q), 0 outside [0, nz)
  float wv[kM + 1];  // w(face k0+q)
  float wt[kM + 1];  // w with the explicit pressure gradient, faces k0..k0+kM
  float rhs[kM], rs[kM], dp[kM], gq[kM];
#pragma unroll
  for (int q = 0; q < kM + 2; ++q) {
    const int kk = k0 - 1 + q;
    pv[q] = (active && kk >= 0 && kk < nz && q <= kn + 1) ? P0[(size_t)kk * pl] : 0.f;
  }
#pragma unroll
  for (int q = 0; q < kM + 1; ++q) {
    const int f = k0 + q;
    wv[q] = (active && q <= kn && f <= nz) ? W0[(size_t)f * pl] : 0.f;
  }
#pragma unroll
  for (int q = 0; q < kM + 1; ++q) {
    const int f = k0 + q;
    wt[q] = wv[q];
    if (q <= kn && f >= 1 && f < nz)
      wt[q] = wv[q] - dtau * ob * cpf * s_tfz[f] * (pv[q + 1] - pv[q]) * s_idzw[f];
  }
  float w_top = 0.f;  // w(face k0+kn)
#pragma unroll
  for (int q = 0; q < kM + 1; ++q)
    if (q == kn) w_top = wv[q];
  float prev = 0.f, g = 1.f, d_last = 0.f, g_last = 1.f;
#pragma unroll
  for (int q = 0; q < kM; ++q) {
    rhs[q] = rs[q] = dp[q] = 0.f;
    gq[q] = 1.f;
    if (q < kn) {
      const int k = k0 + q;
      if (active) {
        const size_t o = (size_t)k * pl;
        const float p_k = pv[q + 1];
        float u0 = U0[o], u1 = U0[o + 1], v0 = V0[o], v1 = V0[o + vn];
        if (apply_uv) {
          const float tx_ = s_t0[k] * cdx, ty_ = s_t0[k] * cdy;
          u0 += tx_ * (p_k - P0[o + ow]);
          u1 += tx_ * (P0[o + oe] - p_k);
          v0 += ty_ * (p_k - P0[o + os]);
          v1 += ty_ * (P0[o + on] - p_k);
        }
        const float Dh = -(s_r0[k] * ((u1 - u0) * dxi + (v1 - v0) * dyi));
        Uo[o] = u0;
        Vo[o] = v0;
        if (last_i) Uo[o + 1] = u1;
        if (last_j) Vo[o + vn] = v1;
        const float rk = s_rfz[k], rk1 = s_rfz[k + 1], idz = s_idzc[k];
        const float dv_old = -(rk1 * wv[q + 1] - rk * wv[q]) * idz;
        const float dv_t = -(rk1 * wt[q + 1] - rk * wt[q]) * idz;
        const float S = Dh + ob * dv_old;
        rhs[q] = p_k + dtau * s_kap[k] * (S + b * dv_t);
        rs[q] = R0[o] + dtau * S;
      }
      dp[q] = (rhs[q] - s_la[k] * prev) * s_li[k];
      prev = dp[q];
      g *= -s_la[k] * s_li[k];
      gq[q] = g;
      d_last = dp[q];
      g_last = g;
    }
  }
  s_a[tid] = d_last;
  s_g[tid] = g_last;
  __syncthreads();
  if (c == 0) {  // forward carries: s_e[cc] = dp(last level of chunk cc-1)
    float e = 0.f;
    s_e[tx] = 0.f;
    for (int cc = 0; cc < C; ++cc) {
      e = s_a[cc * 32 + tx] + s_g[cc * 32 + tx] * e;
      s_e[(cc + 1) * 32 + tx] = e;
    }
  }
  __syncthreads();
  const float ein = s_e[tid];
  float hq[kM];
#pragma unroll
  for (int q = 0; q < kM; ++q) dp[q] += gq[q] * ein;
  float nxt = 0.f, h = 1.f;
#pragma unroll
  for (int q = kM - 1; q >= 0; --q) {
    hq[q] = 1.f;
    if (q < kn) {
      const int k = k0 + q;
      dp[q] = dp[q] - s_lc[k] * nxt;  // local x with zero carry from above
      nxt = dp[q];
      h *= -s_lc[k];
      hq[q] = h;
    }
  }
  s_a[tid] = dp[0];
  s_g[tid] = hq[0];
  __syncthreads();
  if (c == 0) {  // backward carries: s_e[cc] = x(first level of chunk cc), s_e[C] = 0
    float x = 0.f;
    s_e[C * 32 + tx] = 0.f;
    for (int cc = C - 1; cc >= 0; --cc) {
      x = s_a[cc * 32 + tx] + s_g[cc * 32 + tx] * x;
      s_e[cc * 32 + tx] = x;
    }
  }
  __syncthreads();
  const float xin = s_e[(c + 1) * 32 + tx];  // x(k0 + kn), 0 above the top
  float x_last = 0.f;
#pragma unroll
  for (int q = 0; q < kM; ++q) {
    dp[q] += hq[q] * xin;  // dp now holds x
    if (q == kn - 1) x_last = dp[q];
  }
  s_x[tid] = x_last;
  __syncthreads();
  if (!active) return;
  const float xprev = (c > 0) ? s_x[tid - 32] : 0.f;
  // final w on faces k0..k0+kn, then rho' and the outputs
  float wn[kM + 1];
#pragma unroll
  for (int q = 0; q < kM + 1; ++q) {
    const int f = k0 + q;
    wn[q] = wt[q];
    if (q <= kn && f >= 1 && f < nz) {
      const float xf = (q < kn) ? dp[q] : xin;
      const float xb = (q == 0) ? xprev : dp[q - 1];
      wn[q] = wt[q] - dtau * b * cpf * s_tfz[f] * (xf - xb) * s_idzw[f];
    }
  }
#pragma unroll
  for (int q = 0; q < kM; ++q) {
    if (q < kn) {
      const int k = k0 + q;
      const size_t o = (size_t)k * pl;
      const float dv_new = -(s_rfz[k + 1] * wn[q + 1] - s_rfz[k] * wn[q]) * s_idzc[k];
      Ro[o] = rs[q] + dtau * b * dv_new;
      Po[o] = dp[q];
      Wo[o] = wn[q];
    }
  }
  if (k0 + kn == nz) Wo[(size_t)nz * pl] = w_top;
}

template <int kM>
__global__ void __launch_bounds__(640, 2) k_mx_hevi_par(const __grid_constant__ Dims d, const __grid_constant__ Tab t,
                                                      const __grid_constant__ Flags fl, const __grid_constant__ WS win,
                                                      const __grid_constant__ WS wout, float dtau,
                                                      const float* __restrict__ lu, int apply_uv, float cdx,
                                                      float cdy) {
  hevi_par_body<kM>(d, t, fl, win, wout, dtau, lu, apply_uv, cdx, cdy, blockIdx.x, blockIdx.y);
}

template <int kPF, int kRing>
__global__ void __launch_bounds__(128, 8) k_mx_hevi_col(const __grid_constant__ Dims d, const __grid_constant__ Tab t,
                                                         const __grid_constant__ Flags fl,
                                                         const __grid_constant__ WS win,
                                                         const __grid_constant__ WS wout, float dtau,
                                                         const float* __restrict__ lu, int apply_uv, float cdx,
                                                         float cdy) {
  hevi_body<kPF, kRing>(d, t, fl, win, wout, dtau, lu, apply_uv, cdx, cdy, blockIdx.x, blockIdx.y);
}

// Prefetch depth of the HEVI column kernel (levels of loads in flight per
// thread); VIBE_GB300_HEVI_PF=2|4|6|8 overrides the built-in choice.
static int hevi_pf() {
  static int pf = 0;
  if (pf == 0) {
    pf = 2;  // measured best at 512x512x80: 2 < 4 < 6 < 8 (0.237 / 0.267 / 0.273 / 0.310 ms)
    if (const char* e = std::getenv("VIBE_GB300_HEVI_PF")) {
      const int v = std::atoi(e);
      if (v == 2 || v == 4 || v == 6 || v == 8) pf = v;
    }
  }
  return pf;
}

// Depth of the shared-memory cp.async ring of the column kernel's forward
// sweep (0 = the register ring of hevi_pf()); VIBE_GB300_HEVI_RING=0|4|6|8.
int hevi_ring() {
  static int r = -1;
  if (r < 0) {
    r = kDefaultHeviRing;
    if (const char* e = std::getenv("VIBE_GB300_HEVI_RING")) {
      const int v = std::atoi(e);
      if (v == 0 || v == 4 || v == 6 || v == 8) r = v;
    }
  }
  return r;
}

size_t hevi_smem_bytes(int nz, int ring) {
  return (10 * (size_t)(nz + 1) + (size_t)ring * 11 * 128) * sizeof(float);
}

// Levels per thread of the level-split column kernel (0 = one thread per
// column, hevi_body); VIBE_GB300_HEVI_PAR=0|4|8 overrides the built-in choice.
int hevi_par_levels(int nz) {
  static int v = -1;
  if (v < 0) {
    v = kDefaultHeviPar;
    if (const char* e = std::getenv("VIBE_GB300_HEVI_PAR")) {
      const int x = std::atoi(e);
      if (x == 0 || x == 4 || x == 8) v = x;
    }
  }
  if (v == 0) return 0;
  int m = v;
  if ((nz + m - 1) / m > 20) m = 8;       // at most 20 chunks (640 threads)
  return ((nz + m - 1) / m > 20) ? 0 : m;  // taller columns: one thread per column
}

size_t hevi_par_smem_bytes(int nz, int m) {
  const int C = (nz + m - 1) / m;
  return (10 * (size_t)(nz + 1) + (size_t)32 * (4 * C + 1)) * sizeof(float);
}

// Ring depth of the two-columns-per-thread kernel (0 = off);
// VIBE_GB300_HEVI_TWO=0|2|3|4 overrides the built-in choice.
int hevi_two_ring() {
  static int v = -1;
  if (v < 0) {
    v = kDefaultHeviTwo;
    if (const char* e = std::getenv("VIBE_GB300_HEVI_TWO")) {
      const int x = std::atoi(e);
      if (x == 0 || x == 2 || x == 3 || x == 4) v = x;
    }
  }
  return v;
}

bool hevi_tma() {
  static int v = -1;
  if (v < 0) {
    v = kDefaultHeviTma ? 1 : 0;
    if (const char* e = std::getenv("VIBE_GB300_HEVI_TMA")) v = std::atoi(e) != 0;
  }
  return v != 0;
}

// the TMA column kernel defers the w/rho' corrections (kDefer);
// VIBE_GB300_HEVI_DEFER=0 keeps both sweeps on all three fields
bool hevi_defer() {
  static int v = -1;
  if (v < 0) {
    v = kDefaultHeviDefer ? 1 : 0;
    if (const char* e = std::getenv("VIBE_GB300_HEVI_DEFER")) v = std::atoi(e) != 0;
  }
  return v != 0;
}

// the column kernel variant for this grid among the TMA ones: 4 TMA,
// 5 TMA with deferred corrections, -1 neither
int hevi_tma_variant(const Dims& d) {
  MixedTune tn;
  bool tma = hevi_tma(), defer = hevi_defer();
  if (tune_of(d, &tn) && tn.column >= 0) {
    tma = tn.column == 4 || tn.column == 5;
    defer = tn.column == 5;
  }
  if (!tma || hevi_tma_smem_bytes(d.nz) > 48 * 1024) return -1;
  return defer ? 5 : 4;
}

size_t hevi2_smem_bytes(int nz, int ring) {
  return ((((size_t)10 * (nz + 1) + 3) & ~(size_t)3) + (size_t)ring * 19 * 128) * sizeof(float);
}

int mixed_hevi_column(const Dims& d, const Tab& t, const Flags& fl, const WS& win, const WS& wout, float dtau,
                      const float* lu, bool apply_uv, unsigned* err, cudaStream_t stream) {
  MixedTune tn;
  const bool tuned = tune_of(d, &tn) && tn.column >= 0;
  int r2 = hevi_two_ring(), ring = hevi_ring();
  if (tuned) {  // 0: register ring, 1: cp.async ring 4, 2/3: two columns per thread with ring 2/3, 4/5: TMA-fed
    r2 = (tn.column == 2) ? 2 : (tn.column == 3 ? 3 : 0);
    ring = (tn.column == 1) ? 4 : 0;
  }
  if (const int v = hevi_tma_variant(d); v >= 0) {
    ColumnMaps C;
    if (!column_maps(d, win, wout, C)) return -1;
    const dim3 bc(32, 4);
    const dim3 g((d.nx + 63) / 64, (d.ny + 3) / 4);
    const float cdx = -(float)kCp * dtau * t.dx_inv, cdy = -(float)kCp * dtau * t.dy_inv;
    if (v == 5)
      k_mx_hevi_tmad<<<g, bc, hevi_tma_smem_bytes(d.nz), stream>>>(d, t, fl, C, win, wout, dtau, lu,
                                                                     apply_uv ? 1 : 0, cdx, cdy, err);
    else
      k_mx_hevi_tma<<<g, bc, hevi_tma_smem_bytes(d.nz), stream>>>(d, t, fl, C, win, wout, dtau, lu,
                                                                    apply_uv ? 1 : 0, cdx, cdy, err);
    return 0;
  }
  if (r2) {
    const dim3 bc(32, 4);
    const dim3 g((d.nx + 63) / 64, (d.ny + 3) / 4);
    const float cdx = -(float)kCp * dtau * t.dx_inv, cdy = -(float)kCp * dtau * t.dy_inv;
    const size_t sm = hevi2_smem_bytes(d.nz, r2);
    const int au = apply_uv ? 1 : 0;
    if (r2 == 4) k_mx_hevi_col2<4><<<g, bc, sm, stream>>>(d, t, fl, win, wout, dtau, lu, au, cdx, cdy);
    else if (r2 == 3) k_mx_hevi_col2<3><<<g, bc, sm, stream>>>(d, t, fl, win, wout, dtau, lu, au, cdx, cdy);
    else k_mx_hevi_col2<2><<<g, bc, sm, stream>>>(d, t, fl, win, wout, dtau, lu, au, cdx, cdy);
    return 0;
  }
  if (const int m = tuned ? 0 : hevi_par_levels(d.nz)) {
    const dim3 bp(32, (d.nz + m - 1) / m);
    const dim3 gp((d.nx + 31) / 32, d.ny);
    const float cdx = -(float)kCp * dtau * t.dx_inv, cdy = -(float)kCp * dtau * t.dy_inv;
    const size_t sm = hevi_par_smem_bytes(d.nz, m);
    if (m == 4)
      k_mx_hevi_par<4><<<gp, bp, sm, stream>>>(d, t, fl, win, wout, dtau, lu, apply_uv ? 1 : 0, cdx, cdy);
    else
      k_mx_hevi_par<8><<<gp, bp, sm, stream>>>(d, t, fl, win, wout, dtau, lu, apply_uv ? 1 : 0, cdx, cdy);
    return 0;
  }
  const dim3 bc(32, 4);
  const size_t smem = hevi_smem_bytes(d.nz, ring);
  const dim3 g((d.nx + bc.x - 1) / bc.x, (d.ny + bc.y - 1) / bc.y);
  const float cdx = -(float)kCp * dtau * t.dx_inv, cdy = -(float)kCp * dtau * t.dy_inv;
  const int au = apply_uv ? 1 : 0;
  if (ring == 8) {
    k_mx_hevi_col<2, 8><<<g, bc, smem, stream>>>(d, t, fl, win, wout, dtau, lu, au, cdx, cdy);
  } else if (ring == 6) {
    k_mx_hevi_col<2, 6><<<g, bc, smem, stream>>>(d, t, fl, win, wout, dtau, lu, au, cdx, cdy);
  } else if (ring == 4) {
    k_mx_hevi_col<2, 4><<<g, bc, smem, stream>>>(d, t, fl, win, wout, dtau, lu, au, cdx, cdy);
  } else {
    switch (hevi_pf()) {
      case 6: k_mx_hevi_col<6, 0><<<g, bc, smem, stream>>>(d, t, fl, win, wout, dtau, lu, au, cdx, cdy); break;
      case 8: k_mx_hevi_col<8, 0><<<g, bc, smem, stream>>>(d, t, fl, win, wout, dtau, lu, au, cdx, cdy); break;
      case 4: k_mx_hevi_col<4, 0><<<g, bc, smem, stream>>>(d, t, fl, win, wout, dtau, lu, au, cdx, cdy); break;
      default: k_mx_hevi_col<2, 0><<<g, bc, smem, stream>>>(d, t, fl, win, wout, dtau, lu, au, cdx, cdy); break;
    }
  }
  return 0;
}

void mixed_uv_backward(const Dims& d, const Tab& t, const WS& win, const WS& wout, float dtau, cudaStream_t stream) {
  const dim3 b(32, 4);
  k_mx_fb_mom<<<g3(d.nx + 1, d.ny + 1, d.nz, b), b, 0, stream>>>(d, t, win, wout, dtau, 0);
}

bool mixed_hevi_defers(const Dims& d) { return hevi_tma_variant(d) == 5; }

void mixed_uv_fix(const Dims& d, const Tab& t, const Flags& fl, const WS& s, float dtau, cudaStream_t stream) {
  const dim3 b(32, 4);
  k_mx_fix<<<g3((d.nx + 1 + kFixPos - 1) / kFixPos, d.ny + 1, 1, b), b, 0, stream>>>(d, t, fl, s, dtau);
}

int mixed_hevi_substep(const Dims& d, const Tab& t, const Flags& fl, const WS& win, const WS& wout, float dtau,
                       const float* lu, unsigned* err, cudaStream_t stream) {
  if (mixed_hevi_column(d, t, fl, win, wout, dtau, lu, false, err, stream)) return -1;
  // in place: u, v were copied by the column kernel
  if (mixed_hevi_defers(d)) mixed_uv_fix(d, t, fl, wout, dtau, stream);
  else mixed_uv_backward(d, t, wout, wout, dtau, stream);
  return 0;
}

void mixed_finish(const Dims& d, const Tab& t, const Flags& fl, const WS& wfin, const WS& wst, const WS& w0,
                  const WS* rin, double dt, double* const* s0, double* const* s1, unsigned* err,
                  cudaStream_t stream, float uv_dtau, bool defer) {
  const dim3 b(32, 4);
  WS none;
  for (int q = 0; q < NSPECIES; ++q) none.f[q] = nullptr;
  k_mx_finish<<<g3(d.nx + 1, d.ny + 1, d.nz + 1, b), b, 0, stream>>>(d, t, fl, wfin, wst, w0, rin ? *rin : none,
                                                                     (float)dt, cs64(s0), ms64(s1), err, uv_dtau,
                                                                     defer ? 1 : 0);
}

void mixed_unpack_f32(const Dims& d, int nsx, int nsy, int nsz, int ni, int nj, int nk, const float* src, double* dst,
                      cudaStream_t stream) {
  k_mx_unpack_f32<<<1024, 256, 0, stream>>>(d, nsx, nsy, nsz, ni, nj, nk, src, dst);
}

namespace {
struct DaviesW {
  double a[64];
};
// A nest's Davies relaxation toward its boundary buffer (apply_lateral_boundary,
// nest.cpp:107-124: c = (1 - alpha(d)) c + alpha(d) b on the points within
// nzone of the lateral edge, d their distance to it) and, at the same points,
// the FP32 working copy of the relaxed state. One thread per (frame column,
// level); the products and the sum rounded one by one as the reference
// computes them (no fused multiply-add).
__global__ void k_mx_nest_relax(const __grid_constant__ Dims d, const __grid_constant__ Tab t,
                                const __grid_constant__ MS64 s, const __grid_constant__ CS64 bnd, int nvars,
                                const __grid_constant__ DaviesW dw, int nzone, int nframe,
                                const __grid_constant__ WS w) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.z;
  if (e >= nframe) return;
  int i, j;
  frame_column(e, d.nx, d.ny, nzone, i, j);
  const double alpha = dw.a[imin(imin(i, d.nx - 1 - i), imin(j, d.ny - 1 - j))];
  const size_t c = IX(i, j, k);
  for (int q = 0; q < nvars; ++q) {
    const double v = s.f[q][c];
    s.f[q][c] = __dadd_rn(__dmul_rn(__dsub_rn(1.0, alpha), v), __dmul_rn(alpha, bnd.f[q][c]));
  }
  CS64 r;
  for (int q = 0; q < NSPECIES; ++q) r.f[q] = s.f[q];
  to_working_point(d, t, r, w, i, j, k);
}
}  // namespace

int mixed_nest_relax(const Dims& d, const Tab& t, double* const* s, const double* const* bnd, int nvars,
                     const double* davies, int nzone, const WS& w, cudaStream_t stream) {
  if (nzone < 1 || nzone > 64 || nvars < 1 || nvars > NSPECIES) return -1;
  DaviesW dw{};
  for (int q = 0; q < nzone; ++q) dw.a[q] = davies[q];
  MS64 sm = ms64(s);
  CS64 bm;
  for (int q = 0; q < NSPECIES; ++q) bm.f[q] = q < nvars ? bnd[q] : nullptr;
  const int nf = frame_count(d.nx, d.ny, nzone);
  k_mx_nest_relax<<<dim3((nf + 127) / 128, 1, d.nz), 128, 0, stream>>>(d, t, sm, bm, nvars, dw, nzone, nf, w);
  return 0;
}

void mixed_to_working_region(const Dims& d, const Tab& t, double* const* s, const WS& w, int ia, int ja, int ni,
                             int nj, cudaStream_t stream) {
  const int a0 = imax(ia, 0), b0 = imax(ja, 0);
  const int a1 = imin(ia + ni, d.nx + 1), b1 = imin(ja + nj, d.ny + 1);
  if (a1 <= a0 || b1 <= b0) return;
  const dim3 b(32, 4);
  k_mx_to_working_region<<<g3(a1 - a0, b1 - b0, d.nz + 1, b), b, 0, stream>>>(d, t, cs64(s), w, a0, b0, a1, b1);
}

void mixed_to_working(const Dims& d, const Tab& t, double* const* s, const WS& w, cudaStream_t stream) {
  const dim3 b(32, 4);
  k_mx_to_working<<<g3(d.nx + 1, d.ny + 1, d.nz + 1, b), b, 0, stream>>>(d, t, cs64(s), w);
}


// ===========================================================================
// Several domains in one launch per kernel: a work-list of blocks over all
// domains (start[d] = first block of domain d); each block finds its domain
// and runs the single-domain body with that domain's arguments, read from
// device memory (TMA descriptors included, 64-byte aligned).
// ===========================================================================
namespace {
struct StageArgs {  // 64-byte aligned through its CUtensorMap members
  StageMaps M;
  Dims d;
  Tab t;
  Flags fl;
  WS win, w0, wout, rout;
  float dts;
  int kchunk, gx, gy, gz;
};
struct HeviArgs {  // 64-byte aligned through its CUtensorMap members
  ColumnMaps C;     // boxes of the TMA-fed body (unused by the cp.async body)
  Dims d;
  Tab t;
  Flags fl;
  WS win, wout;
  float dtau, cdx, cdy;
  const float* lu;
  int apply_uv, gx, gy;
};
struct UvArgs {
  Dims d;
  Tab t;
  Flags fl;
  WS win, wout;
  float dtau;
  int gx, gy, gz;
};
struct FinishArgs {
  Dims d;
  Tab t;
  Flags fl;
  WS wfin, wst, w0, rin;
  float dtf, uv_dtau;  // uv_dtau: stage 3's last u/v update, applied in the finish
  CS64 s0;
  MS64 s1;
  int gx, gy, gz, defer;
};

__device__ __forceinline__ int find_domain(const int* __restrict__ start, int nd) {
  int dom = 0;
  while (dom + 1 < nd && (int)blockIdx.x >= start[dom + 1]) ++dom;
  return dom;
}

// kSpec: every domain runs the composition the single-domain kSpec kernel
// fixes at compile time (the flags are common to a batch)
template <bool kRaw, bool kSpec>
__global__ void __launch_bounds__(NT, 3) k_b_stage(const StageArgs* __restrict__ A, const int* __restrict__ start,
                                                   int nd, unsigned* err) {
  const int dom = find_domain(start, nd);
  const StageArgs& a = A[dom];
  const int l = (int)blockIdx.x - start[dom];
  stage_body<kRaw, kSpec>(a.d, a.t, a.fl, a.M, a.win, a.w0, a.wout, a.rout, a.dts, a.kchunk, err, l % a.gx,
                          (l / a.gx) % a.gy, l / (a.gx * a.gy));
}

__global__ void __launch_bounds__(128, 7) k_b_hevi(const HeviArgs* __restrict__ A, const int* __restrict__ start,
                                                   int nd) {
  const int dom = find_domain(start, nd);
  const HeviArgs& a = A[dom];
  const int l = (int)blockIdx.x - start[dom];
  hevi2_body<kBatchTwoRing>(a.d, a.t, a.fl, a.win, a.wout, a.dtau, a.lu, a.apply_uv, a.cdx, a.cdy, l % a.gx,
                            l / a.gx);
}

__global__ void __launch_bounds__(128, 7) k_b_hevi_tma(const HeviArgs* __restrict__ A, const int* __restrict__ start,
                                                       int nd, unsigned* err) {
  const int dom = find_domain(start, nd);
  const HeviArgs& a = A[dom];
  const int l = (int)blockIdx.x - start[dom];
  hevi_tma_body<false>(a.d, a.t, a.fl, a.C, a.win, a.wout, a.dtau, a.lu, a.apply_uv, a.cdx, a.cdy, err, l % a.gx,
                l / a.gx);
}

__global__ void __launch_bounds__(128, 7) k_b_hevi_tmad(const HeviArgs* __restrict__ A,
                                                        const int* __restrict__ start, int nd, unsigned* err) {
  const int dom = find_domain(start, nd);
  const HeviArgs& a = A[dom];
  const int l = (int)blockIdx.x - start[dom];
  hevi_tma_body<true>(a.d, a.t, a.fl, a.C, a.win, a.wout, a.dtau, a.lu, a.apply_uv, a.cdx, a.cdy, err, l % a.gx,
                      l / a.gx);
}

__global__ void k_b_uv(const UvArgs* __restrict__ A, const int* __restrict__ start, int nd) {
  const int dom = find_domain(start, nd);
  const UvArgs& a = A[dom];
  const int l = (int)blockIdx.x - start[dom];
  fb_mom_body(a.d, a.t, a.win, a.wout, a.dtau, 0, l % a.gx, (l / a.gx) % a.gy, l / (a.gx * a.gy));
}
__global__ void __launch_bounds__(128, 8) k_b_fix(const UvArgs* __restrict__ A, const int* __restrict__ start, int nd) {
  const int dom = find_domain(start, nd);
  const UvArgs& a = A[dom];
  const int l = (int)blockIdx.x - start[dom];
  fix_body(a.d, a.t, a.fl, a.wout, a.dtau, l % a.gx, l / a.gx);
}

__global__ void k_b_finish(const FinishArgs* __restrict__ A, const int* __restrict__ start, int nd, unsigned* err) {
  const int dom = find_domain(start, nd);
  const FinishArgs& a = A[dom];
  const int l = (int)blockIdx.x - start[dom];
  finish_body(a.d, a.t, a.fl, a.wfin, a.wst, a.w0, a.rin, a.dtf, a.s0, a.s1, err, l % a.gx, (l / a.gx) % a.gy,
              l / (a.gx * a.gy), a.uv_dtau, a.defer != 0);
}

WS ws_from(float* const* a) {
  WS w;
  for (int q = 0; q < NSPECIES; ++q) w.f[q] = a ? a[q] : nullptr;
  return w;
}
WS ws_mix(float* const* sub, float* const* stage) {  // acoustic fields from sub, the rest from stage
  WS w;
  for (int q = 0; q < NSPECIES; ++q)
    w.f[q] = (q == U || q == V || q == W || q == RHO || q == PI) ? sub[q] : stage[q];
  return w;
}
}  // namespace

struct MixedBatch {
  struct Launch {
    int kind = 0;  // 0 stage, 1 column, 2 u/v (with deferral: the u/v/w/rho' fix-up), 3 finish
    int raw = 0, nd = 0, blocks = 0;
    void* args = nullptr;
    int* start = nullptr;
  };
  std::vector<Launch> seq;
  std::vector<void*> allocs;
  size_t hevi_smem = 0;
  bool hevi_tma = false;  // TMA-fed column body (else the cp.async two-column body)
  bool defer = false;     // the TMA body defers its w/rho' corrections (u/v launches become fix-ups)
  bool spec = false;      // the stage body with the flags of the kSpec composition fixed
  unsigned* err = nullptr;
};

namespace {
template <class A>
bool upload_launch(MixedBatch* b, int kind, int raw, const std::vector<A>& args, const std::vector<int>& start,
                   int blocks) {
  MixedBatch::Launch L;
  L.kind = kind;
  L.raw = raw;
  L.nd = (int)args.size();
  L.blocks = blocks;
  if (cudaMalloc(&L.args, args.size() * sizeof(A)) != cudaSuccess) return false;
  b->allocs.push_back(L.args);
  if (cudaMalloc((void**)&L.start, start.size() * sizeof(int)) != cudaSuccess) return false;
  b->allocs.push_back(L.start);
  if (cudaMemcpy(L.args, args.data(), args.size() * sizeof(A), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(L.start, start.data(), start.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess)
    return false;
  b->seq.push_back(L);
  return true;
}
int ceil_div(int a, int b) { return (a + b - 1) / b; }
}  // namespace

MixedBatch* mixed_batch_build(const std::vector<MixedDomain>& doms, const Flags& fl, double dt, int n_sub,
                              unsigned* err) {
  if (doms.empty() || fl.acoustic_mode != 2) return nullptr;
  const int nz = doms[0].d.nz;
  for (const auto& m : doms)
    if (m.d.nz != nz) return nullptr;
  auto* b = new MixedBatch();
  b->err = err;
  b->hevi_tma = hevi_tma() && hevi_tma_smem_bytes(nz) <= 48 * 1024;
  b->defer = b->hevi_tma && hevi_defer();
  b->spec = stage_spec(fl);
  b->hevi_smem = b->hevi_tma ? hevi_tma_smem_bytes(nz) : hevi2_smem_bytes(nz, kBatchTwoRing);
  const double dts[3] = {dt / 3.0, dt / 2.0, dt};
  const int nd = (int)doms.size();
  auto sub_out = [&](const MixedDomain& m, int n) { return (n & 1) ? m.WB : m.WA; };
  bool ok = true;
  for (int stage = 0; stage < 3 && ok; ++stage) {
    std::vector<StageArgs> sa(nd);
    std::vector<int> start(nd);
    int blocks = 0;
    const bool raw = stage == 2;
    for (int q = 0; q < nd && ok; ++q) {
      const MixedDomain& m = doms[q];
      float* const* st_out = stage & 1 ? m.WSt1 : m.WSt0;
      const WS win = (stage == 0) ? ws_from(m.W0) : ws_mix(sub_out(m, n_sub - 1), (stage - 1) & 1 ? m.WSt1 : m.WSt0);
      StageArgs& a = sa[q];
      ok = stage_maps(m.d, win, a.M);
      a.d = m.d;
      a.t = m.t;
      a.fl = fl;
      a.win = win;
      a.w0 = ws_from(m.W0);
      a.wout = ws_from(st_out);
      a.rout = raw ? ws_from(m.WR) : a.wout;
      a.dts = (float)dts[stage];
      a.kchunk = stage_kchunk(m.d, raw);
      a.gx = (m.d.nx + TX) / TX;
      a.gy = (m.d.ny + TY) / TY;
      a.gz = ceil_div(m.d.nz, a.kchunk);
      start[q] = blocks;
      blocks += a.gx * a.gy * a.gz;
    }
    ok = ok && upload_launch(b, 0, raw ? 1 : 0, sa, start, blocks);
    const float dtau = (float)(dts[stage] / (double)n_sub);
    for (int n = 0; n < n_sub && ok; ++n) {
      std::vector<HeviArgs> ha(nd);
      int hb = 0;
      for (int q = 0; q < nd; ++q) {
        const MixedDomain& m = doms[q];
        float* const* in = (n == 0) ? (stage & 1 ? m.WSt1 : m.WSt0) : sub_out(m, n - 1);
        HeviArgs& a = ha[q];
        a.d = m.d;
        a.t = m.t;
        a.fl = fl;
        a.win = ws_from(in);
        a.wout = ws_from(sub_out(m, n));
        a.dtau = dtau;
        a.cdx = -(float)kCp * dtau * m.t.dx_inv;
        a.cdy = -(float)kCp * dtau * m.t.dy_inv;
        a.lu = m.lu + (size_t)stage * 3 * nz;
        a.apply_uv = n > 0;
        if (b->hevi_tma && !column_maps(m.d, a.win, a.wout, a.C)) ok = false;
        a.gx = ceil_div(m.d.nx, 64);  // two columns per thread
        a.gy = ceil_div(m.d.ny, 4);
        start[q] = hb;
        hb += a.gx * a.gy;
      }
      ok = ok && upload_launch(b, 1, 0, ha, start, hb);
    }
    if (stage == 2) break;  // stage 3's last u/v update happens in the finish
    std::vector<UvArgs> ua(nd);
    int ub = 0;
    for (int q = 0; q < nd; ++q) {
      const MixedDomain& m = doms[q];
      UvArgs& a = ua[q];
      a.d = m.d;
      a.t = m.t;
      a.fl = fl;
      a.win = ws_from(sub_out(m, n_sub - 1));
      a.wout = a.win;
      a.dtau = dtau;
      a.gx = ceil_div(m.d.nx + 1, b->defer ? 32 * kFixPos : 32);  // (the fix-up: kFixPos positions per thread)
      a.gy = ceil_div(m.d.ny + 1, 4);
      a.gz = b->defer ? 1 : m.d.nz;  // the deferred fix-up marches the levels
      start[q] = ub;
      ub += a.gx * a.gy * a.gz;
    }
    ok = ok && upload_launch(b, 2, 0, ua, start, ub);
  }
  if (ok) {
    std::vector<FinishArgs> fa(nd);
    std::vector<int> start(nd);
    int fb = 0;
    for (int q = 0; q < nd; ++q) {
      const MixedDomain& m = doms[q];
      FinishArgs& a = fa[q];
      a.d = m.d;
      a.t = m.t;
      a.fl = fl;
      a.wfin = ws_from(sub_out(m, n_sub - 1));
      a.wst = ws_from(m.WSt0);
      a.w0 = ws_from(m.W0);
      a.rin = ws_from(m.WR);
      a.dtf = (float)dt;
      a.uv_dtau = (float)(dt / (double)n_sub);
      a.s0 = cs64(m.S0);
      a.s1 = ms64(m.S1);
      a.defer = b->defer ? 1 : 0;
      a.gx = ceil_div(m.d.nx + 1, 32);
      a.gy = ceil_div(m.d.ny + 1, 4);
      a.gz = m.d.nz + 1;
      start[q] = fb;
      fb += a.gx * a.gy * a.gz;
    }
    ok = upload_launch(b, 3, 0, fa, start, fb);
  }
  if (!ok) {
    mixed_batch_destroy(b);
    return nullptr;
  }
  return b;
}

void mixed_batch_enqueue(const MixedBatch* b, cudaStream_t s) {
  for (const auto& L : b->seq) {
    switch (L.kind) {
      case 0:
        if (L.raw && b->spec)
          k_b_stage<true, true><<<L.blocks, dim3(TX, TY), 0, s>>>((const StageArgs*)L.args, L.start, L.nd, b->err);
        else if (L.raw)
          k_b_stage<true, false><<<L.blocks, dim3(TX, TY), 0, s>>>((const StageArgs*)L.args, L.start, L.nd, b->err);
        else if (b->spec)
          k_b_stage<false, true><<<L.blocks, dim3(TX, TY), 0, s>>>((const StageArgs*)L.args, L.start, L.nd, b->err);
        else
          k_b_stage<false, false><<<L.blocks, dim3(TX, TY), 0, s>>>((const StageArgs*)L.args, L.start, L.nd, b->err);
        break;
      case 1:
        if (b->defer)
          k_b_hevi_tmad<<<L.blocks, dim3(32, 4), b->hevi_smem, s>>>((const HeviArgs*)L.args, L.start, L.nd, b->err);
        else if (b->hevi_tma)
          k_b_hevi_tma<<<L.blocks, dim3(32, 4), b->hevi_smem, s>>>((const HeviArgs*)L.args, L.start, L.nd, b->err);
        else
          k_b_hevi<<<L.blocks, dim3(32, 4), b->hevi_smem, s>>>((const HeviArgs*)L.args, L.start, L.nd);
        break;
      case 2:
        if (b->defer) k_b_fix<<<L.blocks, dim3(32, 4), 0, s>>>((const UvArgs*)L.args, L.start, L.nd);
        else k_b_uv<<<L.blocks, dim3(32, 4), 0, s>>>((const UvArgs*)L.args, L.start, L.nd);
        break;
      default:
        k_b_finish<<<L.blocks, dim3(32, 4), 0, s>>>((const FinishArgs*)L.args, L.start, L.nd, b->err);
        break;
    }
  }
}

int mixed_batch_launches(const MixedBatch* b) { return (int)b->seq.size(); }

void mixed_batch_destroy(MixedBatch* b) {
  if (!b) return;
  for (void* p : b->allocs) cudaFree(p);
  delete b;
}

}  // namespace vgb

namespace vgb {
void mixed_set_tune(const Dims& d, const MixedTune& t) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  if (t.stage_levels <= 0 && t.column < 0) g_tune.erase(TuneKey{d.nx, d.ny, d.nz});
  else g_tune[TuneKey{d.nx, d.ny, d.nz}] = t;
}
int mixed_stage_levels(const Dims& d) { return stage_kchunk(d, false); }
}  // namespace vgb
