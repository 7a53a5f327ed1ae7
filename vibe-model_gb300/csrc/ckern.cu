// vibe-model_gb300/csrc/ckern.cu
//
// GPU implementation of the reference's C11 hot-kernel ABI
// (include/vibe/common/c_kernels.h). The host-pointer entry points copy their
// arrays to the device, run the kernel on an internal stream and copy the
// result back; the *_dev entry points work on device pointers on the
// caller's stream. Reductions (CFL max-scan, Neumaier sum) are two-level:
// warp shuffles inside a block, one partial per block in device scratch, and
// a single-block pass that merges the partials in block order, so results are
// deterministic run to run.
#include <atomic>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "cabi_host.cuh"
#include "vibe_c_kernels.h"
#include "vibe_internal.cuh"

namespace {

thread_local std::string g_cerr;

bool device_ok(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return true;
  g_cerr = std::string(what) + ": " + cudaGetErrorString(e);
  return false;
}

int cur_dev() {
  int d = 0;
  cudaGetDevice(&d);
  return d;
}

// ---- per-thread call contexts (cabi_host.cuh) ----------------------------
constexpr int kMaxDev = 64;
std::atomic<unsigned long long> g_allocs{0};

struct Ctx {
  cudaStream_t st = nullptr;
  cudaEvent_t last = nullptr;  // recorded after the last launch that used scr
  bool has_last = false;
  char* pin = nullptr;         // pinned host staging
  size_t pin_n = 0;
  char* dbuf = nullptr;        // device staging of host-pointer calls
  size_t dbuf_n = 0;
  char* scr = nullptr;         // scratch of _dev calls
  size_t scr_n = 0;
};

// One context per (host thread, device); freed when the thread exits (the
// main thread's at process exit, before the CUDA runtime's own teardown).
struct Holder {
  Ctx* c[kMaxDev] = {};
  ~Holder() {
    for (auto*& x : c) {
      if (!x) continue;
      if (x->st) cudaStreamSynchronize(x->st);
      if (x->has_last) cudaEventSynchronize(x->last);
      if (x->pin) cudaFreeHost(x->pin);
      if (x->dbuf) cudaFree(x->dbuf);
      if (x->scr) cudaFree(x->scr);
      if (x->last) cudaEventDestroy(x->last);
      if (x->st) cudaStreamDestroy(x->st);
      delete x;
      x = nullptr;
    }
  }
};
thread_local Holder t_hold;

Ctx* ctx() {
  int d = -1;
  if (!device_ok(cudaGetDevice(&d), "cudaGetDevice")) return nullptr;
  if (d < 0 || d >= kMaxDev) { g_cerr = "device ordinal out of range"; return nullptr; }
  Ctx*& c = t_hold.c[d];
  if (!c) {
    Ctx* n = new Ctx();
    if (!device_ok(cudaStreamCreateWithFlags(&n->st, cudaStreamNonBlocking), "cudaStreamCreate") ||
        !device_ok(cudaEventCreateWithFlags(&n->last, cudaEventDisableTiming), "cudaEventCreate")) {
      if (n->st) cudaStreamDestroy(n->st);
      delete n;
      return nullptr;
    }
    c = n;
  }
  return c;
}

size_t grown(size_t have, size_t need) {
  size_t n = have ? have : (size_t)4096;
  while (n < need) n *= 2;
  return n;
}

inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// ---------------------------------------------------------------------------
// Thomas: one thread per system. Contract c_kernels.h:38-55 with the
// recurrence of thomas_solve (src/time/helmholtz.cpp:71-85); NULL a/c read
// as 0; exact-zero pivots give VIBE_C_ERR_SINGULAR as c_kernels.c:26,34,40.
// cp (the modified super-diagonal) lives in `work` (n per system).
template <typename T>
__device__ int thomas_seq(const T* __restrict__ as, const T* __restrict__ bs, const T* __restrict__ cs,
                          const T* __restrict__ ds, int n, T* __restrict__ xs, T* __restrict__ cp) {
  if (n == 1) {
    if (bs[0] == (T)0) return VIBE_C_ERR_SINGULAR;
    xs[0] = ds[0] / bs[0];
    return VIBE_C_OK;
  }
  T denom = bs[0];
  if (denom == (T)0) return VIBE_C_ERR_SINGULAR;
  cp[0] = (cs ? cs[0] : (T)0) / denom;
  xs[0] = ds[0] / denom;
  for (int k = 1; k < n; ++k) {
    const T am = as ? as[k - 1] : (T)0;
    denom = bs[k] - am * cp[k - 1];
    if (denom == (T)0) return VIBE_C_ERR_SINGULAR;
    xs[k] = (ds[k] - am * xs[k - 1]) / denom;
    if (k < n - 1) cp[k] = (cs ? cs[k] : (T)0) / denom;
  }
  for (int k = n - 1; k-- > 0;) xs[k] = xs[k] - cp[k] * xs[k + 1];
  return VIBE_C_OK;
}

template <typename T>
__global__ void k_thomas_batched(const T* __restrict__ a, const T* __restrict__ b, const T* __restrict__ c,
                                 const T* __restrict__ d, int n, int n_sys, T* __restrict__ x, T* __restrict__ work,
                                 int* __restrict__ status) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n_sys) return;
  const int rc = thomas_seq<T>(a ? a + (size_t)s * (n - 1) : nullptr, b + (size_t)s * n,
                               c ? c + (size_t)s * (n - 1) : nullptr, d + (size_t)s * n, n, x + (size_t)s * n,
                               work + (size_t)s * n);
  if (status) status[s] = rc;
}

// ---------------------------------------------------------------------------
// Tall systems (n > kTallN): one warp per system. The n rows split into 32
// contiguous chunks, one per lane; each lane factors its chunk once (the
// recurrence above) and solves it for three right-hand sides: the chunk's d
// (y), its coupling to the unknown left of the chunk (v, from a at the first
// row) and to the unknown right of it (w, from c at the last row), so that
// x_i = y_i - v_i x_left - w_i x_right on the chunk. The chunks' first and
// last unknowns z_j = (F_j, E_j) then satisfy a 2x2 block-tridiagonal system,
// z_j + [vF; vE]_j E_{j-1} + [wF; wE]_j F_{j+1} = [yF; yE]_j, which lane 0
// solves by block elimination (32 blocks); every lane then reads its two
// neighbours' interface values from shared memory and finishes its chunk.
// The elimination order differs from one sequential sweep, so results agree
// with it to rounding. A chunk starts from its raw diagonal b[r0], so its
// pivots are not the sweep's: a nonsingular system can have a zero or a
// tiny chunk pivot (b[r0] = 0, non-dominant diagonals) or a near-singular
// 2x2 interface block. Whenever a chunk pivot is at most tall_rel (1e-8 in
// FP64, 1e-3 in FP32) of its row's |a| + |b| + |c|, or a block determinant at
// most tall_rel of its terms, lane 0 solves that system again with the single sequential sweep, whose
// contract is the reference's (c_kernels.c:26,34,40): VIBE_C_ERR_SINGULAR
// only on an exactly zero sweep pivot. Scratch: 3n per system (c', v, w).
constexpr int kTallN = 128;
constexpr int kTallWarps = 4;  // systems per block
template <typename T>
__device__ __forceinline__ T tall_rel();
template <>
__device__ __forceinline__ double tall_rel<double>() { return 1e-8; }
template <>
__device__ __forceinline__ float tall_rel<float>() { return 1e-3f; }

template <typename T>
__global__ void __launch_bounds__(32 * kTallWarps) k_thomas_tall(const T* __restrict__ a, const T* __restrict__ b,
                                                                 const T* __restrict__ c, const T* __restrict__ d,
                                                                 int n, int n_sys, T* __restrict__ x,
                                                                 T* __restrict__ work, int* __restrict__ status) {
  __shared__ T sh[kTallWarps][32][6];  // per lane: yF, yE, vF, vE, wF, wE
  __shared__ T zs[kTallWarps][32][2];  // interface solution F_j, E_j
  __shared__ int seq[kTallWarps];  // 1: this system falls back to the sequential sweep
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int s = blockIdx.x * kTallWarps + wid;
  const bool live = s < n_sys;
  const int m = (n + 31) / 32;                   // rows per chunk
  const int r0 = min(lane * m, n), r1 = min(r0 + m, n), L = r1 - r0;
  const int nch = (n + m - 1) / m;               // chunks with rows (lanes >= nch hold none)
  if (lane == 0) seq[wid] = 0;
  __syncwarp();
  const T rel = tall_rel<T>();
  const T* as = (live && a) ? a + (size_t)s * (n - 1) : nullptr;
  const T* bs = live ? b + (size_t)s * n : nullptr;
  const T* cs = (live && c) ? c + (size_t)s * (n - 1) : nullptr;
  const T* ds = live ? d + (size_t)s * n : nullptr;
  T* xs = live ? x + (size_t)s * n : nullptr;
  T* cp = live ? work + (size_t)s * 3 * n : nullptr;
  T* vv = cp ? cp + n : nullptr;
  T* ww = cp ? cp + 2 * n : nullptr;
  bool ok = true;
  if (live && L > 0) {
    // forward elimination of the chunk with the three right-hand sides
    T den = bs[r0];
    const T a0 = (r0 > 0 && as) ? as[r0 - 1] : (T)0;   // coupling to x_{r0-1}
    const T cl = (r1 < n && cs) ? cs[r1 - 1] : (T)0;   // coupling to x_{r1}
    const T c0 = (r0 + 1 < n && cs) ? cs[r0] : (T)0;
    if (!(fabs(den) > rel * (fabs(a0) + fabs(den) + fabs(c0)))) ok = false;
    if (ok) {
      cp[r0] = (r0 + 1 < r1) ? ((cs ? cs[r0] : (T)0) / den) : (T)0;
      xs[r0] = ds[r0] / den;
      vv[r0] = a0 / den;
      ww[r0] = (L == 1) ? cl / den : (T)0;
      for (int k = r0 + 1; k < r1 && ok; ++k) {
        const T am = as ? as[k - 1] : (T)0;
        const T ck = (k + 1 < n && cs) ? cs[k] : (T)0;
        den = bs[k] - am * cp[k - 1];
        if (!(fabs(den) > rel * (fabs(am) + fabs(bs[k]) + fabs(ck)))) { ok = false; break; }
        xs[k] = (ds[k] - am * xs[k - 1]) / den;
        vv[k] = (-am * vv[k - 1]) / den;
        ww[k] = ((k == r1 - 1 ? cl : (T)0) - am * ww[k - 1]) / den;
        if (k < r1 - 1) cp[k] = (cs ? cs[k] : (T)0) / den;
      }
      if (ok)
        for (int k = r1 - 1; k-- > r0;) {
          xs[k] -= cp[k] * xs[k + 1];
          vv[k] -= cp[k] * vv[k + 1];
          ww[k] -= cp[k] * ww[k + 1];
        }
    }
    if (ok) {
      sh[wid][lane][0] = xs[r0];
      sh[wid][lane][1] = xs[r1 - 1];
      sh[wid][lane][2] = vv[r0];
      sh[wid][lane][3] = vv[r1 - 1];
      sh[wid][lane][4] = ww[r0];
      sh[wid][lane][5] = ww[r1 - 1];
    }
  }
  if (!ok) seq[wid] = 1;
  __syncwarp();
  // the interface system, block elimination by lane 0: z_j + Lj z_{j-1} + Uj z_{j+1} = Yj,
  // Lj = [[0, vF], [0, vE]] and Uj = [[wF, 0], [wE, 0]]
  if (live && lane == 0 && !seq[wid]) {
    T C[32][2][2], Y[32][2];
    for (int j = 0; j < nch; ++j) {
      const T* q = sh[wid][j];
      T D00 = 1, D01 = 0, D10 = 0, D11 = 1, r0v = q[0], r1v = q[1];
      if (j > 0) {  // D = I - Lj C_{j-1}, rhs = Yj - Lj Y_{j-1}; Lj picks row 1 (E) of the previous block
        D00 -= q[2] * C[j - 1][1][0];
        D01 -= q[2] * C[j - 1][1][1];
        D10 -= q[3] * C[j - 1][1][0];
        D11 -= q[3] * C[j - 1][1][1];
        r0v -= q[2] * Y[j - 1][1];
        r1v -= q[3] * Y[j - 1][1];
      }
      const T det = D00 * D11 - D01 * D10;
      if (!(fabs(det) > rel * (fabs(D00 * D11) + fabs(D01 * D10)))) { seq[wid] = 1; break; }
      const T i00 = D11 / det, i01 = -D01 / det, i10 = -D10 / det, i11 = D00 / det;
      // C_j = D^-1 Uj (Uj acts on F_{j+1}: column 0), Y_j = D^-1 rhs
      const T u0 = (j + 1 < nch) ? q[4] : (T)0, u1 = (j + 1 < nch) ? q[5] : (T)0;
      C[j][0][0] = i00 * u0 + i01 * u1;
      C[j][1][0] = i10 * u0 + i11 * u1;
      C[j][0][1] = 0;
      C[j][1][1] = 0;
      Y[j][0] = i00 * r0v + i01 * r1v;
      Y[j][1] = i10 * r0v + i11 * r1v;
    }
    if (!seq[wid])
      for (int j = nch - 1; j >= 0; --j) {
        T f = Y[j][0], e = Y[j][1];
        if (j + 1 < nch) {  // z_j = Y_j - C_j z_{j+1}, C_j acting on F_{j+1}
          f -= C[j][0][0] * zs[wid][j + 1][0];
          e -= C[j][1][0] * zs[wid][j + 1][0];
        }
        zs[wid][j][0] = f;
        zs[wid][j][1] = e;
      }
  }
  __syncwarp();
  if (seq[wid]) {  // the sequential sweep over the whole system, on lane 0
    if (live && lane == 0) {
      const int rc = thomas_seq<T>(as, bs, cs, ds, n, xs, cp);
      if (status) status[s] = rc;
    }
    return;
  }
  if (live && L > 0) {
    const T xl = (lane > 0) ? zs[wid][lane - 1][1] : (T)0;        // E of the chunk to the left
    const T xr = (lane + 1 < nch) ? zs[wid][lane + 1][0] : (T)0;  // F of the chunk to the right
    for (int k = r0; k < r1; ++k) xs[k] = xs[k] - vv[k] * xl - ww[k] * xr;
  }
  if (live && lane == 0 && status) status[s] = VIBE_C_OK;
}

// WENO5 (c_kernels.c:64-104), one thread per stencil
template <typename T>
__device__ void weno5_d(T qm2, T qm1, T q0, T q1, T q2, T* ql, T* qr) {
  const T eps = (T)1e-6, d0 = (T)0.1, d1 = (T)0.6, d2 = (T)0.3;
  const T t12 = (T)13 / (T)12, q4 = (T)0.25;
  const T v0 = ((T)2.0 * qm2 - (T)7.0 * qm1 + (T)11.0 * q0) / (T)6;
  const T v1 = (-qm1 + (T)5.0 * q0 + (T)2.0 * q1) / (T)6;
  const T v2 = ((T)2.0 * q0 + (T)5.0 * q1 - q2) / (T)6;
  const T b0 = t12 * (qm2 - (T)2.0 * qm1 + q0) * (qm2 - (T)2.0 * qm1 + q0) +
                    q4 * (qm2 - (T)4.0 * qm1 + (T)3.0 * q0) * (qm2 - (T)4.0 * qm1 + (T)3.0 * q0);
  const T b1 = t12 * (qm1 - (T)2.0 * q0 + q1) * (qm1 - (T)2.0 * q0 + q1) + q4 * (qm1 - q1) * (qm1 - q1);
  const T b2 = t12 * (q0 - (T)2.0 * q1 + q2) * (q0 - (T)2.0 * q1 + q2) +
                    q4 * ((T)3.0 * q0 - (T)4.0 * q1 + q2) * ((T)3.0 * q0 - (T)4.0 * q1 + q2);
  const T a0 = d0 / ((eps + b0) * (eps + b0)), a1 = d1 / ((eps + b1) * (eps + b1)),
               a2 = d2 / ((eps + b2) * (eps + b2));
  *ql = (a0 * v0 + a1 * v1 + a2 * v2) / (a0 + a1 + a2);
  const T u0 = ((T)2.0 * q2 - (T)7.0 * q1 + (T)11.0 * q0) / (T)6;
  const T u1 = (-q1 + (T)5.0 * q0 + (T)2.0 * qm1) / (T)6;
  const T u2 = ((T)2.0 * q0 + (T)5.0 * qm1 - qm2) / (T)6;
  const T g0 = t12 * (q2 - (T)2.0 * q1 + q0) * (q2 - (T)2.0 * q1 + q0) +
                    q4 * (q2 - (T)4.0 * q1 + (T)3.0 * q0) * (q2 - (T)4.0 * q1 + (T)3.0 * q0);
  const T g1 = t12 * (q1 - (T)2.0 * q0 + qm1) * (q1 - (T)2.0 * q0 + qm1) + q4 * (q1 - qm1) * (q1 - qm1);
  const T g2 = t12 * (q0 - (T)2.0 * qm1 + qm2) * (q0 - (T)2.0 * qm1 + qm2) +
                    q4 * ((T)3.0 * q0 - (T)4.0 * qm1 + qm2) * ((T)3.0 * q0 - (T)4.0 * qm1 + qm2);
  const T c0 = d0 / ((eps + g0) * (eps + g0)), c1 = d1 / ((eps + g1) * (eps + g1)),
               c2 = d2 / ((eps + g2) * (eps + g2));
  *qr = (c0 * u0 + c1 * u1 + c2 * u2) / (c0 + c1 + c2);
}
template <typename T>
__global__ void k_weno_batched(const T* __restrict__ q, size_t n, T* __restrict__ ql, T* __restrict__ qr) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x)
    weno5_d(q[5 * e], q[5 * e + 1], q[5 * e + 2], q[5 * e + 3], q[5 * e + 4], ql + e, qr + e);
}

// bilinear (c_kernels.c:108-144) on one level plane held in `plane`
template <typename T>
__global__ void k_bilinear(const T* __restrict__ plane, int halo, int nsx, int nsy, T xi, T yj, T* out) {
  const int nxi = nsx - 2 * halo, nyi = nsy - 2 * halo;
  const int i0 = (int)floor(xi), j0 = (int)floor(yj);
  const T wx = xi - (T)i0, wy = yj - (T)j0;
  // the reference's clamp order (c_kernels.c:128-135): up to 0 first, then
  // down to n-1, so a grid without interior points reads its last halo point
  auto clamp = [](int v, int n) { v = v < 0 ? 0 : v; return v > n - 1 ? n - 1 : v; };
  const int ia = clamp(i0, nxi), ib = clamp(i0 + 1, nxi);
  const int ja = clamp(j0, nyi), jb = clamp(j0 + 1, nyi);
  auto at = [&](int i, int j) { return plane[(size_t)(j + halo) * nsx + (size_t)(i + halo)]; };
  const T q00 = at(ia, ja), q10 = at(ib, ja), q01 = at(ia, jb), q11 = at(ib, jb);
  *out = (q00 + wx * (q10 - q00)) + wy * ((q01 + wx * (q11 - q01)) - (q00 + wx * (q10 - q00)));
}

// ---- reductions ----------------------------------------------------------
template <typename T>
struct Neu {
  T s, c;
};
// Neumaier add of one value (c_kernels.c:195-203)
template <typename T>
__device__ __forceinline__ void neu_add(Neu<T>& a, T x) {
  const T t = a.s + x;
  if (fabs(a.s) >= fabs(x)) a.c += (a.s - t) + x;
  else a.c += (x - t) + a.s;
  a.s = t;
}
// merge of two compensated partial sums: add b.s with compensation, then b.c
template <typename T>
__device__ __forceinline__ Neu<T> neu_merge(Neu<T> a, Neu<T> b) {
  neu_add(a, b.s);
  a.c += b.c;
  return a;
}
template <typename T>
__device__ Neu<T> neu_block(Neu<T> v) {
  __shared__ T sh_s[32], sh_c[32];
  for (int off = 16; off > 0; off >>= 1) {
    Neu<T> o;
    o.s = __shfl_down_sync(0xffffffffu, v.s, off);
    o.c = __shfl_down_sync(0xffffffffu, v.c, off);
    v = neu_merge(v, o);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) { sh_s[warp] = v.s; sh_c[warp] = v.c; }
  __syncthreads();
  const int nw = (blockDim.x + 31) >> 5;
  if (warp == 0) {
    v.s = lane < nw ? sh_s[lane] : (T)0;
    v.c = lane < nw ? sh_c[lane] : (T)0;
    for (int off = 16; off > 0; off >>= 1) {
      Neu<T> o;
      o.s = __shfl_down_sync(0xffffffffu, v.s, off);
      o.c = __shfl_down_sync(0xffffffffu, v.c, off);
      v = neu_merge(v, o);
    }
  }
  return v;
}
// each block sums a contiguous chunk; partials[2*block] = (s, c)
template <typename T>
__global__ void k_neu_partial(const T* __restrict__ x, size_t n, size_t chunk, T* __restrict__ partials) {
  const size_t lo = (size_t)blockIdx.x * chunk, hi = lo + chunk < n ? lo + chunk : n;
  Neu<T> v{(T)0, (T)0};
  for (size_t e = lo + threadIdx.x; e < hi; e += blockDim.x) neu_add(v, x[e]);
  v = neu_block(v);
  if (threadIdx.x == 0) { partials[2 * blockIdx.x] = v.s; partials[2 * blockIdx.x + 1] = v.c; }
}
template <typename T>
__global__ void k_neu_final(const T* __restrict__ partials, int nb, T* __restrict__ out) {
  Neu<T> v{(T)0, (T)0};
  for (int b = threadIdx.x; b < nb; b += blockDim.x) v = neu_merge(v, Neu<T>{partials[2 * b], partials[2 * b + 1]});
  v = neu_block(v);
  if (threadIdx.x == 0) *out = v.s + v.c;
}

// CFL scan (c_kernels.c:148-186): per cell dz = max(dzeta[k]*scale, 1),
// speed = sqrt(u^2+v^2+w^2), cfl = dt*(|u|/dx + |v|/dy + |w|/dz); block maxima
// of (cfl, speed) and min of dz, then one block merges.
template <typename T>
__device__ __forceinline__ void max3_block(T& a, T& b, T& c) {  // max, max, min
  __shared__ T s1[32], s2[32], s3[32];
  for (int off = 16; off > 0; off >>= 1) {
    a = fmax(a, __shfl_down_sync(0xffffffffu, a, off));
    b = fmax(b, __shfl_down_sync(0xffffffffu, b, off));
    c = fmin(c, __shfl_down_sync(0xffffffffu, c, off));
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  if (lane == 0) { s1[warp] = a; s2[warp] = b; s3[warp] = c; }
  __syncthreads();
  if (warp == 0) {
    a = lane < nw ? s1[lane] : (T)0;
    b = lane < nw ? s2[lane] : (T)0;
    c = lane < nw ? s3[lane] : (T)1e30;
    for (int off = 16; off > 0; off >>= 1) {
      a = fmax(a, __shfl_down_sync(0xffffffffu, a, off));
      b = fmax(b, __shfl_down_sync(0xffffffffu, b, off));
      c = fmin(c, __shfl_down_sync(0xffffffffu, c, off));
    }
  }
}
template <typename T>
__global__ void k_cfl_partial(const T* __restrict__ u, const T* __restrict__ v, const T* __restrict__ w,
                              const T* __restrict__ dzeta, const T* __restrict__ zs, int nx, int ny, int nz, T dx, T dy,
                              T z_top, T dt, T* __restrict__ partials) {
  const size_t n = (size_t)nx * ny * nz, nxy = (size_t)nx * ny;  // (no negative dimension reaches here)
  // the largest squared speed, one square root at the end: a correctly
  // rounded square root is monotone, so the maximum of the roots is the root
  // of the maximum, bit for bit
  T worst = 0, mw2 = 0, mdz = (T)1e30;
  const size_t S = (size_t)gridDim.x * blockDim.x;
  size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e < n) {
    // the cell's level and column, stepped along with e (no division per cell)
    size_t k = e / nxy, col = e - k * nxy;
    const size_t sk = S / nxy, sc = S - sk * nxy;
    for (; e < n; e += S) {
      const T uu = u[e], vv = v[e], ww = w[e];
      const T scale = zs ? (z_top - zs[col]) : z_top;
      T dz = dzeta[k] * scale;
      if (dz < (T)1) dz = (T)1;
      mdz = fmin(mdz, dz);
      mw2 = fmax(mw2, uu * uu + vv * vv + ww * ww);
      worst = fmax(worst, dt * (fabs(uu) / dx + fabs(vv) / dy + fabs(ww) / dz));
      col += sc;
      k += sk;
      if (col >= nxy) {
        col -= nxy;
        ++k;
      }
    }
  }
  T mw = sqrt(mw2);
  max3_block(worst, mw, mdz);
  if (threadIdx.x == 0) {
    partials[3 * blockIdx.x] = worst;
    partials[3 * blockIdx.x + 1] = mw;
    partials[3 * blockIdx.x + 2] = mdz;
  }
}
template <typename T>
__global__ void k_cfl_final(const T* __restrict__ partials, int nb, T* __restrict__ out3) {
  T a = 0, b = 0, c = (T)1e30;
  for (int e = threadIdx.x; e < nb; e += blockDim.x) {
    a = fmax(a, partials[3 * e]);
    b = fmax(b, partials[3 * e + 1]);
    c = fmin(c, partials[3 * e + 2]);
  }
  max3_block(a, b, c);
  if (threadIdx.x == 0) {
    out3[0] = a;
    out3[1] = b;
    out3[2] = (c > (T)1e29) ? (T)0 : c;
  }
}

// flux advection (c_kernels.c:209-286), one thread per cell
template <typename T>
__global__ void k_flux_adv(const T* __restrict__ q, const T* __restrict__ rho, const T* __restrict__ u,
                           const T* __restrict__ v, const T* __restrict__ w, const T* __restrict__ dzeta,
                           const T* __restrict__ zs, int nx, int ny, int nz, T dx, T dy, T z_top, T* __restrict__ dqdt) {
  const size_t nxy = (size_t)nx * ny, n = nxy * nz;
  const T inv_dx = (T)1 / dx, inv_dy = (T)1 / dy, hf = (T)0.5;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(idx / nxy);
    const int j = (int)((idx / nx) % ny);
    const int i = (int)(idx % nx);
    const size_t base_k = (size_t)k * nxy;
    const T scale = zs ? (z_top - zs[(size_t)j * nx + i]) : z_top;
    T dz = dzeta[k] * scale;
    if (dz < (T)1) dz = (T)1;
    const size_t c = idx;
    const size_t e = base_k + (size_t)j * nx + (size_t)((i + 1) % nx);
    const size_t ws = base_k + (size_t)j * nx + (size_t)((i + nx - 1) % nx);
    const T fxE = u[e] * (hf * (rho[c] + rho[e])) * (hf * (q[c] + q[e]));
    const T fxW = u[c] * (hf * (rho[ws] + rho[c])) * (hf * (q[ws] + q[c]));
    const size_t nn = base_k + (size_t)((j + 1) % ny) * nx + (size_t)i;
    const size_t ss = base_k + (size_t)((j + ny - 1) % ny) * nx + (size_t)i;
    const T fyN = v[nn] * (hf * (rho[c] + rho[nn])) * (hf * (q[c] + q[nn]));
    const T fyS = v[c] * (hf * (rho[ss] + rho[c])) * (hf * (q[ss] + q[c]));
    T fzT = 0, fzB = 0;
    if (k > 0 && k + 1 < nz) {
      const size_t t = c + nxy, b = c - nxy;
      fzT = w[t] * (hf * (rho[c] + rho[t])) * (hf * (q[c] + q[t]));
      fzB = w[c] * (hf * (rho[b] + rho[c])) * (hf * (q[b] + q[c]));
    }
    const T div = (fxE - fxW) * inv_dx + (fyN - fyS) * inv_dy + (fzT - fzB) / dz;
    const T rr = (rho[idx] > (T)1e-12) ? rho[idx] : (T)1e-12;
    dqdt[idx] = -div / rr;
  }
}

// ---- allocation-free batched Thomas ------------------------------------
// Some callers of this library may not allocate device memory at all: a host
// model whose own allocator has reserved the device's memory and forbids any
// other allocation, or a time-critical step loop in which a cudaMalloc or
// cudaFree (both can synchronise the whole device) is not acceptable. For
// them, vibe_tridiagonal_solve_batched_f64_dev_noalloc keeps its Thomas
// workspace (the modified super-diagonal, n doubles per system) in this
// fixed device array instead of the allocated scratch buffer. The array is
// sized here, once, and every GPU that loads the library holds it until the
// process exits. It always runs the one-thread-per-system sweep
// (k_thomas_batched), also for n > 128 where the allocating _dev form runs
// the warp-per-system solver: there the two agree to rounding, and this
// form's singular test is the sweep's exact-zero pivot.
constexpr size_t kNoAllocThomasDoubles = (size_t)1 << 18;  // 2 MiB: n * n_sys <= 262144
static __device__ __align__(256) double g_noalloc_thomas_work[kNoAllocThomasDoubles];
// Device address of that array per device. Host code only sees a host-side
// stand-in for the symbol; the address a kernel may use comes from
// cudaGetSymbolAddress, called with the device current, on the first call per
// device, and is kept for the life of the process: a process that resets a
// device (cudaDeviceReset) loads the module into a new context there, and
// must not call this entry point on that device afterwards.
std::mutex g_noalloc_mu;
double* g_noalloc_ptr[64] = {};

constexpr int kRedBlocks = 304;  // 2 x 152 SMs
constexpr int kRedThreads = 256;

// ---- entry points, one template per ABI function: T = double (the
// reference's *_f64 names) or float (the *_f32 twins its header reserves,
// c_kernels.h:15-16). The _dev forms take their scratch from the calling
// thread's DevScratch; the host forms stage everything through one HostCall
// (cabi_host.cuh) and allocate nothing once the thread's buffers are large
// enough. ----
using vgb_cabi::DevScratch;
using vgb_cabi::HostCall;

size_t thomas_work(int n, int n_sys) { return (size_t)n * (size_t)n_sys * (n > kTallN ? 3 : 1); }

template <typename T>
int thomas_launch(const T* a, const T* b, const T* c, const T* d, int n, int n_sys, T* x, T* work, int* status,
                  cudaStream_t st) {
  if (n > kTallN)
    k_thomas_tall<T><<<(n_sys + kTallWarps - 1) / kTallWarps, 32 * kTallWarps, 0, st>>>(a, b, c, d, n, n_sys, x,
                                                                                       work, status);
  else
    k_thomas_batched<T><<<(n_sys + 127) / 128, 128, 0, st>>>(a, b, c, d, n, n_sys, x, work, status);
  return device_ok(cudaGetLastError(), "thomas launch") ? VIBE_C_OK : VIBE_C_ERR_DEVICE;
}

template <typename T>
int thomas_batched_dev(const T* a, const T* b, const T* c, const T* d, int n, int n_sys, T* x, int* status,
                       vibe_stream_t stream) {
  if (n <= 0 || n_sys < 0 || b == nullptr || d == nullptr || x == nullptr) return VIBE_C_ERR_BAD_ARG;
  if (n_sys == 0) return VIBE_C_OK;
  DevScratch w(thomas_work(n, n_sys) * sizeof(T), (cudaStream_t)stream);
  if (!w.get()) return VIBE_C_ERR_DEVICE;
  int rc = thomas_launch<T>(a, b, c, d, n, n_sys, x, (T*)w.get(), status, (cudaStream_t)stream);
  if (!w.release() && rc == VIBE_C_OK) rc = VIBE_C_ERR_DEVICE;
  return rc;
}

template <typename T>
int thomas_batched_host(const T* a, const T* b, const T* c, const T* d, int n, int n_sys, T* x) {
  if (n <= 0 || n_sys < 0 || b == nullptr || d == nullptr || x == nullptr) return VIBE_C_ERR_BAD_ARG;
  if (n_sys == 0) return VIBE_C_OK;
  const size_t e = sizeof(T), nn = (size_t)n * n_sys, no = (size_t)(n - 1) * n_sys;
  HostCall hc;
  const int ia = hc.add(a, no * e, HostCall::kIn), ib = hc.add(b, nn * e, HostCall::kIn);
  const int ic = hc.add(c, no * e, HostCall::kIn), id = hc.add(d, nn * e, HostCall::kIn);
  // x comes back through the staging buffer and is copied out only for the
  // systems that solved: a failed system's x stays as it was, as in the
  // reference, which returns before it writes x (c_kernels.c:26,34,40)
  const int ix = hc.add(nullptr, nn * e, HostCall::kOut);
  const int is = hc.add(nullptr, (size_t)n_sys * sizeof(int), HostCall::kOut);
  const int iw = hc.add(nullptr, thomas_work(n, n_sys) * e, HostCall::kScratch);
  if (!hc.commit()) return VIBE_C_ERR_DEVICE;
  int rc = thomas_launch<T>(hc.dev<T>(ia), hc.dev<T>(ib), hc.dev<T>(ic), hc.dev<T>(id), n, n_sys, hc.dev<T>(ix),
                            hc.dev<T>(iw), hc.dev<int>(is), hc.stream());
  if (!hc.finish()) return VIBE_C_ERR_DEVICE;
  if (rc) return rc;
  const int* sv = (const int*)hc.host(is);
  const T* xv = (const T*)hc.host(ix);
  for (int q = 0; q < n_sys; ++q) {
    if (sv[q] == VIBE_C_OK)
      std::memcpy(x + (size_t)q * n, xv + (size_t)q * n, (size_t)n * e);
    else if (rc == VIBE_C_OK)
      rc = sv[q];
  }
  return rc;
}

template <typename T>
int weno_batched_dev(const T* q, size_t n, T* q_left, T* q_right, vibe_stream_t stream) {
  if (!q || !q_left || !q_right) return VIBE_C_ERR_BAD_ARG;
  if (n == 0) return VIBE_C_OK;
  const int blocks = (int)((n + 255) / 256 < 65535 ? (n + 255) / 256 : 65535);
  k_weno_batched<T><<<blocks, 256, 0, (cudaStream_t)stream>>>(q, n, q_left, q_right);
  return device_ok(cudaGetLastError(), "weno launch") ? VIBE_C_OK : VIBE_C_ERR_DEVICE;
}

template <typename T>
void weno_host(T qm2, T qm1, T q0, T q1, T q2, T* q_left, T* q_right) {
  if (q_left == nullptr || q_right == nullptr) return;
  const T q[5] = {qm2, qm1, q0, q1, q2};
  const size_t e = sizeof(T);
  HostCall hc;
  const int iq = hc.add(q, 5 * e, HostCall::kIn), il = hc.add(q_left, e, HostCall::kOut),
            ir = hc.add(q_right, e, HostCall::kOut);
  bool ok = hc.commit();
  ok = ok && weno_batched_dev<T>(hc.dev<T>(iq), 1, hc.dev<T>(il), hc.dev<T>(ir), (vibe_stream_t)hc.stream()) ==
                 VIBE_C_OK;
  ok = hc.finish() && ok;
  if (!ok) *q_left = *q_right = (T)NAN;
}

template <typename T>
T bilinear_host(const T* f, int halo, int nsx, int nsy, int nz, T xi, T yj, int k) {
  if (f == nullptr || nz <= 0) return (T)0;
  if (halo < 0 || nsx < halo + 1 || nsy < halo + 1) {  // the clamped point would lie outside the plane
    g_cerr = "bilinear: halo < 0 or a plane narrower than halo + 1";
    return (T)NAN;
  }
  if (k < 0) k = 0;
  if (k >= nz) k = nz - 1;
  const size_t plane = (size_t)nsx * nsy, e = sizeof(T);
  T r = (T)NAN;
  HostCall hc;
  const int ip = hc.add(f + (size_t)(k + halo) * plane, plane * e, HostCall::kIn), io = hc.add(&r, e, HostCall::kOut);
  bool ok = hc.commit();
  if (ok) {
    k_bilinear<T><<<1, 1, 0, hc.stream()>>>(hc.dev<T>(ip), halo, nsx, nsy, xi, yj, hc.dev<T>(io));
    ok = device_ok(cudaGetLastError(), "bilinear launch");
  }
  ok = hc.finish() && ok;
  return ok ? r : (T)NAN;
}

template <typename T>
int cfl_launch(const T* u, const T* v, const T* w, const T* dzeta, const T* zs, int nx, int ny, int nz, T dx, T dy,
               T z_top, T dt, T* out3, T* part, cudaStream_t st) {
  k_cfl_partial<T><<<kRedBlocks, kRedThreads, 0, st>>>(u, v, w, dzeta, zs, nx, ny, nz, dx, dy, z_top, dt, part);
  k_cfl_final<T><<<1, kRedThreads, 0, st>>>(part, kRedBlocks, out3);
  return device_ok(cudaGetLastError(), "cfl launch") ? VIBE_C_OK : VIBE_C_ERR_DEVICE;
}

template <typename T>
int cfl_dev(const T* u, const T* v, const T* w, const T* dzeta, const T* zs, int nx, int ny, int nz, T dx, T dy,
            T z_top, T dt, T* out3, vibe_stream_t stream) {
  if (!u || !v || !w || !dzeta || !out3 || nx < 0 || ny < 0 || nz < 0) return VIBE_C_ERR_BAD_ARG;
  DevScratch part((size_t)3 * kRedBlocks * sizeof(T), (cudaStream_t)stream);
  if (!part.get()) return VIBE_C_ERR_DEVICE;
  int rc = cfl_launch<T>(u, v, w, dzeta, zs, nx, ny, nz, dx, dy, z_top, dt, out3, (T*)part.get(),
                         (cudaStream_t)stream);
  if (!part.release() && rc == VIBE_C_OK) rc = VIBE_C_ERR_DEVICE;
  return rc;
}

template <typename T>
T cfl_host(const T* u, const T* v, const T* w, const T* dzeta, const T* zs, int nx, int ny, int nz, T dx, T dy, T z_top,
           T dt, T* max_wind_out, T* min_dz_out) {
  if (u == nullptr || v == nullptr || w == nullptr || dzeta == nullptr) return (T)0;
  if (nx <= 0 || ny <= 0 || nz <= 0) {  // no cells: the reference's loops run zero times
    if (max_wind_out) *max_wind_out = (T)0;
    if (min_dz_out) *min_dz_out = (T)0;
    return (T)0;
  }
  const size_t e = sizeof(T);
  const size_t n = (size_t)nx * ny * nz, nzp = (size_t)nz, nxy = (size_t)nx * ny;
  T r[3] = {(T)NAN, (T)NAN, (T)NAN};
  HostCall hc;
  const int iu = hc.add(u, n * e, HostCall::kIn), iv = hc.add(v, n * e, HostCall::kIn),
            iw = hc.add(w, n * e, HostCall::kIn), iz = hc.add(dzeta, nzp * e, HostCall::kIn),
            izs = hc.add(zs, zs ? nxy * e : 0, HostCall::kIn), io = hc.add(r, 3 * e, HostCall::kOut),
            ip = hc.add(nullptr, (size_t)3 * kRedBlocks * e, HostCall::kScratch);
  bool ok = hc.commit();
  ok = ok && cfl_launch<T>(hc.dev<T>(iu), hc.dev<T>(iv), hc.dev<T>(iw), hc.dev<T>(iz), hc.dev<T>(izs), nx, ny, nz, dx,
                           dy, z_top, dt, hc.dev<T>(io), hc.dev<T>(ip), hc.stream()) == VIBE_C_OK;
  ok = hc.finish() && ok;
  if (!ok) return (T)NAN;
  if (max_wind_out) *max_wind_out = r[1];
  if (min_dz_out) *min_dz_out = r[2];
  return r[0];
}

template <typename T>
int neu_launch(const T* x, size_t n, T* out, T* part, cudaStream_t st) {
  const size_t chunk = (n + kRedBlocks - 1) / kRedBlocks;
  k_neu_partial<T><<<kRedBlocks, kRedThreads, 0, st>>>(x, n, chunk > 0 ? chunk : 1, part);
  k_neu_final<T><<<1, kRedThreads, 0, st>>>(part, kRedBlocks, out);
  return device_ok(cudaGetLastError(), "neumaier launch") ? VIBE_C_OK : VIBE_C_ERR_DEVICE;
}

template <typename T>
int neu_dev(const T* x, size_t n, T* out, vibe_stream_t stream) {
  if (!x || !out) return VIBE_C_ERR_BAD_ARG;
  DevScratch part((size_t)2 * kRedBlocks * sizeof(T), (cudaStream_t)stream);
  if (!part.get()) return VIBE_C_ERR_DEVICE;
  int rc = neu_launch<T>(x, n, out, (T*)part.get(), (cudaStream_t)stream);
  if (!part.release() && rc == VIBE_C_OK) rc = VIBE_C_ERR_DEVICE;
  return rc;
}

template <typename T>
T neu_host(const T* x, size_t n) {
  if (x == nullptr) return (T)0;
  const size_t e = sizeof(T);
  T r = (T)NAN;
  HostCall hc;
  const int ix = hc.add(x, n * e, HostCall::kIn), io = hc.add(&r, e, HostCall::kOut),
            ip = hc.add(nullptr, (size_t)2 * kRedBlocks * e, HostCall::kScratch);
  bool ok = hc.commit();
  ok = ok && neu_launch<T>(hc.dev<T>(ix), n, hc.dev<T>(io), hc.dev<T>(ip), hc.stream()) == VIBE_C_OK;
  ok = hc.finish() && ok;
  return ok ? r : (T)NAN;
}

template <typename T>
int flux_dev(const T* q, const T* rho, const T* u, const T* v, const T* w, const T* dzeta, const T* zs, int nx, int ny,
             int nz, T dx, T dy, T z_top, T* dqdt, vibe_stream_t stream) {
  if (!q || !rho || !u || !v || !w || !dzeta || !dqdt || nx < 0 || ny < 0 || nz < 0) return VIBE_C_ERR_BAD_ARG;
  const size_t n = (size_t)nx * ny * nz;
  if (n == 0) return VIBE_C_OK;
  const int blocks = (int)((n + 255) / 256 < 65535 ? (n + 255) / 256 : 65535);
  k_flux_adv<T><<<blocks, 256, 0, (cudaStream_t)stream>>>(q, rho, u, v, w, dzeta, zs, nx, ny, nz, dx, dy, z_top, dqdt);
  return device_ok(cudaGetLastError(), "flux advection launch") ? VIBE_C_OK : VIBE_C_ERR_DEVICE;
}

template <typename T>
void flux_host(const T* q, const T* rho, const T* u, const T* v, const T* w, const T* dzeta, const T* zs, int nx, int ny,
               int nz, T dx, T dy, T z_top, T* dqdt) {
  if (q == nullptr || rho == nullptr || u == nullptr || v == nullptr || w == nullptr || dzeta == nullptr ||
      dqdt == nullptr)
    return;
  if (nx <= 0 || ny <= 0 || nz <= 0) return;  // no cells: the reference's loops run zero times
  const size_t n = (size_t)nx * ny * nz, e = sizeof(T);
  HostCall hc;
  const int iq = hc.add(q, n * e, HostCall::kIn), ir = hc.add(rho, n * e, HostCall::kIn),
            iu = hc.add(u, n * e, HostCall::kIn), iv = hc.add(v, n * e, HostCall::kIn),
            iw = hc.add(w, n * e, HostCall::kIn), iz = hc.add(dzeta, (size_t)nz * e, HostCall::kIn),
            izs = hc.add(zs, zs ? (size_t)nx * ny * e : 0, HostCall::kIn), io = hc.add(dqdt, n * e, HostCall::kOut);
  bool ok = hc.commit();
  ok = ok && flux_dev<T>(hc.dev<T>(iq), hc.dev<T>(ir), hc.dev<T>(iu), hc.dev<T>(iv), hc.dev<T>(iw), hc.dev<T>(iz),
                         hc.dev<T>(izs), nx, ny, nz, dx, dy, z_top, hc.dev<T>(io), (vibe_stream_t)hc.stream()) ==
                 VIBE_C_OK;
  hc.finish();
}

}  // namespace

// ---- vgb_cabi: the call machinery declared in cabi_host.cuh ----
namespace vgb_cabi {

void set_error(const char* what, cudaError_t e) { device_ok(e, what); }
unsigned long long allocations() { return g_allocs.load(); }

HostCall::HostCall() {
  Ctx* c = ctx();
  ctx_ = c;
  ok_ = c != nullptr;
}

int HostCall::add(const void* h, size_t bytes, Kind kind) {
  Arg a{h, bytes, 0, kind, (kind == kIn || kind == kInOut) && h == nullptr};
  args_.push_back(a);
  return (int)args_.size() - 1;
}

cudaStream_t HostCall::stream() const { return ctx_ ? static_cast<Ctx*>(ctx_)->st : nullptr; }

// Layout in the device buffer: [inputs | in-outs | outputs | scratch]; the
// pinned buffer mirrors the first three regions. One copy moves
// [0, end of in-outs) to the device, one copy moves [in-outs, outputs) back.
bool HostCall::commit() {
  if (!ok_) return false;
  Ctx* c = static_cast<Ctx*>(ctx_);
  size_t off = 0;
  for (int k = kIn; k <= kScratch; ++k) {
    if (k == kInOut) d2h_beg_ = off;
    for (auto& a : args_)
      if (a.kind == k && !a.absent) {
        a.off = off;
        off = align256(off + a.bytes);
      }
    if (k == kInOut) h2d_end_ = off;
    if (k == kOut) d2h_end_ = off;
  }
  const size_t total = off > 0 ? off : 256;
  if (c->dbuf_n < total) {
    if (c->dbuf) cudaFree(c->dbuf);
    c->dbuf = nullptr;
    const size_t n = grown(c->dbuf_n, total);
    c->dbuf_n = 0;
    ++g_allocs;
    if (!device_ok(cudaMalloc(&c->dbuf, n), "cudaMalloc (staging)")) return ok_ = false;
    c->dbuf_n = n;
  }
  if (c->pin_n < d2h_end_) {
    if (c->pin) cudaFreeHost(c->pin);
    c->pin = nullptr;
    const size_t n = grown(c->pin_n, d2h_end_);
    c->pin_n = 0;
    ++g_allocs;
    if (!device_ok(cudaMallocHost(&c->pin, n), "cudaMallocHost (staging)")) return ok_ = false;
    c->pin_n = n;
  }
  base_ = c->dbuf;
  for (const auto& a : args_)
    if ((a.kind == kIn || a.kind == kInOut) && !a.absent && a.bytes) std::memcpy(c->pin + a.off, a.h, a.bytes);
  if (h2d_end_ && !device_ok(cudaMemcpyAsync(c->dbuf, c->pin, h2d_end_, cudaMemcpyHostToDevice, c->st), "H2D"))
    return ok_ = false;
  return true;
}

bool HostCall::finish() {
  if (!ctx_) return false;
  Ctx* c = static_cast<Ctx*>(ctx_);
  bool good = ok_;
  if (good && d2h_end_ > d2h_beg_)
    good = device_ok(cudaMemcpyAsync(c->pin + d2h_beg_, c->dbuf + d2h_beg_, d2h_end_ - d2h_beg_,
                                     cudaMemcpyDeviceToHost, c->st),
                     "D2H");
  // always wait: the staging buffers must be idle before the thread's next call
  good = device_ok(cudaStreamSynchronize(c->st), "sync") && good;
  if (good)
    for (const auto& a : args_)
      if ((a.kind == kInOut || a.kind == kOut) && a.h && a.bytes)
        std::memcpy(const_cast<void*>(a.h), c->pin + a.off, a.bytes);
  return ok_ = good;
}

const void* HostCall::host(int id) const {
  return ctx_ ? static_cast<Ctx*>(ctx_)->pin + args_[id].off : nullptr;
}

DevScratch::DevScratch(size_t bytes, cudaStream_t stream) : s_(stream) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (!device_ok(cudaStreamIsCapturing(stream, &cs), "cudaStreamIsCapturing")) return;
  if (cs != cudaStreamCaptureStatusNone) {  // inside a capture: graph-owned, stream-ordered memory
    graph_ = true;
    if (!device_ok(cudaMallocAsync(&p_, bytes > 0 ? bytes : 256, stream), "cudaMallocAsync (captured scratch)"))
      p_ = nullptr;
    return;
  }
  Ctx* c = ctx();
  if (!c) return;
  if (c->scr_n < bytes) {
    // the old buffer goes once its last user has finished
    if (c->has_last && !device_ok(cudaEventSynchronize(c->last), "scratch wait")) return;
    if (c->scr) cudaFree(c->scr);
    c->scr = nullptr;
    const size_t n = grown(c->scr_n, bytes);
    c->scr_n = 0;
    ++g_allocs;
    if (!device_ok(cudaMalloc(&c->scr, n), "cudaMalloc (scratch)")) return;
    c->scr_n = n;
  }
  // after the previous user of this thread's scratch, whatever its stream
  if (c->has_last && !device_ok(cudaStreamWaitEvent(stream, c->last, 0), "scratch order")) return;
  p_ = c->scr;
}

bool DevScratch::release() {
  if (released_) return p_ != nullptr;
  released_ = true;
  if (!p_) return false;
  if (graph_) return device_ok(cudaFreeAsync(p_, s_), "cudaFreeAsync (captured scratch)");
  Ctx* c = ctx();
  if (!c) return false;
  if (!device_ok(cudaEventRecord(c->last, s_), "scratch record")) return false;
  c->has_last = true;
  return true;
}

DevScratch::~DevScratch() {
  if (!released_) release();
}

}  // namespace vgb_cabi

extern "C" {

const char* vibe_c_last_error(void) { return g_cerr.c_str(); }

unsigned long long vibe_c_allocations(void) { return vgb_cabi::allocations(); }

// ---- FP64: the reference's names ----
int vibe_tridiagonal_solve_batched_f64_dev(const double* a, const double* b, const double* c, const double* d, int n,
                                           int n_sys, double* x, int* status, vibe_stream_t stream) {
  return thomas_batched_dev<double>(a, b, c, d, n, n_sys, x, status, stream);
}

int vibe_tridiagonal_solve_batched_f64_dev_noalloc(const double* a, const double* b, const double* c,
                                                   const double* d, int n, int n_sys, double* x, int* status,
                                                   vibe_stream_t stream) {
  if (n <= 0 || n_sys < 0 || b == nullptr || d == nullptr || x == nullptr) return VIBE_C_ERR_BAD_ARG;
  if ((size_t)n * (size_t)n_sys > kNoAllocThomasDoubles) {
    g_cerr = "vibe_tridiagonal_solve_batched_f64_dev_noalloc: n * n_sys = " + std::to_string((size_t)n * n_sys) +
             " exceeds the fixed workspace of " + std::to_string(kNoAllocThomasDoubles) + " doubles";
    return VIBE_C_ERR_BAD_ARG;
  }
  if (n_sys == 0) return VIBE_C_OK;
  const int dev = cur_dev();
  if (dev < 0 || dev >= 64) { g_cerr = "device ordinal out of range"; return VIBE_C_ERR_DEVICE; }
  double* work = nullptr;
  {
    // set-up on the first call per device: resolve the array's device address
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
      void* p = nullptr;
      if (!device_ok(cudaGetSymbolAddress(&p, g_noalloc_thomas_work), "cudaGetSymbolAddress")) return VIBE_C_ERR_DEVICE;
      g_noalloc_ptr[dev] = (double*)p;
    }
    work = g_noalloc_ptr[dev];
  }
  // the workspace needs no clearing: every system writes cp[k] before it reads it
  k_thomas_batched<double><<<(n_sys + 127) / 128, 128, 0, (cudaStream_t)stream>>>(a, b, c, d, n, n_sys, x, work,
                                                                                 status);
  return device_ok(cudaGetLastError(), "thomas (no-alloc) launch") ? VIBE_C_OK : VIBE_C_ERR_DEVICE;
}

int vibe_tridiagonal_solve_batched_f64(const double* a, const double* b, const double* c, const double* d, int n,
                                       int n_sys, double* x) {
  return thomas_batched_host<double>(a, b, c, d, n, n_sys, x);
}

int vibe_tridiagonal_solve_f64(const double* a, const double* b, const double* c, const double* d, int n, double* x,
                               double* ws) {
  if (n <= 0 || b == nullptr || d == nullptr || x == nullptr || ws == nullptr) return VIBE_C_ERR_BAD_ARG;
  return thomas_batched_host<double>(a, b, c, d, n, 1, x);
}

int vibe_weno5_reconstruct_batched_f64_dev(const double* q, size_t n, double* q_left, double* q_right,
                                           vibe_stream_t stream) {
  return weno_batched_dev<double>(q, n, q_left, q_right, stream);
}

void vibe_weno5_reconstruct_f64(double qm2, double qm1, double q0, double q1, double q2, double* q_left,
                                double* q_right) {
  weno_host<double>(qm2, qm1, q0, q1, q2, q_left, q_right);
}

double vibe_bilinear_f64(const double* f, int halo, int nsx, int nsy, int nz, double xi, double yj, int k) {
  return bilinear_host<double>(f, halo, nsx, nsy, nz, xi, yj, k);
}

int vibe_cfl_scan_f64_dev(const double* u, const double* v, const double* w, const double* dzeta, const double* zs,
                          int nx, int ny, int nz, double dx, double dy, double z_top, double dt, double* out3,
                          vibe_stream_t stream) {
  return cfl_dev<double>(u, v, w, dzeta, zs, nx, ny, nz, dx, dy, z_top, dt, out3, stream);
}

double vibe_cfl_scan_f64(const double* u, const double* v, const double* w, const double* dzeta, const double* zs,
                         int nx, int ny, int nz, double dx, double dy, double z_top, double dt, double* max_wind_out,
                         double* min_dz_out) {
  return cfl_host<double>(u, v, w, dzeta, zs, nx, ny, nz, dx, dy, z_top, dt, max_wind_out, min_dz_out);
}

int vibe_neumaier_sum_f64_dev(const double* x, size_t n, double* out, vibe_stream_t stream) {
  return neu_dev<double>(x, n, out, stream);
}

double vibe_neumaier_sum_f64(const double* x, size_t n) { return neu_host<double>(x, n); }

int vibe_advect_scalar_flux_f64_dev(const double* q, const double* rho, const double* u, const double* v,
                                    const double* w, const double* dzeta, const double* zs, int nx, int ny, int nz,
                                    double dx, double dy, double z_top, double* dqdt, vibe_stream_t stream) {
  return flux_dev<double>(q, rho, u, v, w, dzeta, zs, nx, ny, nz, dx, dy, z_top, dqdt, stream);
}

void vibe_advect_scalar_flux_f64(const double* q, const double* rho, const double* u, const double* v, const double* w,
                                 const double* dzeta, const double* zs, int nx, int ny, int nz, double dx, double dy,
                                 double z_top, double* dqdt) {
  flux_host<double>(q, rho, u, v, w, dzeta, zs, nx, ny, nz, dx, dy, z_top, dqdt);
}

// ---- FP32 twins ----
int vibe_tridiagonal_solve_f32(const float* a, const float* b, const float* c, const float* d, int n, float* x,
                               float* ws) {
  if (n <= 0 || b == nullptr || d == nullptr || x == nullptr || ws == nullptr) return VIBE_C_ERR_BAD_ARG;
  return thomas_batched_host<float>(a, b, c, d, n, 1, x);
}
int vibe_tridiagonal_solve_batched_f32(const float* a, const float* b, const float* c, const float* d, int n,
                                       int n_sys, float* x) {
  return thomas_batched_host<float>(a, b, c, d, n, n_sys, x);
}
int vibe_tridiagonal_solve_batched_f32_dev(const float* a, const float* b, const float* c, const float* d, int n,
                                           int n_sys, float* x, int* status, vibe_stream_t stream) {
  return thomas_batched_dev<float>(a, b, c, d, n, n_sys, x, status, stream);
}
void vibe_weno5_reconstruct_f32(float qm2, float qm1, float q0, float q1, float q2, float* q_left, float* q_right) {
  weno_host<float>(qm2, qm1, q0, q1, q2, q_left, q_right);
}
int vibe_weno5_reconstruct_batched_f32_dev(const float* q, size_t n, float* q_left, float* q_right,
                                           vibe_stream_t stream) {
  return weno_batched_dev<float>(q, n, q_left, q_right, stream);
}
float vibe_bilinear_f32(const float* f, int halo, int nsx, int nsy, int nz, float xi, float yj, int k) {
  return bilinear_host<float>(f, halo, nsx, nsy, nz, xi, yj, k);
}
float vibe_cfl_scan_f32(const float* u, const float* v, const float* w, const float* dzeta, const float* zs, int nx,
                        int ny, int nz, float dx, float dy, float z_top, float dt, float* max_wind_out,
                        float* min_dz_out) {
  return cfl_host<float>(u, v, w, dzeta, zs, nx, ny, nz, dx, dy, z_top, dt, max_wind_out, min_dz_out);
}
int vibe_cfl_scan_f32_dev(const float* u, const float* v, const float* w, const float* dzeta, const float* zs, int nx,
                          int ny, int nz, float dx, float dy, float z_top, float dt, float* out3, vibe_stream_t stream) {
  return cfl_dev<float>(u, v, w, dzeta, zs, nx, ny, nz, dx, dy, z_top, dt, out3, stream);
}
float vibe_neumaier_sum_f32(const float* x, size_t n) { return neu_host<float>(x, n); }
int vibe_neumaier_sum_f32_dev(const float* x, size_t n, float* out, vibe_stream_t stream) {
  return neu_dev<float>(x, n, out, stream);
}
void vibe_advect_scalar_flux_f32(const float* q, const float* rho, const float* u, const float* v, const float* w,
                                 const float* dzeta, const float* zs, int nx, int ny, int nz, float dx, float dy,
                                 float z_top, float* dqdt) {
  flux_host<float>(q, rho, u, v, w, dzeta, zs, nx, ny, nz, dx, dy, z_top, dqdt);
}
int vibe_advect_scalar_flux_f32_dev(const float* q, const float* rho, const float* u, const float* v, const float* w,
                                    const float* dzeta, const float* zs, int nx, int ny, int nz, float dx, float dy,
                                    float z_top, float* dqdt, vibe_stream_t stream) {
  return flux_dev<float>(q, rho, u, v, w, dzeta, zs, nx, ny, nz, dx, dy, z_top, dqdt, stream);
}

}  // extern "C"
