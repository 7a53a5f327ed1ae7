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
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "vibe_c_kernels.h"
#include "vibe_internal.cuh"

namespace {

thread_local std::string g_cerr;

// Per-device scratch for block partials and per-system workspace. Grows on
// demand, never shrinks; guarded by a mutex (the ABI promises reentrancy).
std::mutex g_scr_mu;
void* g_scr[64] = {};
size_t g_scr_n[64] = {};
cudaStream_t g_stream[64] = {};

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

void* scratch(size_t bytes) {
  const int dev = cur_dev();
  if (dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lk(g_scr_mu);
  if (g_scr_n[dev] < bytes) {
    if (g_scr[dev]) cudaFree(g_scr[dev]);
    g_scr[dev] = nullptr;
    g_scr_n[dev] = 0;
    if (cudaMalloc(&g_scr[dev], bytes) != cudaSuccess) return nullptr;
    g_scr_n[dev] = bytes;
  }
  return g_scr[dev];
}

cudaStream_t own_stream() {
  const int dev = cur_dev();
  std::lock_guard<std::mutex> lk(g_scr_mu);
  if (!g_stream[dev]) cudaStreamCreateWithFlags(&g_stream[dev], cudaStreamNonBlocking);
  return g_stream[dev];
}

// RAII device buffer for the host-pointer entry points
struct DBuf {
  void* p = nullptr;
  explicit DBuf(size_t bytes) {
    if (bytes && cudaMalloc(&p, bytes) != cudaSuccess) p = nullptr;
  }
  ~DBuf() {
    if (p) cudaFree(p);
  }
  template <class T>
  T* as() const { return (T*)p; }
};

// ---------------------------------------------------------------------------
// Thomas: one thread per system. Contract c_kernels.h:38-55 with the
// recurrence of thomas_solve (src/time/helmholtz.cpp:71-85); NULL a/c read
// as 0; exact-zero pivots give VIBE_C_ERR_SINGULAR as c_kernels.c:26,34,40.
// cp (the modified super-diagonal) lives in `work` (n per system).
template <typename T>
__global__ void k_thomas_batched(const T* __restrict__ a, const T* __restrict__ b, const T* __restrict__ c,
                                 const T* __restrict__ d, int n, int n_sys, T* __restrict__ x, T* __restrict__ work,
                                 int* __restrict__ status) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n_sys) return;
  const T* as = a ? a + (size_t)s * (n - 1) : nullptr;
  const T* bs = b + (size_t)s * n;
  const T* cs = c ? c + (size_t)s * (n - 1) : nullptr;
  const T* ds = d + (size_t)s * n;
  T* xs = x + (size_t)s * n;
  T* cp = work + (size_t)s * n;
  int rc = VIBE_C_OK;
  if (n == 1) {
    if (bs[0] == (T)0) rc = VIBE_C_ERR_SINGULAR;
    else xs[0] = ds[0] / bs[0];
  } else {
    T denom = bs[0];
    if (denom == (T)0) {
      rc = VIBE_C_ERR_SINGULAR;
    } else {
      cp[0] = (cs ? cs[0] : (T)0) / denom;
      xs[0] = ds[0] / denom;
      for (int k = 1; k < n; ++k) {
        const T am = as ? as[k - 1] : (T)0;
        denom = bs[k] - am * cp[k - 1];
        if (denom == (T)0) { rc = VIBE_C_ERR_SINGULAR; break; }
        xs[k] = (ds[k] - am * xs[k - 1]) / denom;
        if (k < n - 1) cp[k] = (cs ? cs[k] : (T)0) / denom;
      }
      if (rc == VIBE_C_OK)
        for (int k = n - 1; k-- > 0;) xs[k] = xs[k] - cp[k] * xs[k + 1];
    }
  }
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
// A zero pivot of a chunk or a singular 2x2 block gives VIBE_C_ERR_SINGULAR.
// The elimination order differs from one sequential sweep, so results agree
// with it to rounding. Scratch: 3n per system (c', v, w).
constexpr int kTallN = 128;
constexpr int kTallWarps = 4;  // systems per block

template <typename T>
__global__ void __launch_bounds__(32 * kTallWarps) k_thomas_tall(const T* __restrict__ a, const T* __restrict__ b,
                                                                 const T* __restrict__ c, const T* __restrict__ d,
                                                                 int n, int n_sys, T* __restrict__ x,
                                                                 T* __restrict__ work, int* __restrict__ status) {
  __shared__ T sh[kTallWarps][32][6];  // per lane: yF, yE, vF, vE, wF, wE
  __shared__ T zs[kTallWarps][32][2];  // interface solution F_j, E_j
  __shared__ int bad[kTallWarps];
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int s = blockIdx.x * kTallWarps + wid;
  const bool live = s < n_sys;
  const int m = (n + 31) / 32;                   // rows per chunk
  const int r0 = min(lane * m, n), r1 = min(r0 + m, n), L = r1 - r0;
  const int nch = (n + m - 1) / m;               // chunks with rows (lanes >= nch hold none)
  if (lane == 0) bad[wid] = 0;
  __syncwarp();
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
    if (den == (T)0) ok = false;
    if (ok) {
      const T a0 = (r0 > 0 && as) ? as[r0 - 1] : (T)0;   // coupling to x_{r0-1}
      const T cl = (r1 < n && cs) ? cs[r1 - 1] : (T)0;   // coupling to x_{r1}
      cp[r0] = (r0 + 1 < r1) ? ((cs ? cs[r0] : (T)0) / den) : (T)0;
      xs[r0] = ds[r0] / den;
      vv[r0] = a0 / den;
      ww[r0] = (L == 1) ? cl / den : (T)0;
      for (int k = r0 + 1; k < r1 && ok; ++k) {
        const T am = as ? as[k - 1] : (T)0;
        den = bs[k] - am * cp[k - 1];
        if (den == (T)0) { ok = false; break; }
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
  if (!ok) bad[wid] = 1;
  __syncwarp();
  // the interface system, block elimination by lane 0: z_j + Lj z_{j-1} + Uj z_{j+1} = Yj,
  // Lj = [[0, vF], [0, vE]] and Uj = [[wF, 0], [wE, 0]]
  if (live && lane == 0 && !bad[wid]) {
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
      if (det == (T)0) { bad[wid] = 1; break; }
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
    if (!bad[wid])
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
  if (live && L > 0 && !bad[wid]) {
    const T xl = (lane > 0) ? zs[wid][lane - 1][1] : (T)0;        // E of the chunk to the left
    const T xr = (lane + 1 < nch) ? zs[wid][lane + 1][0] : (T)0;  // F of the chunk to the right
    for (int k = r0; k < r1; ++k) xs[k] = xs[k] - vv[k] * xl - ww[k] * xr;
  }
  if (live && lane == 0 && status) status[s] = bad[wid] ? VIBE_C_ERR_SINGULAR : VIBE_C_OK;
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
  const int ia = vgb::iclamp(i0, 0, nxi - 1), ib = vgb::iclamp(i0 + 1, 0, nxi - 1);
  const int ja = vgb::iclamp(j0, 0, nyi - 1), jb = vgb::iclamp(j0 + 1, 0, nyi - 1);
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
  const size_t n = (size_t)nx * ny * nz, nxy = (size_t)nx * ny;
  T worst = 0, mw = 0, mdz = (T)1e30;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(e / nxy);
    const size_t col = e % nxy;
    const T uu = u[e], vv = v[e], ww = w[e];
    const T scale = zs ? (z_top - zs[col]) : z_top;
    T dz = dzeta[k] * scale;
    if (dz < (T)1) dz = (T)1;
    mdz = fmin(mdz, dz);
    mw = fmax(mw, sqrt(uu * uu + vv * vv + ww * ww));
    worst = fmax(worst, dt * (fabs(uu) / dx + fabs(vv) / dy + fabs(ww) / dz));
  }
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
// process exits.
constexpr size_t kNoAllocThomasDoubles = (size_t)1 << 18;  // 2 MiB: n * n_sys <= 262144
static __device__ __align__(256) double g_noalloc_thomas_work[kNoAllocThomasDoubles];
// Device address of that array per device. Host code only sees a host-side
// stand-in for the symbol; the address a kernel may use comes from
// cudaGetSymbolAddress, called with the device current.
std::mutex g_noalloc_mu;
double* g_noalloc_ptr[64] = {};

constexpr int kRedBlocks = 304;  // 2 x 152 SMs
constexpr int kRedThreads = 256;

// ---- entry points, one template per ABI function: T = double (the
// reference's *_f64 names) or float (the *_f32 twins its header reserves,
// c_kernels.h:15-16) ----
template <typename T>
int thomas_batched_dev(const T* a, const T* b, const T* c, const T* d, int n, int n_sys, T* x, int* status,
                       vibe_stream_t stream) {
  if (n <= 0 || n_sys < 0 || b == nullptr || d == nullptr || x == nullptr) return VIBE_C_ERR_BAD_ARG;
  if (n_sys == 0) return VIBE_C_OK;
  const bool tall = n > kTallN;
  T* work = (T*)scratch((size_t)n * n_sys * sizeof(T) * (tall ? 3 : 1));
  if (!work) { g_cerr = "scratch allocation failed"; return VIBE_C_ERR_DEVICE; }
  if (tall)
    k_thomas_tall<T><<<(n_sys + kTallWarps - 1) / kTallWarps, 32 * kTallWarps, 0, (cudaStream_t)stream>>>(
        a, b, c, d, n, n_sys, x, work, status);
  else
    k_thomas_batched<T><<<(n_sys + 127) / 128, 128, 0, (cudaStream_t)stream>>>(a, b, c, d, n, n_sys, x, work,
                                                                              status);
  return device_ok(cudaGetLastError(), "thomas launch") ? VIBE_C_OK : VIBE_C_ERR_DEVICE;
}

template <typename T>
int thomas_batched_host(const T* a, const T* b, const T* c, const T* d, int n, int n_sys, T* x) {
  if (n <= 0 || n_sys < 0 || b == nullptr || d == nullptr || x == nullptr) return VIBE_C_ERR_BAD_ARG;
  if (n_sys == 0) return VIBE_C_OK;
  const size_t e = sizeof(T), nn = (size_t)n * n_sys, no = (size_t)(n - 1) * n_sys;
  DBuf da(a ? no * e + e : 0), db(nn * e), dc(c ? no * e + e : 0), dd(nn * e), dx(nn * e), ds((size_t)n_sys * 4);
  if (!db.p || !dd.p || !dx.p || !ds.p || (a && !da.p) || (c && !dc.p)) { g_cerr = "cudaMalloc failed"; return VIBE_C_ERR_DEVICE; }
  cudaStream_t st = own_stream();
  bool ok = true;
  if (a && no) ok &= device_ok(cudaMemcpyAsync(da.p, a, no * e, cudaMemcpyHostToDevice, st), "H2D a");
  if (c && no) ok &= device_ok(cudaMemcpyAsync(dc.p, c, no * e, cudaMemcpyHostToDevice, st), "H2D c");
  ok &= device_ok(cudaMemcpyAsync(db.p, b, nn * e, cudaMemcpyHostToDevice, st), "H2D b");
  ok &= device_ok(cudaMemcpyAsync(dd.p, d, nn * e, cudaMemcpyHostToDevice, st), "H2D d");
  if (!ok) return VIBE_C_ERR_DEVICE;
  int rc = thomas_batched_dev<T>(a ? da.as<T>() : nullptr, db.as<T>(), c ? dc.as<T>() : nullptr, dd.as<T>(), n, n_sys,
                                 dx.as<T>(), ds.as<int>(), (vibe_stream_t)st);
  if (rc) return rc;
  std::string st_host((size_t)n_sys * 4, '\0');
  ok &= device_ok(cudaMemcpyAsync(x, dx.p, nn * e, cudaMemcpyDeviceToHost, st), "D2H x");
  ok &= device_ok(cudaMemcpyAsync(&st_host[0], ds.p, (size_t)n_sys * 4, cudaMemcpyDeviceToHost, st), "D2H status");
  ok &= device_ok(cudaStreamSynchronize(st), "sync");
  if (!ok) return VIBE_C_ERR_DEVICE;
  const int* sv = (const int*)st_host.data();
  for (int s = 0; s < n_sys; ++s)
    if (sv[s] != VIBE_C_OK) return sv[s];
  return VIBE_C_OK;
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
  const size_t e = sizeof(T);
  DBuf dq(5 * e), dl(e), dr(e);
  if (!dq.p || !dl.p || !dr.p) { g_cerr = "cudaMalloc failed"; *q_left = *q_right = (T)NAN; return; }
  const T q[5] = {qm2, qm1, q0, q1, q2};
  cudaStream_t st = own_stream();
  bool ok = device_ok(cudaMemcpyAsync(dq.p, q, 5 * e, cudaMemcpyHostToDevice, st), "H2D");
  ok = ok && weno_batched_dev<T>(dq.as<T>(), 1, dl.as<T>(), dr.as<T>(), (vibe_stream_t)st) == VIBE_C_OK;
  ok = ok && device_ok(cudaMemcpyAsync(q_left, dl.p, e, cudaMemcpyDeviceToHost, st), "D2H");
  ok = ok && device_ok(cudaMemcpyAsync(q_right, dr.p, e, cudaMemcpyDeviceToHost, st), "D2H");
  ok = ok && device_ok(cudaStreamSynchronize(st), "sync");
  if (!ok) *q_left = *q_right = (T)NAN;
}

template <typename T>
T bilinear_host(const T* f, int halo, int nsx, int nsy, int nz, T xi, T yj, int k) {
  if (f == nullptr || nz <= 0) return (T)0;
  if (k < 0) k = 0;
  if (k >= nz) k = nz - 1;
  const size_t plane = (size_t)nsx * nsy, e = sizeof(T);
  DBuf dp(plane * e), dout(e);
  if (!dp.p || !dout.p) { g_cerr = "cudaMalloc failed"; return (T)NAN; }
  cudaStream_t st = own_stream();
  T r = (T)NAN;
  bool ok = device_ok(cudaMemcpyAsync(dp.p, f + (size_t)(k + halo) * plane, plane * e, cudaMemcpyHostToDevice, st), "H2D");
  if (ok) {
    k_bilinear<T><<<1, 1, 0, st>>>(dp.as<T>(), halo, nsx, nsy, xi, yj, dout.as<T>());
    ok = device_ok(cudaGetLastError(), "bilinear launch");
  }
  ok = ok && device_ok(cudaMemcpyAsync(&r, dout.p, e, cudaMemcpyDeviceToHost, st), "D2H");
  ok = ok && device_ok(cudaStreamSynchronize(st), "sync");
  return ok ? r : (T)NAN;
}

template <typename T>
int cfl_dev(const T* u, const T* v, const T* w, const T* dzeta, const T* zs, int nx, int ny, int nz, T dx, T dy,
            T z_top, T dt, T* out3, vibe_stream_t stream) {
  if (!u || !v || !w || !dzeta || !out3 || nx < 0 || ny < 0 || nz < 0) return VIBE_C_ERR_BAD_ARG;
  T* part = (T*)scratch((size_t)3 * kRedBlocks * sizeof(T));
  if (!part) { g_cerr = "scratch allocation failed"; return VIBE_C_ERR_DEVICE; }
  cudaStream_t st = (cudaStream_t)stream;
  k_cfl_partial<T><<<kRedBlocks, kRedThreads, 0, st>>>(u, v, w, dzeta, zs, nx, ny, nz, dx, dy, z_top, dt, part);
  k_cfl_final<T><<<1, kRedThreads, 0, st>>>(part, kRedBlocks, out3);
  return device_ok(cudaGetLastError(), "cfl launch") ? VIBE_C_OK : VIBE_C_ERR_DEVICE;
}

template <typename T>
T cfl_host(const T* u, const T* v, const T* w, const T* dzeta, const T* zs, int nx, int ny, int nz, T dx, T dy, T z_top,
           T dt, T* max_wind_out, T* min_dz_out) {
  if (u == nullptr || v == nullptr || w == nullptr || dzeta == nullptr) return (T)0;
  const size_t e = sizeof(T);
  const size_t n = (size_t)(nx > 0 ? nx : 0) * (ny > 0 ? ny : 0) * (nz > 0 ? nz : 0);
  const size_t nzp = (size_t)(nz > 0 ? nz : 0);
  DBuf du(n * e + e), dv(n * e + e), dw(n * e + e), dz(nzp * e + e), dzs(zs ? (size_t)nx * ny * e + e : 0), dout(3 * e);
  if (!du.p || !dv.p || !dw.p || !dz.p || !dout.p || (zs && !dzs.p)) { g_cerr = "cudaMalloc failed"; return (T)NAN; }
  cudaStream_t st = own_stream();
  bool ok = true;
  ok &= device_ok(cudaMemcpyAsync(du.p, u, n * e, cudaMemcpyHostToDevice, st), "H2D");
  ok &= device_ok(cudaMemcpyAsync(dv.p, v, n * e, cudaMemcpyHostToDevice, st), "H2D");
  ok &= device_ok(cudaMemcpyAsync(dw.p, w, n * e, cudaMemcpyHostToDevice, st), "H2D");
  ok &= device_ok(cudaMemcpyAsync(dz.p, dzeta, nzp * e, cudaMemcpyHostToDevice, st), "H2D");
  if (zs) ok &= device_ok(cudaMemcpyAsync(dzs.p, zs, (size_t)nx * ny * e, cudaMemcpyHostToDevice, st), "H2D");
  if (!ok) return (T)NAN;
  if (cfl_dev<T>(du.as<T>(), dv.as<T>(), dw.as<T>(), dz.as<T>(), zs ? dzs.as<T>() : nullptr, nx, ny, nz, dx, dy, z_top,
                 dt, dout.as<T>(), (vibe_stream_t)st) != VIBE_C_OK)
    return (T)NAN;
  T r[3];
  ok &= device_ok(cudaMemcpyAsync(r, dout.p, 3 * e, cudaMemcpyDeviceToHost, st), "D2H");
  ok &= device_ok(cudaStreamSynchronize(st), "sync");
  if (!ok) return (T)NAN;
  if (max_wind_out) *max_wind_out = r[1];
  if (min_dz_out) *min_dz_out = r[2];
  return r[0];
}

template <typename T>
int neu_dev(const T* x, size_t n, T* out, vibe_stream_t stream) {
  if (!x || !out) return VIBE_C_ERR_BAD_ARG;
  T* part = (T*)scratch((size_t)2 * kRedBlocks * sizeof(T));
  if (!part) { g_cerr = "scratch allocation failed"; return VIBE_C_ERR_DEVICE; }
  cudaStream_t st = (cudaStream_t)stream;
  const size_t chunk = (n + kRedBlocks - 1) / kRedBlocks;
  k_neu_partial<T><<<kRedBlocks, kRedThreads, 0, st>>>(x, n, chunk > 0 ? chunk : 1, part);
  k_neu_final<T><<<1, kRedThreads, 0, st>>>(part, kRedBlocks, out);
  return device_ok(cudaGetLastError(), "neumaier launch") ? VIBE_C_OK : VIBE_C_ERR_DEVICE;
}

template <typename T>
T neu_host(const T* x, size_t n) {
  if (x == nullptr) return (T)0;
  const size_t e = sizeof(T);
  DBuf dx(n * e + e), dout(e);
  if (!dx.p || !dout.p) { g_cerr = "cudaMalloc failed"; return (T)NAN; }
  cudaStream_t st = own_stream();
  bool ok = device_ok(cudaMemcpyAsync(dx.p, x, n * e, cudaMemcpyHostToDevice, st), "H2D");
  ok = ok && neu_dev<T>(dx.as<T>(), n, dout.as<T>(), (vibe_stream_t)st) == VIBE_C_OK;
  T r = (T)NAN;
  ok = ok && device_ok(cudaMemcpyAsync(&r, dout.p, e, cudaMemcpyDeviceToHost, st), "D2H");
  ok = ok && device_ok(cudaStreamSynchronize(st), "sync");
  return ok ? r : (T)NAN;
}

template <typename T>
int flux_dev(const T* q, const T* rho, const T* u, const T* v, const T* w, const T* dzeta, const T* zs, int nx, int ny,
             int nz, T dx, T dy, T z_top, T* dqdt, vibe_stream_t stream) {
  if (!q || !rho || !u || !v || !w || !dzeta || !dqdt) return VIBE_C_ERR_BAD_ARG;
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
  const size_t n = (size_t)nx * ny * nz, e = sizeof(T);
  if (n == 0) return;
  DBuf dq(n * e), dr(n * e), du(n * e), dv(n * e), dw(n * e), dz((size_t)nz * e), dzs(zs ? (size_t)nx * ny * e : 0),
      dout(n * e);
  if (!dq.p || !dr.p || !du.p || !dv.p || !dw.p || !dz.p || !dout.p || (zs && !dzs.p)) { g_cerr = "cudaMalloc failed"; return; }
  cudaStream_t st = own_stream();
  bool ok = true;
  ok &= device_ok(cudaMemcpyAsync(dq.p, q, n * e, cudaMemcpyHostToDevice, st), "H2D");
  ok &= device_ok(cudaMemcpyAsync(dr.p, rho, n * e, cudaMemcpyHostToDevice, st), "H2D");
  ok &= device_ok(cudaMemcpyAsync(du.p, u, n * e, cudaMemcpyHostToDevice, st), "H2D");
  ok &= device_ok(cudaMemcpyAsync(dv.p, v, n * e, cudaMemcpyHostToDevice, st), "H2D");
  ok &= device_ok(cudaMemcpyAsync(dw.p, w, n * e, cudaMemcpyHostToDevice, st), "H2D");
  ok &= device_ok(cudaMemcpyAsync(dz.p, dzeta, (size_t)nz * e, cudaMemcpyHostToDevice, st), "H2D");
  if (zs) ok &= device_ok(cudaMemcpyAsync(dzs.p, zs, (size_t)nx * ny * e, cudaMemcpyHostToDevice, st), "H2D");
  if (!ok) return;
  if (flux_dev<T>(dq.as<T>(), dr.as<T>(), du.as<T>(), dv.as<T>(), dw.as<T>(), dz.as<T>(), zs ? dzs.as<T>() : nullptr,
                  nx, ny, nz, dx, dy, z_top, dout.as<T>(), (vibe_stream_t)st) != VIBE_C_OK)
    return;
  device_ok(cudaMemcpyAsync(dqdt, dout.p, n * e, cudaMemcpyDeviceToHost, st), "D2H");
  device_ok(cudaStreamSynchronize(st), "sync");
}

}  // namespace

extern "C" {

const char* vibe_c_last_error(void) { return g_cerr.c_str(); }

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
