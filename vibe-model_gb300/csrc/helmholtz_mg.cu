// vibe-model_gb300/csrc/helmholtz_mg.cu
//
// Right-preconditioned BiCGSTAB (van der Vorst 1992) with a geometric
// multigrid V-cycle as preconditioner, for the reference's Helmholtz
// operator y = -div(a grad x) + b x (src/time/helmholtz.cpp:173-201),
// templated on the working precision (FP32 for the mixed solver, FP64).
//
// Operator in coupling form. For a cell, with W/E/S/N/B/T neighbours,
//   (A x) = cD x + cE (x - xE) + cW (x - xW) + cN (x - xN) + cS (x - xS)
//           + cT (x - xT) + cB (x - xB),
// cE = (a + aE)/2 / dx^2 (0 on the east boundary: the reference's clamp
// makes that flux vanish), cW(i) = cE(i-1), likewise N/S; cT = (a + aT)/2 /
// dz^2 and cB = (a + aB)/2 / dz^2 with the cell's own dz (so A is not
// symmetric on a stretched grid), cD = b.
//
// Multigrid. The vertical couplings dominate (dz << dx), so the smoother is
// a vertical-line Gauss-Seidel: every column solves its tridiagonal system
// exactly with the horizontal neighbours fixed, columns in red-black order
// ((i + j) parity), 32 columns per 256 threads with the column recurrences
// run as scans over 8 level segments (k_smooth_scan); the column LU factors
// are computed once per coefficient set. Coarse grids halve nx and ny and
// keep nz (semi-coarsening); coarse couplings are the 2x2 aggregates: cT,
// cB, cD averaged, the horizontal face couplings summed over the two fine
// faces of the coarse face and divided by 8 (= the rediscretised
// a/(2h)^2). Residuals are restricted by the 2x2 mean (computed and
// restricted in one pass) and corrections prolonged piecewise constant.
// V(1,1) cycle, the coarsest grid smoothed 8 times in one block. The
// BiCGSTAB loop runs on the device as a conditional CUDA graph.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "helmholtz.cuh"

namespace vgb {

constexpr int kMgMaxLevels = 8;
constexpr int kMT = 256;
// blocks of the Krylov kernels that reduce (6 x 152 SMs: the occupancy of
// their 256-thread blocks, so the grid-stride loops keep enough loads in flight)
constexpr int kMgRedBlocks = 912;
static_assert(kMgRedBlocks >= kRedBlocks, "dot64 shares the partials");

template <typename T>
struct MgLevel {
  int nx, ny, nz;
  size_t n;
  T *cE, *cN, *cT, *cB, *cD;  // couplings and mass term
  T *lc, *li;                 // column LU: c'_k, 1/denom_k
  T *x, *r;                   // correction, right-hand side
};

template <typename T>
struct MgSolver {
  HGeo g;
  int L = 0;
  MgLevel<T> lv[kMgMaxLevels];
  T *x, *r, *r0, *p, *v, *s, *t, *ph, *sh;  // Krylov vectors (fine level)
  double* part = nullptr;                   // 2 x kMgRedBlocks partial sums
  double* sc = nullptr;                     // device scalars
  double* hsc = nullptr;                    // pinned host copy
  std::vector<void*> allocs;
  // the iteration loop as a CUDA graph: a WHILE node around one iteration,
  // whose condition the last kernel of the iteration clears (0 = not built
  // yet, 1 = built, -1 = not available: the host loop runs instead)
  int graph_state = 0;
  int coarse_ctas = 0;  // CTAs of the one-cluster coarsest smoothing (0: one launch per half sweep)
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
};

namespace {

enum Sc {
  RHO_OLD = 0, ALPHA = 1, OMEGA = 2, RHO_NEW = 3, RV = 4, TS = 5, TT = 6, RR = 7, BREAK = 8,
  ITERS = 9, RTOL2 = 10, MAXIT = 11,  // iterations done; stop test (squared tolerance, iteration limit)
  BETA = 12,                           // the next iteration's (rho_new / rho_old) (alpha / omega)
  NSC = 16
};

__device__ __forceinline__ void cell_of(size_t c, int nx, int ny, int& i, int& j, int& k) {
  if (c <= 0xffffffffull) {  // 32-bit divisions (64-bit ones are long integer sequences)
    const unsigned cu = (unsigned)c, row = cu / (unsigned)nx, plane = row / (unsigned)ny;
    i = (int)(cu - row * (unsigned)nx);
    j = (int)(row - plane * (unsigned)ny);
    k = (int)plane;
    return;
  }
  i = (int)(c % nx);
  const size_t cj = c / nx;
  j = (int)(cj % ny);
  k = (int)(cj / ny);
}

// A x at cell c of level l (coupling form)
template <typename T>
__device__ __forceinline__ T apply_at(const MgLevel<T>& l, const T* __restrict__ x, size_t c, int i, int j, int k) {
  const size_t pl = (size_t)l.nx * l.ny;
  const T xc = x[c];
  T y = l.cD[c] * xc;
  const T ce = l.cE[c], cn = l.cN[c], ct = l.cT[c], cb = l.cB[c];
  if (i + 1 < l.nx) y += ce * (xc - x[c + 1]);
  if (i > 0) y += l.cE[c - 1] * (xc - x[c - 1]);
  if (j + 1 < l.ny) y += cn * (xc - x[c + l.nx]);
  if (j > 0) y += l.cN[c - l.nx] * (xc - x[c - l.nx]);
  if (k + 1 < l.nz) y += ct * (xc - x[c + pl]);
  if (k > 0) y += cb * (xc - x[c - pl]);
  return y;
}

// ---- coefficient set-up ----
template <typename T>
__global__ void k_fine_coefs(HGeo g, const double* __restrict__ a, const double* __restrict__ b, MgLevel<T> l) {
  const size_t n = g.n(), pl = (size_t)g.nx * g.ny;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
    int i, j, k;
    cell_of(c, g.nx, g.ny, i, j, k);
    const double dz = dmax(g.dzeta[k] * g.scale[(size_t)j * g.nx + i], 1.0);
    const double ac = a[c], idx2 = 1.0 / (g.dx * g.dx), idy2 = 1.0 / (g.dy * g.dy), idz2 = 1.0 / (dz * dz);
    l.cE[c] = (T)(i + 1 < g.nx ? 0.5 * (ac + a[c + 1]) * idx2 : 0.0);
    l.cN[c] = (T)(j + 1 < g.ny ? 0.5 * (ac + a[c + g.nx]) * idy2 : 0.0);
    l.cT[c] = (T)(k + 1 < g.nz ? 0.5 * (ac + a[c + pl]) * idz2 : 0.0);
    l.cB[c] = (T)(k > 0 ? 0.5 * (ac + a[c - pl]) * idz2 : 0.0);
    l.cD[c] = (T)b[c];
  }
}

template <typename T>
__global__ void k_coarse_coefs(MgLevel<T> f, MgLevel<T> cl) {
  const size_t pf = (size_t)f.nx * f.ny;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < cl.n; c += (size_t)gridDim.x * blockDim.x) {
    int I, J, k;
    cell_of(c, cl.nx, cl.ny, I, J, k);
    const size_t f00 = (size_t)k * pf + (size_t)(2 * J) * f.nx + 2 * I;
    const size_t f10 = f00 + 1, f01 = f00 + f.nx, f11 = f01 + 1;
    cl.cE[c] = (f.cE[f10] + f.cE[f11]) * (T)0.125;
    cl.cN[c] = (f.cN[f01] + f.cN[f11]) * (T)0.125;
    cl.cT[c] = (f.cT[f00] + f.cT[f10] + f.cT[f01] + f.cT[f11]) * (T)0.25;
    cl.cB[c] = (f.cB[f00] + f.cB[f10] + f.cB[f01] + f.cB[f11]) * (T)0.25;
    cl.cD[c] = (f.cD[f00] + f.cD[f10] + f.cD[f01] + f.cD[f11]) * (T)0.25;
  }
}

template <typename T>
__device__ __forceinline__ T diag_at(const MgLevel<T>& l, size_t c, int i, int j) {
  T m = l.cD[c] + l.cE[c] + l.cN[c] + l.cT[c] + l.cB[c];
  if (i > 0) m += l.cE[c - 1];
  if (j > 0) m += l.cN[c - l.nx];
  return m;
}

// column LU of (diag, -cB, -cT): denom_k = m_k + cB_k c'_{k-1}, c'_k = -cT_k / denom_k
template <typename T>
__global__ void k_column_lu(MgLevel<T> l) {
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= l.nx * l.ny) return;
  const int i = col % l.nx, j = col / l.nx;
  const size_t pl = (size_t)l.nx * l.ny;
  T cprev = 0;
  for (int k = 0; k < l.nz; ++k) {
    const size_t c = (size_t)k * pl + col;
    const T den = diag_at(l, c, i, j) + (k > 0 ? l.cB[c] * cprev : (T)0);
    const T inv = (T)1 / den;
    cprev = -l.cT[c] * inv;
    l.li[c] = inv;
    l.lc[c] = cprev;
  }
}

// ---- multigrid kernels ----
// one red-black half sweep of vertical-line Gauss-Seidel on columns with
// (i + j) % 2 == color; zero_nb: the horizontal neighbours are taken as 0
// (first half sweep from a zero initial guess), one thread per column, the
// levels in order (the recurrence carries dp from level to level). Used for
// columns too tall for the tiled form below.
template <typename T>
__global__ void k_smooth(MgLevel<T> l, const T* __restrict__ rhs, T* __restrict__ x, int color, int zero_nb) {
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= l.nx * l.ny) return;
  const int i = col % l.nx, j = col / l.nx;
  if (((i + j) & 1) != color) return;
  const size_t pl = (size_t)l.nx * l.ny;
  T dp = 0;
  for (int k = 0; k < l.nz; ++k) {
    const size_t c = (size_t)k * pl + col;
    T d = rhs[c];
    if (!zero_nb) {
      if (i + 1 < l.nx) d += l.cE[c] * x[c + 1];
      if (i > 0) d += l.cE[c - 1] * x[c - 1];
      if (j + 1 < l.ny) d += l.cN[c] * x[c + l.nx];
      if (j > 0) d += l.cN[c - l.nx] * x[c - l.nx];
    }
    dp = (d + (k > 0 ? l.cB[c] * dp : (T)0)) * l.li[c];
    x[c] = dp;
  }
  T xn = dp;
  for (int k = l.nz - 1; k-- > 0;) {
    const size_t c = (size_t)k * pl + col;
    xn = x[c] - l.lc[c] * xn;
    x[c] = xn;
  }
}
// The same half sweep, tiled: 256 threads take a tile of 32 columns of the
// colour (the colour's columns numbered row by row, q = j per_row + m, column
// i = 2m + (j + colour) % 2; 32 consecutive q, which at 64 columns per row
// and more lie in one row) and all nz levels.
//   1. loads, coalesced along the row: per level and column the right-hand
//      side d (with the other colour's current neighbours unless zero_nb) and
//      the recurrences' coefficients, A = cB li, B = d li, C = -lc, into
//      shared memory (rows padded to 33 against bank conflicts). The loads
//      of a batch of levels are all issued before any of them is used: their
//      addresses are clamped into the grid and the values masked afterwards,
//      so no branch separates them (one memory round trip per batch);
//   2. the forward recurrence dp_k = A_k dp_(k-1) + B_k and then the back
//      substitution x_k = C_k x_(k+1) + dp_k, each as a scan: a column's
//      levels are cut into 8 segments held by 8 consecutive lanes; every lane
//      composes its segment into one affine map, the maps are scanned across
//      the 8 lanes with shuffles (3 steps), and each lane re-runs its segment
//      from its incoming value;
//   3. coalesced stores.
// A column then costs one memory round trip instead of 2 nz dependent ones.
// The result equals the sequential sweep up to rounding (the scan
// reassociates the recurrence; 2e-7 relative in FP32).
constexpr int kScanRS = 33;  // shared-memory row stride of a tile (32 columns + 1)

template <typename T>
struct ScanTile {
  T *A, *B, *C;
  __device__ ScanTile(T* base, int nz) : A(base), B(base + (size_t)nz * kScanRS), C(base + 2 * (size_t)nz * kScanRS) {}
};

// lane's column of tile t of the colour; false outside the grid
template <typename T>
__device__ __forceinline__ bool tile_column(const MgLevel<T>& l, int t, int color, int lane, int& i, int& j) {
  const int per_row = (l.nx + 1) / 2;
  const int q = t * 32 + lane;
  j = q / per_row;
  i = 2 * (q - j * per_row) + ((j + color) & 1);
  const bool ok = j < l.ny && i < l.nx;
  if (!ok) i = j = 0;
  return ok;
}

// kB: levels per batch and thread (12 kB values in registers)
template <typename T, bool kZeroNb, int kB>
__device__ __forceinline__ void scan_tile_load(const MgLevel<T>& l, const T* __restrict__ rhs,
                                               const T* __restrict__ x, int t, int color, ScanTile<T> st,
                                               int tid) {
  const int nz = l.nz;
  const int lane = tid & 31, w = tid >> 5;
  int i, j;
  const bool ok = tile_column(l, t, color, lane, i, j);
  const size_t pl = (size_t)l.nx * l.ny;
  const int col = j * l.nx + i;
  const bool e = ok && i + 1 < l.nx, wv = ok && i > 0, n = ok && j + 1 < l.ny, so = ok && j > 0;
  const int de = e ? 1 : 0, dw = wv ? 1 : 0, dn = n ? l.nx : 0, ds = so ? l.nx : 0;
  for (int kb = w; kb < nz; kb += 8 * kB) {
    T rv[kB], ce[kB], xe[kB], cw[kB], xw[kB], cn[kB], xn[kB], cs[kB], xs[kB], li[kB], cb[kB], lc[kB];
#pragma unroll
    for (int u = 0; u < kB; ++u) {
      const int k = kb + 8 * u;
      const size_t c = (size_t)(k < nz ? k : nz - 1) * pl + col;
      rv[u] = rhs[c];
      if (!kZeroNb) {
        ce[u] = l.cE[c];
        xe[u] = x[c + de];
        cw[u] = l.cE[c - dw];
        xw[u] = x[c - dw];
        cn[u] = l.cN[c];
        xn[u] = x[c + dn];
        cs[u] = l.cN[c - ds];
        xs[u] = x[c - ds];
      }
      li[u] = l.li[c];
      cb[u] = l.cB[c];
      lc[u] = l.lc[c];
    }
#pragma unroll
    for (int u = 0; u < kB; ++u) {
      const int k = kb + 8 * u;
      if (k < nz) {
        T d = rv[u];
        if (!kZeroNb) {
          if (e) d += ce[u] * xe[u];
          if (wv) d += cw[u] * xw[u];
          if (n) d += cn[u] * xn[u];
          if (so) d += cs[u] * xs[u];
        }
        st.A[k * kScanRS + lane] = (ok && k > 0) ? cb[u] * li[u] : (T)0;
        st.B[k * kScanRS + lane] = ok ? d * li[u] : (T)0;
        st.C[k * kScanRS + lane] = (ok && k + 1 < nz) ? -lc[u] : (T)0;
      }
    }
  }
}

template <typename T>
__device__ __forceinline__ void scan_tile_solve(int nz, ScanTile<T> st, int tid) {
  const int cl = tid >> 3, sg = tid & 7;  // column, segment: a column's segments in consecutive lanes
  const int S = (nz + 7) / 8, k0 = sg * S, k1 = (k0 + S < nz) ? k0 + S : nz;
  T a = 1, b = 0;
  for (int kq = k0; kq < k1; kq += 8) {
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int k = kq + u;
      if (k < k1) {
        const T Ak = st.A[k * kScanRS + cl];
        a = Ak * a;
        b = Ak * b + st.B[k * kScanRS + cl];
      }
    }
  }
#pragma unroll
  for (int off = 1; off < 8; off <<= 1) {
    const T ap = __shfl_up_sync(0xffffffffu, a, off, 8);
    const T bp = __shfl_up_sync(0xffffffffu, b, off, 8);
    if (sg >= off) {
      b = a * bp + b;
      a = a * ap;
    }
  }
  T dp = __shfl_up_sync(0xffffffffu, b, 1, 8);  // dp at the top of the segment below
  if (sg == 0) dp = 0;
  for (int kq = k0; kq < k1; kq += 8) {
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int k = kq + u;
      if (k < k1) {
        dp = st.A[k * kScanRS + cl] * dp + st.B[k * kScanRS + cl];
        st.B[k * kScanRS + cl] = dp;
      }
    }
  }
  a = 1;
  b = 0;
  for (int kq = k1 - 1; kq >= k0; kq -= 8) {
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int k = kq - u;
      if (k >= k0) {
        const T Ck = st.C[k * kScanRS + cl];
        a = Ck * a;
        b = Ck * b + st.B[k * kScanRS + cl];
      }
    }
  }
#pragma unroll
  for (int off = 1; off < 8; off <<= 1) {
    const T an = __shfl_down_sync(0xffffffffu, a, off, 8);
    const T bn = __shfl_down_sync(0xffffffffu, b, off, 8);
    if (sg + off < 8) {
      b = a * bn + b;
      a = a * an;
    }
  }
  T xv = __shfl_down_sync(0xffffffffu, b, 1, 8);  // x at the bottom of the segment above
  if (sg == 7) xv = 0;
  for (int kq = k1 - 1; kq >= k0; kq -= 8) {
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int k = kq - u;
      if (k >= k0) {
        xv = st.C[k * kScanRS + cl] * xv + st.B[k * kScanRS + cl];
        st.B[k * kScanRS + cl] = xv;
      }
    }
  }
}

template <typename T>
__device__ __forceinline__ void scan_tile_store(const MgLevel<T>& l, T* __restrict__ x, int t, int color,
                                                ScanTile<T> st, int tid) {
  const int lane = tid & 31, w = tid >> 5;
  int i, j;
  if (!tile_column(l, t, color, lane, i, j)) return;
  const size_t pl = (size_t)l.nx * l.ny;
  const int col = j * l.nx + i;
#pragma unroll 8
  for (int k = w; k < l.nz; k += 8) x[(size_t)k * pl + col] = st.B[k * kScanRS + lane];
}

template <typename T, bool kZeroNb>
__global__ void __launch_bounds__(256) k_smooth_scan(MgLevel<T> l, const T* __restrict__ rhs, T* __restrict__ x,
                                                     int color) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const ScanTile<T> st(reinterpret_cast<T*>(smem_raw), l.nz);
  scan_tile_load<T, kZeroNb, sizeof(T) == 4 ? 8 : 4>(l, rhs, x, blockIdx.x, color, st, threadIdx.x);
  __syncthreads();
  scan_tile_solve<T>(l.nz, st, threadIdx.x);
  __syncthreads();
  scan_tile_store<T>(l, x, blockIdx.x, color, st, threadIdx.x);
}

// The coarsest grid's smoothing, kCoarseSweeps red-black sweeps (the first
// half sweep from a zero guess), in one launch of one thread-block cluster:
// CTA b takes tiles b, b + gridDim.x, ... of each half sweep, and the
// cluster barrier (release/acquire at cluster scope, so x's global stores
// are seen by the cluster's loads after it) separates the half sweeps; a
// half sweep reads only the other colour, so its tiles are independent.
// Replaces 2 kCoarseSweeps launches of a few tiles each (16 x 16 x 64: 4
// tiles per half sweep).
constexpr int kCoarseSweeps = 8;
constexpr int kCoarseMaxCtas = 8;  // portable cluster size

__device__ __forceinline__ void cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

template <typename T>
__global__ void __launch_bounds__(256) k_coarse_smooth(MgLevel<T> l, const T* __restrict__ rhs, T* __restrict__ x) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const ScanTile<T> st(reinterpret_cast<T*>(smem_raw), l.nz);
  const int ntiles = ((l.nx + 1) / 2 * l.ny + 31) / 32;
  constexpr int kB = sizeof(T) == 4 ? 8 : 4;
  for (int sw = 0; sw < 2 * kCoarseSweeps; ++sw) {
    const int color = sw & 1;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
      if (sw == 0)
        scan_tile_load<T, true, kB>(l, rhs, x, t, color, st, threadIdx.x);
      else
        scan_tile_load<T, false, kB>(l, rhs, x, t, color, st, threadIdx.x);
      __syncthreads();
      scan_tile_solve<T>(l.nz, st, threadIdx.x);
      __syncthreads();
      scan_tile_store<T>(l, x, t, color, st, threadIdx.x);
      __syncthreads();  // the next tile overwrites the shared memory
    }
    cluster_sync();  // the half sweep's stores before the next half sweep's loads
  }
}

constexpr size_t kScanSmemMax = 200 * 1024;   // one tile's shared memory, at most
constexpr int kCoarseMaxTiles = 64;             // tiles per half sweep up to which one cluster smooths the coarsest grid
template <typename T>
size_t scan_smem(int nz) {
  return 3 * (size_t)nz * kScanRS * sizeof(T);
}

// the residual rhs - A x on the four fine cells of each coarse cell, their
// mean written as the coarse right-hand side (restriction by the 2 x 2 mean)
template <typename T>
__global__ void k_resid_restrict(MgLevel<T> f, const T* __restrict__ rhs, const T* __restrict__ x, MgLevel<T> cl) {
  const size_t pf = (size_t)f.nx * f.ny;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < cl.n; c += (size_t)gridDim.x * blockDim.x) {
    int I, J, k;
    cell_of(c, cl.nx, cl.ny, I, J, k);
    const int i = 2 * I, j = 2 * J;
    const size_t f00 = (size_t)k * pf + (size_t)j * f.nx + i;
    const size_t f10 = f00 + 1, f01 = f00 + f.nx, f11 = f01 + 1;
    const T t00 = rhs[f00] - apply_at(f, x, f00, i, j, k);
    const T t10 = rhs[f10] - apply_at(f, x, f10, i + 1, j, k);
    const T t01 = rhs[f01] - apply_at(f, x, f01, i, j + 1, k);
    const T t11 = rhs[f11] - apply_at(f, x, f11, i + 1, j + 1, k);
    cl.r[c] = (t00 + t10 + t01 + t11) * (T)0.25;
  }
}

template <typename T>
__global__ void k_prolong_add(MgLevel<T> f, T* __restrict__ x, MgLevel<T> cl) {
  const size_t pc = (size_t)cl.nx * cl.ny;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < f.n; c += (size_t)gridDim.x * blockDim.x) {
    int i, j, k;
    cell_of(c, f.nx, f.ny, i, j, k);
    x[c] += cl.x[(size_t)k * pc + (size_t)(j >> 1) * cl.nx + (i >> 1)];
  }
}

// ---- Krylov kernels ----
// Dot products: an FP32 solver's threads accumulate their partial in FP32
// carrying the products' rounding errors (fmaf) and the sums' (Neumaier), so
// a partial is as accurate as an FP64 sum of the exact products while the
// FP64 pipe (a small fraction of the FP32 rate on this GPU) sees one
// conversion per thread; the partials are then summed in FP64. An FP64
// solver accumulates in FP64.
template <typename T>
struct DotAcc;
template <>
struct DotAcc<float> {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float v) {
    const float t = s + v;
    c += (fabsf(s) >= fabsf(v)) ? (s - t) + v : (v - t) + s;
    s = t;
  }
  __device__ __forceinline__ void prod(float a, float b) {
    const float p = a * b;
    add(p);
    c += fmaf(a, b, -p);
  }
  __device__ __forceinline__ double value() const { return (double)s + (double)c; }
};
template <>
struct DotAcc<double> {
  double s = 0.0;
  __device__ __forceinline__ void prod(double a, double b) { s = fma(a, b, s); }
  __device__ __forceinline__ double value() const { return s; }
};

__device__ __forceinline__ double block_sum(double v, double* sh) {
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int w = kMT / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  const double s = sh[0];
  __syncthreads();
  return s;
}

template <typename T>
__global__ void k_init(const double* __restrict__ r64, double inv, size_t n, T* r, T* r0, T* x, T* p, T* v,
                       double* part) {
  __shared__ double sh[kMT];
  DotAcc<T> acc;
  for (size_t q = blockIdx.x * (size_t)kMT + threadIdx.x; q < n; q += (size_t)gridDim.x * kMT) {
    const T rv = (T)(r64[q] * inv);
    r[q] = rv;
    r0[q] = rv;
    x[q] = 0;
    p[q] = 0;
    v[q] = 0;
    acc.prod(rv, rv);
  }
  const double s = block_sum(acc.value(), sh);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// p = r + beta (p - omega v), beta from the previous iteration's scalars
template <typename T>
__global__ void k_upd_p(const T* __restrict__ r, T* __restrict__ p, const T* __restrict__ v, size_t n,
                        const double* __restrict__ sc) {
  const T b = (T)sc[BETA], om = (T)sc[OMEGA];
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x)
    p[q] = r[q] + b * (p[q] - om * v[q]);
}

// y = A xin, partials of (w1, y) [and (y, y) when two]
template <typename T, bool kTwo>
__global__ void k_apply_dot(MgLevel<T> l, const T* __restrict__ xin, T* __restrict__ y, const T* __restrict__ w1,
                            double* part) {
  __shared__ double sh[kMT];
  DotAcc<T> a1, a2;
  for (size_t c = blockIdx.x * (size_t)kMT + threadIdx.x; c < l.n; c += (size_t)gridDim.x * kMT) {
    int i, j, k;
    cell_of(c, l.nx, l.ny, i, j, k);
    const T yv = apply_at(l, xin, c, i, j, k);
    y[c] = yv;
    a1.prod(w1[c], yv);
    if (kTwo) a2.prod(yv, yv);
  }
  const double s1 = block_sum(a1.value(), sh);
  if (threadIdx.x == 0) part[blockIdx.x] = s1;
  if (kTwo) {
    const double s2 = block_sum(a2.value(), sh);
    if (threadIdx.x == 0) part[kMgRedBlocks + blockIdx.x] = s2;
  }
}

// s = r - alpha v
template <typename T>
__global__ void k_upd_s(const T* __restrict__ r, const T* __restrict__ v, T* __restrict__ s, size_t n,
                        const double* __restrict__ sc) {
  const T al = (T)sc[ALPHA];
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x)
    s[q] = r[q] - al * v[q];
}

// x += alpha ph + omega sh; r = s - omega t; partials (r, r), (r0, r)
template <typename T>
__global__ void k_upd_xr(T* __restrict__ x, const T* __restrict__ ph, const T* __restrict__ shv,
                         const T* __restrict__ s, const T* __restrict__ t, T* __restrict__ r,
                         const T* __restrict__ r0, size_t n, const double* __restrict__ sc, double* part) {
  __shared__ double sh[kMT];
  const T al = (T)sc[ALPHA], om = (T)sc[OMEGA];
  DotAcc<T> a1, a2;
  for (size_t q = blockIdx.x * (size_t)kMT + threadIdx.x; q < n; q += (size_t)gridDim.x * kMT) {
    x[q] += al * ph[q] + om * shv[q];
    const T rv = s[q] - om * t[q];
    r[q] = rv;
    a1.prod(rv, rv);
    a2.prod(r0[q], rv);
  }
  const double s1 = block_sum(a1.value(), sh);
  if (threadIdx.x == 0) part[blockIdx.x] = s1;
  const double s2 = block_sum(a2.value(), sh);
  if (threadIdx.x == 0) part[kMgRedBlocks + blockIdx.x] = s2;
}

enum Op { OP_INIT = 0, OP_ALPHA = 1, OP_OMEGA = 2, OP_XR = 3 };

// use_cond: the iteration runs as the body of a graph WHILE node whose
// condition OP_XR sets (1 = go on, 0 = stop: converged, broken down, or at
// the iteration limit)
__global__ void k_finish(const double* __restrict__ part, int nb, int op, double* sc,
                         cudaGraphConditionalHandle cond, int use_cond) {
  __shared__ double sh[kMT];
  double a1 = 0.0, a2 = 0.0;
  for (int q = threadIdx.x; q < nb; q += kMT) {
    a1 += part[q];
    a2 += part[kMgRedBlocks + q];
  }
  const double s1 = block_sum(a1, sh);
  const double s2 = block_sum(a2, sh);
  if (threadIdx.x != 0) return;
  if (op == OP_INIT) {
    sc[RR] = s1;
    sc[RHO_NEW] = s1;
    sc[RHO_OLD] = 1.0;
    sc[ALPHA] = 1.0;
    sc[OMEGA] = 1.0;
    sc[BETA] = 0.0;  // (p = v = 0: the first p is r whatever beta is)
    sc[BREAK] = 0.0;
  } else if (op == OP_ALPHA) {
    sc[RV] = s1;
    if (s1 == 0.0 || !isfinite(s1)) {
      sc[BREAK] = 1.0;
      sc[ALPHA] = 0.0;
    } else {
      sc[ALPHA] = sc[RHO_NEW] / s1;
    }
  } else if (op == OP_OMEGA) {
    sc[TS] = s1;
    sc[TT] = s2;
    if (!(s2 > 0.0) || !isfinite(s2)) {
      sc[BREAK] = 1.0;
      sc[OMEGA] = 0.0;
    } else {
      sc[OMEGA] = s1 / s2;
      if (sc[OMEGA] == 0.0) sc[BREAK] = 1.0;
    }
  } else {  // OP_XR
    sc[RR] = s1;
    sc[RHO_OLD] = sc[RHO_NEW];
    sc[RHO_NEW] = s2;
    if (s2 == 0.0 || !isfinite(s1)) sc[BREAK] = 1.0;
    const double ro = sc[RHO_OLD], om = sc[OMEGA];
    sc[BETA] = (ro != 0.0 && om != 0.0) ? (s2 / ro) * (sc[ALPHA] / om) : 0.0;
    sc[ITERS] += 1.0;
    if (use_cond) {
      const bool stop = sc[BREAK] != 0.0 || !(s1 > sc[RTOL2]) || sc[ITERS] >= sc[MAXIT];
      cudaGraphSetConditional(cond, stop ? 0u : 1u);
    }
  }
}
__global__ void k_stop_test(double* sc, double rtol2, int max_iter) {
  sc[RTOL2] = rtol2;
  sc[MAXIT] = (double)max_iter;
  sc[ITERS] = 0.0;
}

template <typename T>
__global__ void k_out(const T* __restrict__ x, double scale, double* __restrict__ d, size_t n) {
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x)
    d[q] = (double)x[q] * scale;
}

int cells_grid(size_t n) {
  const size_t b = (n + kMT - 1) / kMT;
  return (int)(b < 4096 ? (b > 0 ? b : 1) : 4096);
}
int red_grid(size_t n) {
  const size_t b = (n + kMT - 1) / kMT;
  return (int)(b < (size_t)kMgRedBlocks ? (b > 0 ? b : 1) : kMgRedBlocks);
}
int cols_grid(const int cols) { return (cols + 127) / 128; }

// the launch of k_coarse_smooth: one cluster of ctas CTAs
void coarse_config(int ctas, size_t smem, cudaStream_t s, cudaLaunchConfig_t& cfg, cudaLaunchAttribute& at) {
  at = cudaLaunchAttribute{};
  at.id = cudaLaunchAttributeClusterDimension;
  at.val.clusterDim.x = ctas;
  at.val.clusterDim.y = 1;
  at.val.clusterDim.z = 1;
  cfg = cudaLaunchConfig_t{};
  cfg.gridDim = dim3(ctas);
  cfg.blockDim = dim3(256);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cfg.attrs = &at;
  cfg.numAttrs = 1;
}

template <typename T>
void smooth(const MgLevel<T>& l, const T* rhs, T* x, int color, int zero_nb, cudaStream_t s) {
  const size_t sm = scan_smem<T>(l.nz);
  if (sm <= kScanSmemMax) {  // (the shared-memory limit is raised in mg_create)
    const int g = ((l.nx + 1) / 2 * l.ny + 31) / 32;
    if (zero_nb)
      k_smooth_scan<T, true><<<g, 256, sm, s>>>(l, rhs, x, color);
    else
      k_smooth_scan<T, false><<<g, 256, sm, s>>>(l, rhs, x, color);
  } else {
    k_smooth<T><<<cols_grid(l.nx * l.ny), 128, 0, s>>>(l, rhs, x, color, zero_nb);
  }
}

// x = V(rhs) on level li (zero initial guess)
template <typename T>
void vcycle(MgSolver<T>* m, int li, const T* rhs, T* x, cudaStream_t s) {
  MgLevel<T>& l = m->lv[li];
  if (li == m->L - 1) {
    if (m->coarse_ctas > 0) {
      cudaLaunchConfig_t cfg;
      cudaLaunchAttribute at;
      coarse_config(m->coarse_ctas, scan_smem<T>(l.nz), s, cfg, at);
      cudaLaunchKernelEx(&cfg, k_coarse_smooth<T>, l, rhs, x);
      return;
    }
    smooth(l, rhs, x, 0, 1, s);
    smooth(l, rhs, x, 1, 0, s);
    for (int it = 1; it < kCoarseSweeps; ++it) {
      smooth(l, rhs, x, 0, 0, s);
      smooth(l, rhs, x, 1, 0, s);
    }
    return;
  }
  MgLevel<T>& cl = m->lv[li + 1];
  smooth(l, rhs, x, 0, 1, s);
  smooth(l, rhs, x, 1, 0, s);
  k_resid_restrict<T><<<cells_grid(cl.n), kMT, 0, s>>>(l, rhs, x, cl);
  vcycle(m, li + 1, cl.r, cl.x, s);
  k_prolong_add<T><<<cells_grid(l.n), kMT, 0, s>>>(l, x, cl);
  smooth(l, rhs, x, 1, 0, s);
  smooth(l, rhs, x, 0, 0, s);
}

template <typename T>
T* dev_alloc(MgSolver<T>* m, size_t n) {
  void* p = nullptr;
  if (cudaMalloc(&p, n * sizeof(T)) != cudaSuccess) return nullptr;
  m->allocs.push_back(p);
  return (T*)p;
}

}  // namespace

template <typename T>
MgSolver<T>* mg_create(const HGeo& g, int max_levels) {
  auto* m = new MgSolver<T>();
  m->g = g;
  int nx = g.nx, ny = g.ny;
  const int cap = max_levels < 1 ? 1 : (max_levels > kMgMaxLevels ? kMgMaxLevels : max_levels);
  bool ok = true;
  for (int l = 0; l < cap; ++l) {
    MgLevel<T>& L = m->lv[l];
    L.nx = nx;
    L.ny = ny;
    L.nz = g.nz;
    L.n = (size_t)nx * ny * g.nz;
    T** arrs[] = {&L.cE, &L.cN, &L.cT, &L.cB, &L.cD, &L.lc, &L.li, &L.x, &L.r};
    for (T** a : arrs) {
      *a = dev_alloc(m, L.n);
      ok = ok && *a != nullptr;
    }
    m->L = l + 1;
    if (nx % 2 || ny % 2 || nx / 2 < 4 || ny / 2 < 4) break;
    nx /= 2;
    ny /= 2;
  }
  const size_t n = g.n();
  T** kv[] = {&m->x, &m->r, &m->r0, &m->p, &m->v, &m->s, &m->t, &m->ph, &m->sh};
  for (T** a : kv) {
    *a = dev_alloc(m, n);
    ok = ok && *a != nullptr;
  }
  void* p = nullptr;
  ok = ok && cudaMalloc(&p, 2 * kMgRedBlocks * sizeof(double)) == cudaSuccess;
  if (p) m->allocs.push_back(p), m->part = (double*)p;
  p = nullptr;
  ok = ok && cudaMalloc(&p, NSC * sizeof(double)) == cudaSuccess;
  if (p) m->allocs.push_back(p), m->sc = (double*)p;
  ok = ok && cudaMallocHost(&m->hsc, NSC * sizeof(double)) == cudaSuccess;
  // the tiled smoother's FP64 tiles need more than the default 48 KB
  if (scan_smem<T>(g.nz) <= kScanSmemMax) {
    ok = ok && cudaFuncSetAttribute(k_smooth_scan<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)kScanSmemMax) == cudaSuccess;
    ok = ok && cudaFuncSetAttribute(k_smooth_scan<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)kScanSmemMax) == cudaSuccess;
    // the coarsest grid in one cluster launch when it is a few tiles: one
    // CTA per tile, up to a portable cluster (FP32 only: the FP64 rate of a
    // few SMs is far too low for the whole coarse solve)
    const MgLevel<T>& c = m->lv[m->L - 1];
    const int ntiles = ((c.nx + 1) / 2 * c.ny + 31) / 32;
    const int ctas = ntiles < kCoarseMaxCtas ? ntiles : kCoarseMaxCtas;
    if (sizeof(T) == 4 && ok && ntiles <= kCoarseMaxTiles) {
      ok = ok && cudaFuncSetAttribute(k_coarse_smooth<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)kScanSmemMax) == cudaSuccess;
      cudaLaunchConfig_t cfg;
      cudaLaunchAttribute at;
      coarse_config(ctas, scan_smem<T>(g.nz), nullptr, cfg, at);
      int clusters = 0;
      if (cudaOccupancyMaxActiveClusters(&clusters, k_coarse_smooth<T>, &cfg) == cudaSuccess && clusters > 0)
        m->coarse_ctas = ctas;
      cudaGetLastError();  // (a cluster launch that cannot run leaves the launches per half sweep)
    }
  }
  if (!ok) {
    mg_destroy(m);
    return nullptr;
  }
  return m;
}

template <typename T>
void mg_destroy(MgSolver<T>* m) {
  if (!m) return;
  if (m->gexec) cudaGraphExecDestroy(m->gexec);
  if (m->graph) cudaGraphDestroy(m->graph);
  for (void* p : m->allocs) cudaFree(p);
  if (m->hsc) cudaFreeHost(m->hsc);
  delete m;
}

template <typename T>
int mg_levels(const MgSolver<T>* m) {
  return m->L;
}

template <typename T>
int mg_set_coefficients(MgSolver<T>* m, const double* a, const double* b, cudaStream_t s) {
  k_fine_coefs<T><<<cells_grid(m->g.n()), kMT, 0, s>>>(m->g, a, b, m->lv[0]);
  for (int l = 1; l < m->L; ++l)
    k_coarse_coefs<T><<<cells_grid(m->lv[l].n), kMT, 0, s>>>(m->lv[l - 1], m->lv[l]);
  for (int l = 0; l < m->L; ++l)
    k_column_lu<T><<<cols_grid(m->lv[l].nx * m->lv[l].ny), 128, 0, s>>>(m->lv[l]);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// one BiCGSTAB iteration (right-preconditioned by a V-cycle)
template <typename T>
void enqueue_iteration(MgSolver<T>* m, cudaStream_t s, cudaGraphConditionalHandle cond, int use_cond) {
  const size_t n = m->g.n();
  const int nb = red_grid(n), cg = cells_grid(n);
  MgLevel<T>& f = m->lv[0];
  k_upd_p<T><<<cg, kMT, 0, s>>>(m->r, m->p, m->v, n, m->sc);
  vcycle(m, 0, m->p, m->ph, s);
  k_apply_dot<T, false><<<nb, kMT, 0, s>>>(f, m->ph, m->v, m->r0, m->part);
  k_finish<<<1, kMT, 0, s>>>(m->part, nb, OP_ALPHA, m->sc, cond, 0);
  k_upd_s<T><<<cg, kMT, 0, s>>>(m->r, m->v, m->s, n, m->sc);
  vcycle(m, 0, m->s, m->sh, s);
  k_apply_dot<T, true><<<nb, kMT, 0, s>>>(f, m->sh, m->t, m->s, m->part);
  k_finish<<<1, kMT, 0, s>>>(m->part, nb, OP_OMEGA, m->sc, cond, 0);
  k_upd_xr<T><<<nb, kMT, 0, s>>>(m->x, m->ph, m->sh, m->s, m->t, m->r, m->r0, n, m->sc, m->part);
  k_finish<<<1, kMT, 0, s>>>(m->part, nb, OP_XR, m->sc, cond, use_cond);
}

// The iteration loop as one graph: a WHILE conditional node (default 1 at
// every launch) whose body is one iteration captured from the stream.
template <typename T>
bool build_loop_graph(MgSolver<T>* m, cudaStream_t s) {
  cudaGraph_t g = nullptr;
  if (cudaGraphCreate(&g, 0) != cudaSuccess) return false;
  cudaGraphConditionalHandle cond;
  cudaGraphNodeParams p = {};
  cudaGraphNode_t node;
  cudaGraph_t captured = nullptr;
  bool ok = cudaGraphConditionalHandleCreate(&cond, g, 1, cudaGraphCondAssignDefault) == cudaSuccess;
  if (ok) {
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = cond;
    p.conditional.type = cudaGraphCondTypeWhile;
    p.conditional.size = 1;
    ok = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &p) == cudaSuccess;
  }
  if (ok) {
    cudaGraph_t body = p.conditional.phGraph_out[0];
    ok = cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) ==
         cudaSuccess;
    if (ok) {
      enqueue_iteration(m, s, cond, 1);
      ok = cudaStreamEndCapture(s, &captured) == cudaSuccess && captured == body;
    }
  }
  if (ok) ok = cudaGraphInstantiate(&m->gexec, g, 0) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();  // the host loop takes over
    if (m->gexec) cudaGraphExecDestroy(m->gexec);
    m->gexec = nullptr;
    cudaGraphDestroy(g);
    return false;
  }
  m->graph = g;
  return true;
}

template <typename T>
int mg_solve(MgSolver<T>* m, const double* r64, double* d64, double rtol, int max_iter, cudaStream_t s,
             double r_norm2) {
  const size_t n = m->g.n();
  const int nb = red_grid(n), cg = cells_grid(n);
  // scale the right-hand side to unit norm (FP32 range), FP64 dot
  if (r_norm2 < 0.0) {
    dot64(r64, r64, n, m->part, m->sc + NSC - 1, s);
    if (cudaMemcpyAsync(m->hsc, m->sc + NSC - 1, sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess)
      return -1;
    if (cudaStreamSynchronize(s) != cudaSuccess) return -1;
    r_norm2 = m->hsc[0];
  }
  const double rn = std::sqrt(r_norm2);
  if (!(rn > 0.0) || !std::isfinite(rn)) {
    cudaMemsetAsync(d64, 0, n * sizeof(double), s);
    return 0;
  }
  k_init<T><<<nb, kMT, 0, s>>>(r64, 1.0 / rn, n, m->r, m->r0, m->x, m->p, m->v, m->part);
  k_finish<<<1, kMT, 0, s>>>(m->part, nb, OP_INIT, m->sc, cudaGraphConditionalHandle{}, 0);
  k_stop_test<<<1, 1, 0, s>>>(m->sc, rtol * rtol, max_iter);
  if (m->graph_state == 0) {
    // VIBE_GB300_HELMHOLTZ_GRAPH=0 keeps the host loop (one scalar read per iteration)
    const char* e = std::getenv("VIBE_GB300_HELMHOLTZ_GRAPH");
    m->graph_state = (e && std::atoi(e) == 0) ? -1 : (build_loop_graph(m, s) ? 1 : -1);
  }
  int it = 0;
  bool broke = false;
  if (m->graph_state == 1 && max_iter > 0) {
    // the whole loop on the device: one launch, one read of the scalars
    if (cudaGraphLaunch(m->gexec, s) != cudaSuccess) return -1;
    if (cudaMemcpyAsync(m->hsc, m->sc, NSC * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess) return -1;
    if (cudaStreamSynchronize(s) != cudaSuccess) return -1;
    it = (int)m->hsc[ITERS];
    broke = m->hsc[BREAK] != 0.0;
  } else {
    for (; it < max_iter; ++it) {
      enqueue_iteration(m, s, cudaGraphConditionalHandle{}, 0);
      if (cudaMemcpyAsync(m->hsc, m->sc, NSC * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess) return -1;
      if (cudaStreamSynchronize(s) != cudaSuccess) return -1;
      if (m->hsc[BREAK] != 0.0) {
        broke = true;
        ++it;
        break;
      }
      if (std::sqrt(m->hsc[RR]) <= rtol) {
        ++it;
        break;
      }
    }
  }
  k_out<T><<<cg, kMT, 0, s>>>(m->x, rn, d64, n);
  if (cudaGetLastError() != cudaSuccess) return -1;
  return broke ? -it : it;
}

template MgSolver<float>* mg_create<float>(const HGeo&, int);
template MgSolver<double>* mg_create<double>(const HGeo&, int);
template void mg_destroy<float>(MgSolver<float>*);
template void mg_destroy<double>(MgSolver<double>*);
template int mg_levels<float>(const MgSolver<float>*);
template int mg_levels<double>(const MgSolver<double>*);
template int mg_set_coefficients<float>(MgSolver<float>*, const double*, const double*, cudaStream_t);
template int mg_set_coefficients<double>(MgSolver<double>*, const double*, const double*, cudaStream_t);
template int mg_solve<float>(MgSolver<float>*, const double*, double*, double, int, cudaStream_t, double);
template int mg_solve<double>(MgSolver<double>*, const double*, double*, double, int, cudaStream_t, double);

}  // namespace vgb
