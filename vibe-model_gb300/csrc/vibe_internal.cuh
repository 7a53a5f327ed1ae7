// vibe-model_gb300/csrc/vibe_internal.cuh
//
// Device data layout and shared helpers of the GB300 dynamics step.
//
// Layout in HBM. Every prognostic field of one domain uses the same 3-D
// index, so one thread computes one offset for all fields it touches:
//     idx(i, j, k) = (k * NY1 + j) * P + i,   NY1 = ny + 1,
//     P = pitch in elements >= nx + 1, rounded up to 8 (64-byte rows).
// u faces use i = 0..nx, v faces j = 0..ny, w faces k = 0..nz (nz+1 planes),
// cells i < nx, j < ny, k < nz. The cell fields keep one ghost column
// (i = nx) and one ghost row (j = ny): they hold the caller's halo values at
// those points, which the reference's serial step reads without a clamp
// (src/dyn/equations.cpp:120-123, rho(i+1) and rho(j+1)) and never writes.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace vgb {

// include/vibe/common/constants.hpp:16-60
constexpr double kG = 9.80665;
constexpr double kRd = 287.05;
constexpr double kCp = 1004.64;
constexpr double kCv = 717.63;
constexpr double kEpsVap = 0.62197;
constexpr double kP0 = 100000.0;
constexpr double kPi = 3.14159265358979323846;
constexpr double kOmega = 7.2921159e-5;
constexpr double kEarthRadius = 6.371229e6;
constexpr double kBuoyMoist = 0.608;  // equations.cpp:40

enum Species { U = 0, V, W, RHO, THETA, PI, QV, QC, QR, QI, QS, QG, NSPECIES };

struct Dims {
  int nx, ny, nz;
  int P;        // pitch (elements)
  int NY1;      // ny + 1
  size_t plane; // NY1 * P
  __host__ __device__ size_t idx(int i, int j, int k) const {
    return ((size_t)k * NY1 + j) * (size_t)P + i;
  }
};

// Per-domain constants for the FP64 path (mirrors the reference's metric
// accessors; all arrays are device pointers).
struct Metric {
  double dx, dy, z_top;
  const double* dzeta;   // nz (dzeta(k) = zeta[k+1]-zeta[k], geometry.cpp:242-245)
  const double* scale;   // nx*ny: z_top - zs(i,j)
  const double* sponge;  // nz: damping.cpp:24-41 profile
  const double* th0;     // 3-D reference theta0 (cell layout)
  const double* pi0;
  const double* rho0;
  double f0, beta;       // Coriolis (coriolis.cpp:25-41)
  double inv_dx, inv_dy; // 1/dx, 1/dy (the fast FP64 build multiplies by them)
};

// Composition switches (same meaning as the setup struct in vibe_gb300.h).
struct Flags {
  int advection;         // 2/4/6 central, 5 = weno5 id
  int weno_scalars;
  int weno_advective;
  int moist;
  int coriolis;          // 0 none, 1 f-plane, 2 beta-plane
  double div_damp;
  int div_order;
  int pgf_pert;
  int split_fast;
  int acoustic_mode;     // 0 explicit FB, 1 reference HEVI, 2 consistent HEVI
  double hevi_beta;
  int w_rigid;           // w = 0 on the ground and lid faces after every step
};

__host__ __device__ inline int iclamp(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }
__host__ __device__ inline int imin(int a, int b) { return (b < a) ? b : a; }
__host__ __device__ inline int imax(int a, int b) { return (a < b) ? b : a; }
__host__ __device__ inline double dmax(double a, double b) { return (a < b) ? b : a; }

// The lateral frame of an nx x ny cell grid: the columns within f points of
// its edge (min(i, nx-1-i, j, ny-1-j) < f), numbered bottom rows, top rows,
// then the left and right ends of the rows between. frame_count gives how
// many, frame_column the e-th one.
__host__ __device__ inline void frame_shape(int nx, int ny, int f, int& rb, int& rt, int& cl, int& cr) {
  rb = imin(f, ny);
  rt = imin(f, ny - rb);
  const int mid = ny - rb - rt;
  cl = mid > 0 ? imin(f, nx) : 0;
  cr = mid > 0 ? imin(f, nx - cl) : 0;
}
__host__ __device__ inline int frame_count(int nx, int ny, int f) {
  int rb, rt, cl, cr;
  frame_shape(nx, ny, f, rb, rt, cl, cr);
  return (rb + rt) * nx + (ny - rb - rt) * (cl + cr);
}
__host__ __device__ inline void frame_column(int e, int nx, int ny, int f, int& i, int& j) {
  int rb, rt, cl, cr;
  frame_shape(nx, ny, f, rb, rt, cl, cr);
  const int nrow = (rb + rt) * nx;
  if (e < nrow) {
    const int r = e / nx;
    i = e - r * nx;
    j = r < rb ? r : ny - rt + (r - rb);
  } else {
    const int e2 = e - nrow, w = cl + cr, r = e2 / w, c = e2 - r * w;
    j = rb + r;
    i = c < cl ? c : nx - cr + (c - cl);
  }
}
__host__ __device__ inline float fmaxr(float a, float b) { return (a < b) ? b : a; }

// Error word bits written by kernels, read by the host once per step.
enum ErrorBits : unsigned { kErrNonFinite = 1u, kErrSingular = 2u, kErrWaitTimeout = 4u };

}  // namespace vgb
