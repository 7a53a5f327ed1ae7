// vibe-model_gb300/csrc/nest.cu
//
// Nest transfers (include/vibe_nest.h): the reference's grid::Nest
// operations (src/grid/nest.cpp:34-124) as device kernels. Built without FMA
// contraction so the interpolation weights, the r x r means and the Davies
// blend give the reference's bits. A field is addressed through an affine
// view (element (i, j, k) at off + k*sk + j*sj + i), which covers the
// reference's FieldT storage and the model's device layout alike; one launch
// transfers up to kNestVars fields.
#include <cmath>
#include <string>
#include <vector>

#include "vibe_internal.cuh"
#include "vibe_nest.h"

namespace vgb {

constexpr int kNestVars = 16;
constexpr int kNestZone = 64;
constexpr int kHalo = 4;

struct NestViews {
  double* p[kNestVars];
  long long off[kNestVars], sk[kNestVars];
  int sj[kNestVars];
};

struct NestArgs {
  int i0, j0, iext, jext, ratio, nzone;
  int pnx, pny, pnz, cnx, cny, cnz, nvars;
  double inv, w;
  double davies[kNestZone];
};

namespace {

__device__ __forceinline__ double& at(const NestViews& v, int q, int i, int j, int k) {
  return v.p[q][v.off[q] + (long long)k * v.sk[q] + (long long)j * v.sj[q] + i];
}
__device__ __forceinline__ double lerpd(double a, double b, double w) { return a + w * (b - a); }

__device__ __forceinline__ void interp_point(const NestArgs& a, const NestViews& P, const NestViews& C, int i, int j,
                                             int k) {
  const double xp = ((double)(a.i0 + i) + 0.5) * a.inv - 0.5;
  const double yp = ((double)(a.j0 + j) + 0.5) * a.inv - 0.5;
  const int ip = (int)floor(xp), jp = (int)floor(yp);
  const double wx = xp - (double)ip, wy = yp - (double)jp;
  const int i0 = iclamp(ip, 0, a.pnx - 1), i1 = iclamp(ip + 1, 0, a.pnx - 1);
  const int j0 = iclamp(jp, 0, a.pny - 1), j1 = iclamp(jp + 1, 0, a.pny - 1);
  const int kp = iclamp(k, 0, a.pnz - 1);
  for (int q = 0; q < a.nvars; ++q) {
    at(C, q, i, j, k) = lerpd(lerpd(at(P, q, i0, j0, kp), at(P, q, i1, j0, kp), wx),
                              lerpd(at(P, q, i0, j1, kp), at(P, q, i1, j1, kp), wx), wy);
  }
}
__global__ void k_interp(const __grid_constant__ NestArgs a, const __grid_constant__ NestViews P,
                         const __grid_constant__ NestViews C) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
  if (i >= a.cnx || j >= a.cny) return;
  interp_point(a, P, C, i, j, k);
}
// only the points of the Davies zone (the ones k_lateral reads), one thread
// per (frame column, level)
__global__ void k_interp_zone(const __grid_constant__ NestArgs a, const __grid_constant__ NestViews P,
                              const __grid_constant__ NestViews C, int nframe) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.z;
  if (e >= nframe) return;
  int i, j;
  frame_column(e, a.cnx, a.cny, a.nzone, i, j);
  interp_point(a, P, C, i, j, k);
}

__global__ void k_restrict(const __grid_constant__ NestArgs a, const __grid_constant__ NestViews C,
                           const __grid_constant__ NestViews P) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
  if (i >= a.iext || j >= a.jext) return;
  const int r = a.ratio, kc = iclamp(k, 0, a.cnz - 1);
  for (int q = 0; q < a.nvars; ++q) {
    double acc = 0.0;
    for (int jj = 0; jj < r; ++jj) {
      const int cj = iclamp(j * r + jj, 0, a.cny - 1);
      for (int ii = 0; ii < r; ++ii) acc += at(C, q, iclamp(i * r + ii, 0, a.cnx - 1), cj, kc);
    }
    at(P, q, a.i0 + i, a.j0 + j, k) = acc * a.w;
  }
}

__global__ void k_lateral(const __grid_constant__ NestArgs a, const __grid_constant__ NestViews C,
                          const __grid_constant__ NestViews PI) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
  if (i >= a.cnx || j >= a.cny) return;
  const int d = imin(imin(i, a.cnx - 1 - i), imin(j, a.cny - 1 - j));
  if (d >= a.nzone) return;
  const double alpha = a.davies[d];
  for (int q = 0; q < a.nvars; ++q) {
    double& c = at(C, q, i, j, k);
    c = (1.0 - alpha) * c + alpha * at(PI, q, i, j, k);
  }
}

thread_local std::string g_nerr;

// FieldT storage view of field q (nx, ny, nz grid, halo 4)
void fieldt_view(NestViews& v, int q, double* p, int nx, int ny, int stagger) {
  const long long nsx = nx + 2 * kHalo + (stagger == 1), nsy = ny + 2 * kHalo + (stagger == 2);
  v.p[q] = p;
  v.sj[q] = (int)nsx;
  v.sk[q] = nsx * nsy;
  v.off[q] = (kHalo * nsy + kHalo) * nsx + kHalo;
}

size_t fieldt_size(int nx, int ny, int nz, int stagger) {
  return (size_t)(nx + 2 * kHalo + (stagger == 1)) * (ny + 2 * kHalo + (stagger == 2)) *
         (nz + 2 * kHalo + (stagger == 3));
}

bool check_placement(const vibe_nest_placement* p) {
  if (!p || p->ratio < 2 || p->boundary_zone < 1 || p->boundary_zone > kNestZone || p->iext < 0 || p->jext < 0) {
    g_nerr = "bad placement (ratio >= 2, 1 <= boundary_zone <= 64, extents >= 0)";
    return false;
  }
  return true;
}

NestArgs args_of(const vibe_nest_placement* p, int pnx, int pny, int pnz, int cnx, int cny, int cnz) {
  NestArgs a{};
  a.i0 = p->i0;
  a.j0 = p->j0;
  a.iext = p->iext;
  a.jext = p->jext;
  a.ratio = p->ratio;
  a.nzone = p->boundary_zone;
  a.pnx = pnx; a.pny = pny; a.pnz = pnz;
  a.cnx = cnx; a.cny = cny; a.cnz = cnz;
  a.inv = 1.0 / (double)p->ratio;
  a.w = 1.0 / (double)(p->ratio * p->ratio);
  vibe_davies_profile(p->boundary_zone, 1.0, a.davies);
  return a;
}

enum Op { INTERP, RESTRICT, LATERAL };

int run_dev(Op op, const vibe_nest_placement* p, int nvars, const int* stagger, int pnx, int pny, int pnz,
            const double* const* parent, int cnx, int cny, int cnz, const double* const* child_in,
            double* const* out, cudaStream_t s) {
  if (!check_placement(p)) return VIBE_C_ERR_BAD_ARG;
  if (nvars < 0 || (nvars > 0 && (!stagger || !out)) || pnx <= 0 || pny <= 0 || pnz <= 0 || cnx <= 0 || cny <= 0 ||
      cnz <= 0) {
    g_nerr = "bad sizes or NULL arrays";
    return VIBE_C_ERR_BAD_ARG;
  }
  if (op == RESTRICT && (p->i0 < -kHalo || p->j0 < -kHalo || p->i0 + p->iext > pnx + kHalo ||
                         p->j0 + p->jext > pny + kHalo)) {
    g_nerr = "restriction box outside the parent's storage";
    return VIBE_C_ERR_BAD_ARG;
  }
  NestArgs a = args_of(p, pnx, pny, pnz, cnx, cny, cnz);
  for (int v0 = 0; v0 < nvars; v0 += kNestVars) {
    NestViews A{}, B{};
    const int nv = imin(kNestVars, nvars - v0);
    a.nvars = nv;
    for (int q = 0; q < nv; ++q) {
      const int st = stagger[v0 + q];
      if (st < 0 || st > 3) {
        g_nerr = "bad stagger";
        return VIBE_C_ERR_BAD_ARG;
      }
      if (op == INTERP) {
        fieldt_view(A, q, const_cast<double*>(parent[v0 + q]), pnx, pny, st);
        fieldt_view(B, q, out[v0 + q], cnx, cny, st);
      } else if (op == RESTRICT) {
        fieldt_view(A, q, const_cast<double*>(child_in[v0 + q]), cnx, cny, st);
        fieldt_view(B, q, out[v0 + q], pnx, pny, st);
      } else {
        fieldt_view(A, q, out[v0 + q], cnx, cny, st);
        fieldt_view(B, q, const_cast<double*>(child_in[v0 + q]), cnx, cny, st);
      }
    }
    const dim3 b(32, 8);
    if (op == INTERP)
      k_interp<<<dim3((cnx + 31) / 32, (cny + 7) / 8, cnz), b, 0, s>>>(a, A, B);
    else if (op == RESTRICT) {
      if (p->iext > 0 && p->jext > 0)
        k_restrict<<<dim3((p->iext + 31) / 32, (p->jext + 7) / 8, pnz), b, 0, s>>>(a, A, B);
    } else
      k_lateral<<<dim3((cnx + 31) / 32, (cny + 7) / 8, cnz), b, 0, s>>>(a, A, B);
  }
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    g_nerr = cudaGetErrorString(e);
    return VIBE_C_ERR_DEVICE;
  }
  return VIBE_C_OK;
}

// host form: stage the fields through device memory on a private stream
int run_host(Op op, const vibe_nest_placement* p, int nvars, const int* stagger, int pnx, int pny, int pnz,
             const double* const* parent, int cnx, int cny, int cnz, const double* const* child_in,
             double* const* out) {
  if (nvars <= 0) return check_placement(p) ? VIBE_C_OK : VIBE_C_ERR_BAD_ARG;
  if (!stagger || !out) {
    g_nerr = "NULL arrays";
    return VIBE_C_ERR_BAD_ARG;
  }
  cudaStream_t s = nullptr;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
    g_nerr = "stream";
    return VIBE_C_ERR_DEVICE;
  }
  std::vector<double*> dsrc(nvars, nullptr), dout(nvars, nullptr);
  int rc = VIBE_C_OK;
  const bool outer_parent = (op == RESTRICT);
  for (int v = 0; v < nvars && rc == VIBE_C_OK; ++v) {
    const int st = (stagger[v] >= 0 && stagger[v] <= 3) ? stagger[v] : 0;
    const size_t ns = (op == INTERP) ? fieldt_size(pnx, pny, pnz, st) : fieldt_size(cnx, cny, cnz, st);
    const size_t no = outer_parent ? fieldt_size(pnx, pny, pnz, st) : fieldt_size(cnx, cny, cnz, st);
    const double* hs = (op == INTERP) ? parent[v] : child_in[v];
    if (!hs || !out[v] || cudaMalloc(&dsrc[v], ns * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&dout[v], no * sizeof(double)) != cudaSuccess ||
        cudaMemcpyAsync(dsrc[v], hs, ns * sizeof(double), cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(dout[v], out[v], no * sizeof(double), cudaMemcpyHostToDevice, s) != cudaSuccess) {
      g_nerr = "staging failed";
      rc = (!hs || !out[v]) ? VIBE_C_ERR_BAD_ARG : VIBE_C_ERR_DEVICE;
    }
  }
  if (rc == VIBE_C_OK) {
    std::vector<const double*> src(dsrc.begin(), dsrc.end());
    rc = (op == INTERP) ? run_dev(op, p, nvars, stagger, pnx, pny, pnz, src.data(), cnx, cny, cnz, nullptr,
                                  dout.data(), s)
                        : run_dev(op, p, nvars, stagger, pnx, pny, pnz, nullptr, cnx, cny, cnz, src.data(),
                                  dout.data(), s);
  }
  for (int v = 0; v < nvars && rc == VIBE_C_OK; ++v) {
    const int st = stagger[v];
    const size_t no = outer_parent ? fieldt_size(pnx, pny, pnz, st) : fieldt_size(cnx, cny, cnz, st);
    if (cudaMemcpyAsync(out[v], dout[v], no * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess) {
      g_nerr = "copy back failed";
      rc = VIBE_C_ERR_DEVICE;
    }
  }
  if (cudaStreamSynchronize(s) != cudaSuccess && rc == VIBE_C_OK) {
    g_nerr = "nest kernels failed";
    rc = VIBE_C_ERR_DEVICE;
  }
  for (int v = 0; v < nvars; ++v) {
    cudaFree(dsrc[v]);
    cudaFree(dout[v]);
  }
  cudaStreamDestroy(s);
  return rc;
}

}  // namespace

// The same transfers on fields in the model's device layout (element (i,j,k)
// at k*plane + j*pitch + i, no halo): op 0 interpolate parent -> child,
// 1 restrict child -> parent, 2 Davies blend of child with child_in. The
// restriction box must lie inside the parent's interior plus its extra face.
int nest_model_layout(int op, const vibe_nest_placement* p, int nvars, int pnx, int pny, int pnz,
                      const double* const* parent, size_t p_pitch, size_t p_plane, int cnx, int cny, int cnz,
                      const double* const* child_in, double* const* out, size_t c_pitch, size_t c_plane,
                      cudaStream_t s, bool zone_only) {
  if (!check_placement(p)) return VIBE_C_ERR_BAD_ARG;
  if (op == 1 && (p->i0 < 0 || p->j0 < 0 || p->i0 + p->iext > pnx + 1 || p->j0 + p->jext > pny + 1)) {
    g_nerr = "restriction box outside the parent";
    return VIBE_C_ERR_BAD_ARG;
  }
  NestArgs a = args_of(p, pnx, pny, pnz, cnx, cny, cnz);
  auto view = [](NestViews& v, int q, const double* ptr, size_t pitch, size_t plane) {
    v.p[q] = const_cast<double*>(ptr);
    v.sj[q] = (int)pitch;
    v.sk[q] = (long long)plane;
    v.off[q] = 0;
  };
  for (int v0 = 0; v0 < nvars; v0 += kNestVars) {
    NestViews A{}, B{};
    const int nv = imin(kNestVars, nvars - v0);
    a.nvars = nv;
    for (int q = 0; q < nv; ++q) {
      if (op == 0) {
        view(A, q, parent[v0 + q], p_pitch, p_plane);
        view(B, q, out[v0 + q], c_pitch, c_plane);
      } else if (op == 1) {
        view(A, q, child_in[v0 + q], c_pitch, c_plane);
        view(B, q, out[v0 + q], p_pitch, p_plane);
      } else {
        view(A, q, out[v0 + q], c_pitch, c_plane);
        view(B, q, child_in[v0 + q], c_pitch, c_plane);
      }
    }
    const dim3 b(32, 8);
    if (op == 0 && zone_only) {
      const int nf = frame_count(cnx, cny, a.nzone);
      k_interp_zone<<<dim3((nf + 127) / 128, 1, cnz), 128, 0, s>>>(a, A, B, nf);
    } else if (op == 0)
      k_interp<<<dim3((cnx + 31) / 32, (cny + 7) / 8, cnz), b, 0, s>>>(a, A, B);
    else if (op == 1) {
      if (p->iext > 0 && p->jext > 0)
        k_restrict<<<dim3((p->iext + 31) / 32, (p->jext + 7) / 8, pnz), b, 0, s>>>(a, A, B);
    } else
      k_lateral<<<dim3((cnx + 31) / 32, (cny + 7) / 8, cnz), b, 0, s>>>(a, A, B);
  }
  return cudaGetLastError() == cudaSuccess ? VIBE_C_OK : VIBE_C_ERR_DEVICE;
}

namespace {
}  // namespace
}  // namespace vgb

using namespace vgb;

extern "C" {

int vibe_davies_profile(int n_zone, double alpha_max, double* out) {
  if (n_zone < 0 || (n_zone > 0 && !out)) return VIBE_C_ERR_BAD_ARG;
  for (int n = 0; n < n_zone; ++n) {
    const double arg = kPi * (double)(n_zone - n) / (double)n_zone;
    out[n] = alpha_max * 0.5 * (1.0 - std::cos(arg));
  }
  return VIBE_C_OK;
}

int vibe_nest_interpolate_from_parent_dev(const vibe_nest_placement* p, int nvars, const int* stagger, int pnx,
                                          int pny, int pnz, const double* const* parent, int cnx, int cny, int cnz,
                                          double* const* child, vibe_stream_t stream) {
  if (nvars > 0 && !parent) return VIBE_C_ERR_BAD_ARG;
  return run_dev(INTERP, p, nvars, stagger, pnx, pny, pnz, parent, cnx, cny, cnz, nullptr, child,
                 (cudaStream_t)stream);
}
int vibe_nest_restrict_to_parent_dev(const vibe_nest_placement* p, int nvars, const int* stagger, int cnx, int cny,
                                     int cnz, const double* const* child, int pnx, int pny, int pnz,
                                     double* const* parent, vibe_stream_t stream) {
  if (nvars > 0 && !child) return VIBE_C_ERR_BAD_ARG;
  return run_dev(RESTRICT, p, nvars, stagger, pnx, pny, pnz, nullptr, cnx, cny, cnz, child, parent,
                 (cudaStream_t)stream);
}
int vibe_nest_apply_lateral_boundary_dev(const vibe_nest_placement* p, int nvars, const int* stagger, int cnx,
                                         int cny, int cnz, double* const* child, const double* const* parent_interp,
                                         vibe_stream_t stream) {
  if (nvars > 0 && !parent_interp) return VIBE_C_ERR_BAD_ARG;
  return run_dev(LATERAL, p, nvars, stagger, cnx, cny, cnz, nullptr, cnx, cny, cnz, parent_interp, child,
                 (cudaStream_t)stream);
}
int vibe_nest_interpolate_from_parent(const vibe_nest_placement* p, int nvars, const int* stagger, int pnx, int pny,
                                      int pnz, const double* const* parent, int cnx, int cny, int cnz,
                                      double* const* child) {
  if (nvars > 0 && !parent) return VIBE_C_ERR_BAD_ARG;
  return run_host(INTERP, p, nvars, stagger, pnx, pny, pnz, parent, cnx, cny, cnz, nullptr, child);
}
int vibe_nest_restrict_to_parent(const vibe_nest_placement* p, int nvars, const int* stagger, int cnx, int cny,
                                 int cnz, const double* const* child, int pnx, int pny, int pnz,
                                 double* const* parent) {
  if (nvars > 0 && !child) return VIBE_C_ERR_BAD_ARG;
  return run_host(RESTRICT, p, nvars, stagger, pnx, pny, pnz, nullptr, cnx, cny, cnz, child, parent);
}
int vibe_nest_apply_lateral_boundary(const vibe_nest_placement* p, int nvars, const int* stagger, int cnx, int cny,
                                     int cnz, double* const* child, const double* const* parent_interp) {
  if (nvars > 0 && !parent_interp) return VIBE_C_ERR_BAD_ARG;
  return run_host(LATERAL, p, nvars, stagger, cnx, cny, cnz, nullptr, cnx, cny, cnz, parent_interp, child);
}

}  // extern "C"
