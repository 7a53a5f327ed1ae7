// vibe-model_gb300/csrc/helmholtz_api.cu
//
// Host side of the Helmholtz solvers: the C ABI of include/vibe_helmholtz.h
// (the reference's HelmholtzSolver family, src/time/helmholtz.cpp:126-495),
// the reference's Jacobi-BiCGSTAB loop driven from the host with FP64
// device kernels, and the FP64 iterative-refinement loop around the
// multigrid-preconditioned BiCGSTAB.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "helmholtz.cuh"
#include "vibe_helmholtz.h"

using namespace vgb;

namespace {
thread_local std::string g_herr;
constexpr int kHalo = 4;
constexpr int kMgLevelsDefault = 5;
constexpr int kMaxRefinements = 30;  // FP64 refinement passes of kinds 3-4

bool ok(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return true;
  g_herr = std::string(what) + ": " + cudaGetErrorString(e);
  return false;
}
}  // namespace

struct vibe_helmholtz {
  int kind = 0, max_iter = 200;
  double tol = 1e-8;
  bool refine = true;
  HGeo g{};
  double *d_dzeta = nullptr, *d_scale = nullptr;
  double *a = nullptr, *b = nullptr, *f = nullptr, *x = nullptr;
  // work vectors: r, r0, p, v, s, t, prec, rhat/shat, lx/dx
  double* w[10] = {};
  double *part = nullptr, *scal = nullptr, *hscal = nullptr;
  unsigned *err = nullptr, *herr = nullptr;
  MgSolver<float>* mg32 = nullptr;
  MgSolver<double>* mg64 = nullptr;
  cudaStream_t stream = nullptr;
  bool coef = false;
  int iterations = 0;
  double residual = 1.0;
  std::vector<double> hbuf;  // host staging (device layout)
};

namespace {

size_t cells(const vibe_helmholtz* h) { return h->g.n(); }

// FieldT cell storage <-> device layout (nx*ny*nz, i fastest)
void pack(const vibe_helmholtz* h, const double* st, double* out) {
  const int nx = h->g.nx, ny = h->g.ny, nz = h->g.nz, sx = nx + 2 * kHalo, sy = ny + 2 * kHalo;
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      std::memcpy(out + ((size_t)k * ny + j) * nx, st + ((size_t)(k + kHalo) * sy + (j + kHalo)) * sx + kHalo,
                  sizeof(double) * nx);
}
void unpack(const vibe_helmholtz* h, const double* in, double* st) {
  const int nx = h->g.nx, ny = h->g.ny, nz = h->g.nz, sx = nx + 2 * kHalo, sy = ny + 2 * kHalo;
  std::memset(st, 0, sizeof(double) * (size_t)sx * sy * (nz + 2 * kHalo));
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      std::memcpy(st + ((size_t)(k + kHalo) * sy + (j + kHalo)) * sx + kHalo, in + ((size_t)k * ny + j) * nx,
                  sizeof(double) * nx);
}
bool upload(vibe_helmholtz* h, const double* st, double* dev) {
  pack(h, st, h->hbuf.data());
  return ok(cudaMemcpyAsync(dev, h->hbuf.data(), cells(h) * sizeof(double), cudaMemcpyHostToDevice, h->stream),
            "upload") &&
         ok(cudaStreamSynchronize(h->stream), "upload sync");
}
bool download(vibe_helmholtz* h, const double* dev, double* st) {
  if (!ok(cudaMemcpyAsync(h->hbuf.data(), dev, cells(h) * sizeof(double), cudaMemcpyDeviceToHost, h->stream),
          "download") ||
      !ok(cudaStreamSynchronize(h->stream), "download sync"))
    return false;
  unpack(h, h->hbuf.data(), st);
  return true;
}

// dot product read back to the host (the reference's serial dot_field,
// helmholtz.cpp:203-207, summed in a fixed tree order here)
bool hdot(vibe_helmholtz* h, const double* x, const double* y, cudaStream_t s, double& out) {
  dot64(x, y, cells(h), h->part, h->scal, s);
  if (!ok(cudaMemcpyAsync(h->hscal, h->scal, sizeof(double), cudaMemcpyDeviceToHost, s), "dot readback") ||
      !ok(cudaStreamSynchronize(s), "dot sync"))
    return false;
  out = h->hscal[0];
  return true;
}

// KrylovJacobiSolver::solve, helmholtz.cpp:296-366, step for step: x = 0;
// each iteration recomputes v = A x and r = f - v, takes rhat = M r,
// updates p with that v, and moves x by alpha p + omega s
int krylov_jacobi(vibe_helmholtz* h, const double* f, double* x, cudaStream_t s, int& iters, double& res) {
  const size_t n = cells(h);
  double *r = h->w[0], *r0 = h->w[1], *p = h->w[2], *v = h->w[3], *sv = h->w[4], *t = h->w[5], *prec = h->w[6],
         *hat = h->w[7];
  hz_jacobi_prec(h->g, h->a, h->b, prec, s);
  cudaMemsetAsync(x, 0, n * sizeof(double), s);
  cudaMemcpyAsync(r, f, n * sizeof(double), cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(r0, f, n * sizeof(double), cudaMemcpyDeviceToDevice, s);
  cudaMemsetAsync(p, 0, n * sizeof(double), s);
  cudaMemsetAsync(v, 0, n * sizeof(double), s);
  double rho = 1.0, alpha = 1.0, omega = 1.0, rho_prev = 1.0, ff = 0.0;
  if (!hdot(h, f, f, s, ff)) return VIBE_C_ERR_DEVICE;
  const double f_norm = std::sqrt(dmax(ff, 1e-300));
  res = 1.0;
  int it = 0;
  for (; it < h->max_iter; ++it) {
    hz_apply_ref(h->g, h->a, h->b, x, v, s);
    vop_sub(f, v, r, n, s);
    double rr = 0.0;
    if (!hdot(h, r, r, s, rr)) return VIBE_C_ERR_DEVICE;
    res = std::sqrt(rr) / f_norm;
    if (res < h->tol) break;
    vop_mul(prec, r, hat, n, s);
    if (!hdot(h, hat, r0, s, rho)) return VIBE_C_ERR_DEVICE;
    if (std::fabs(rho) < 1e-300) break;
    const double beta = (rho / rho_prev) * (alpha / omega);
    vop_pupdate(hat, p, v, beta, omega, n, s);
    hz_apply_ref(h->g, h->a, h->b, p, v, s);
    double denom = 0.0;
    if (!hdot(h, r0, v, s, denom)) return VIBE_C_ERR_DEVICE;
    alpha = (std::fabs(denom) > 1e-300) ? rho / denom : 0.0;
    vop_axpy_to(r, v, alpha, sv, n, s);
    double ss = 0.0;
    if (!hdot(h, sv, sv, s, ss)) return VIBE_C_ERR_DEVICE;
    if (std::sqrt(ss) / f_norm < h->tol) {
      vop_xadd1(x, p, alpha, n, s);
      break;
    }
    vop_mul(prec, sv, hat, n, s);
    hz_apply_ref(h->g, h->a, h->b, hat, t, s);
    double tt = 0.0, ts = 0.0;
    if (!hdot(h, t, t, s, tt)) return VIBE_C_ERR_DEVICE;
    if (tt > 1e-300 && !hdot(h, t, sv, s, ts)) return VIBE_C_ERR_DEVICE;
    omega = (tt > 1e-300) ? ts / tt : 0.0;
    vop_xadd2(x, p, sv, alpha, omega, n, s);
    vop_axpy_to(sv, t, omega, r, n, s);
    rho_prev = rho;
    if (std::fabs(omega) < 1e-300) break;
  }
  iters = it;
  return ok(cudaGetLastError(), "krylov_jacobi") ? VIBE_C_OK : VIBE_C_ERR_DEVICE;
}

// RefinementSolver::solve (helmholtz.cpp:433-462) around the multigrid
// wrapper; the wrapper's coarse solve (restrict f, solve, prolong into x,
// :393-405) is discarded by the inner solver's x = 0 and is not repeated
int krylov_multigrid_refined(vibe_helmholtz* h, const double* f, double* x, cudaStream_t s) {
  int it = 0;
  double res = 1.0;
  int rc = krylov_jacobi(h, f, x, s, it, res);
  if (rc) return rc;
  if (!h->refine) {
    h->iterations = it;
    h->residual = res;
    return VIBE_C_OK;
  }
  const size_t n = cells(h);
  double *r = h->w[8], *dx = h->w[9];
  int total = it;
  for (int pass = 0; pass < 3; ++pass) {
    hz_residual_ref(h->g, h->a, h->b, f, x, r, s);
    double rn = 0.0, fn = 0.0;
    if (!hdot(h, r, r, s, rn) || !hdot(h, f, f, s, fn)) return VIBE_C_ERR_DEVICE;
    const double rel = std::sqrt(rn / dmax(fn, 1e-300));
    res = rel;
    if (rel < h->tol) break;
    rc = krylov_jacobi(h, r, dx, s, it, res);
    if (rc) return rc;
    res = rel;
    vop_add(x, dx, n, s);
    total += it;
  }
  h->iterations = total;
  h->residual = res;
  return VIBE_C_OK;
}

// kinds 3-4: x = 0; repeat r = f - A x (exact FP64 operator), stop when
// ||r|| / ||f|| < tol, else x += MG-BiCGSTAB(r)
int mg_refined(vibe_helmholtz* h, const double* f, double* x, cudaStream_t s) {
  const size_t n = cells(h);
  double *r = h->w[8], *dx = h->w[9];
  cudaMemsetAsync(x, 0, n * sizeof(double), s);
  double fn = 0.0;
  if (!hdot(h, f, f, s, fn)) return VIBE_C_ERR_DEVICE;
  const double fnorm = std::sqrt(fn);
  int total = 0;
  double rel = 0.0;
  const bool fp32 = h->kind == VIBE_HZ_MG_BICGSTAB_MIXED;
  const double rtol = fp32 ? 1e-4 : dmax(0.1 * h->tol, 1e-14);
  for (int pass = 0; pass <= kMaxRefinements; ++pass) {
    hz_residual_ref(h->g, h->a, h->b, f, x, r, s);
    double rn = 0.0;
    if (!hdot(h, r, r, s, rn)) return VIBE_C_ERR_DEVICE;
    rel = (fnorm > 0.0) ? std::sqrt(rn) / fnorm : std::sqrt(rn);
    if (!(rel >= h->tol) || pass == kMaxRefinements) break;  // converged, or NaN
    const int it = fp32 ? mg_solve(h->mg32, r, dx, rtol, h->max_iter, s, rn)
                        : mg_solve(h->mg64, r, dx, rtol, h->max_iter, s, rn);
    if (it == -1 && cudaGetLastError() != cudaSuccess) return VIBE_C_ERR_DEVICE;
    total += it < 0 ? -it : it;
    vop_add(x, dx, n, s);
    if (it == 0) break;
  }
  h->iterations = total;
  h->residual = rel;
  return ok(cudaGetLastError(), "mg solve") ? VIBE_C_OK : VIBE_C_ERR_DEVICE;
}

int solve_dev(vibe_helmholtz* h, const double* f, double* x, cudaStream_t s) {
  if (!h->coef) {
    g_herr = "coefficients not set";
    return VIBE_C_ERR_BAD_ARG;
  }
  switch (h->kind) {
    case VIBE_HZ_VERTICAL_TRIDIAGONAL: {
      cudaMemsetAsync(h->err, 0, sizeof(unsigned), s);
      hz_vertical_solve(h->g, h->a, h->b, f, x, h->w[0], nullptr, h->err, s);
      if (!ok(cudaMemcpyAsync(h->herr, h->err, sizeof(unsigned), cudaMemcpyDeviceToHost, s), "status") ||
          !ok(cudaStreamSynchronize(s), "vertical solve"))
        return VIBE_C_ERR_DEVICE;
      h->iterations = 1;
      h->residual = 0.0;
      if (*h->herr & kErrSingular) {
        g_herr = "singular column";
        return VIBE_C_ERR_SINGULAR;
      }
      return VIBE_C_OK;
    }
    case VIBE_HZ_KRYLOV_JACOBI: {
      int it = 0;
      double res = 1.0;
      const int rc = krylov_jacobi(h, f, x, s, it, res);
      h->iterations = it;
      h->residual = res;
      return rc;
    }
    case VIBE_HZ_KRYLOV_MULTIGRID:
      return krylov_multigrid_refined(h, f, x, s);
    default:
      return mg_refined(h, f, x, s);
  }
}

int set_coef_dev(vibe_helmholtz* h, cudaStream_t s) {
  if (h->mg32 && mg_set_coefficients(h->mg32, h->a, h->b, s)) return VIBE_C_ERR_DEVICE;
  if (h->mg64 && mg_set_coefficients(h->mg64, h->a, h->b, s)) return VIBE_C_ERR_DEVICE;
  h->coef = true;
  return ok(cudaGetLastError(), "set coefficients") ? VIBE_C_OK : VIBE_C_ERR_DEVICE;
}

}  // namespace

extern "C" {

const char* vibe_helmholtz_last_error(void) { return g_herr.c_str(); }

int vibe_helmholtz_create(int kind, int nx, int ny, int nz, double dx, double dy, double z_top, const double* dzeta,
                          const double* zs, int max_iter, double tol, vibe_helmholtz** out) {
  if (!out || kind < 0 || kind > 4 || nx <= 0 || ny <= 0 || nz <= 0 || !dzeta || !(dx > 0.0) || !(dy > 0.0) ||
      max_iter < 1) {
    g_herr = "vibe_helmholtz_create: bad argument";
    return VIBE_C_ERR_BAD_ARG;
  }
  auto* h = new vibe_helmholtz();
  h->kind = kind;
  h->max_iter = max_iter;
  h->tol = tol;
  h->g.nx = nx;
  h->g.ny = ny;
  h->g.nz = nz;
  h->g.dx = dx;
  h->g.dy = dy;
  const size_t n = (size_t)nx * ny * nz, cols = (size_t)nx * ny;
  h->hbuf.resize(n);
  std::vector<double> scale(cols);
  for (size_t c = 0; c < cols; ++c) scale[c] = z_top - (zs ? zs[c] : 0.0);  // Grid::terrain, geometry.cpp:247-253
  bool good = ok(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking), "stream") &&
              ok(cudaMalloc(&h->d_dzeta, nz * sizeof(double)), "alloc") &&
              ok(cudaMalloc(&h->d_scale, cols * sizeof(double)), "alloc") &&
              ok(cudaMalloc(&h->a, n * sizeof(double)), "alloc") && ok(cudaMalloc(&h->b, n * sizeof(double)), "alloc") &&
              ok(cudaMalloc(&h->f, n * sizeof(double)), "alloc") && ok(cudaMalloc(&h->x, n * sizeof(double)), "alloc") &&
              ok(cudaMalloc(&h->part, 2 * kRedBlocks * sizeof(double)), "alloc") &&
              ok(cudaMalloc(&h->scal, 4 * sizeof(double)), "alloc") &&
              ok(cudaMallocHost(&h->hscal, 4 * sizeof(double)), "alloc") &&
              ok(cudaMalloc(&h->err, sizeof(unsigned)), "alloc") &&
              ok(cudaMallocHost(&h->herr, sizeof(unsigned)), "alloc");
  for (int q = 0; q < 10 && good; ++q) good = ok(cudaMalloc(&h->w[q], n * sizeof(double)), "alloc");
  if (good) {
    good = ok(cudaMemcpy(h->d_dzeta, dzeta, nz * sizeof(double), cudaMemcpyHostToDevice), "upload dzeta") &&
           ok(cudaMemcpy(h->d_scale, scale.data(), cols * sizeof(double), cudaMemcpyHostToDevice), "upload terrain");
  }
  h->g.dzeta = h->d_dzeta;
  h->g.scale = h->d_scale;
  if (good && kind == VIBE_HZ_MG_BICGSTAB_MIXED) {
    h->mg32 = mg_create<float>(h->g, kMgLevelsDefault);
    good = h->mg32 != nullptr;
  }
  if (good && kind == VIBE_HZ_MG_BICGSTAB_FP64) {
    h->mg64 = mg_create<double>(h->g, kMgLevelsDefault);
    good = h->mg64 != nullptr;
  }
  if (!good) {
    if (g_herr.empty()) g_herr = "device allocation failed";
    vibe_helmholtz_destroy(h);
    return VIBE_C_ERR_DEVICE;
  }
  *out = h;
  return VIBE_C_OK;
}

void vibe_helmholtz_destroy(vibe_helmholtz* h) {
  if (!h) return;
  if (h->stream) cudaStreamSynchronize(h->stream);
  mg_destroy(h->mg32);
  mg_destroy(h->mg64);
  double* ps[] = {h->d_dzeta, h->d_scale, h->a, h->b, h->f, h->x, h->part, h->scal};
  for (double* p : ps) cudaFree(p);
  for (double* p : h->w) cudaFree(p);
  cudaFree(h->err);
  if (h->hscal) cudaFreeHost(h->hscal);
  if (h->herr) cudaFreeHost(h->herr);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
}

int vibe_helmholtz_set_coefficients(vibe_helmholtz* h, const double* a, const double* b) {
  if (!h || !a || !b) {
    g_herr = "vibe_helmholtz_set_coefficients: NULL argument";
    return VIBE_C_ERR_BAD_ARG;
  }
  if (!upload(h, a, h->a) || !upload(h, b, h->b)) return VIBE_C_ERR_DEVICE;
  const int rc = set_coef_dev(h, h->stream);
  return (rc == VIBE_C_OK && ok(cudaStreamSynchronize(h->stream), "set coefficients")) ? rc : VIBE_C_ERR_DEVICE;
}

int vibe_helmholtz_set_coefficients_dev(vibe_helmholtz* h, const double* a, const double* b, vibe_stream_t stream) {
  if (!h || !a || !b) {
    g_herr = "vibe_helmholtz_set_coefficients_dev: NULL argument";
    return VIBE_C_ERR_BAD_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const size_t n = cells(h) * sizeof(double);
  if (!ok(cudaMemcpyAsync(h->a, a, n, cudaMemcpyDeviceToDevice, s), "copy a") ||
      !ok(cudaMemcpyAsync(h->b, b, n, cudaMemcpyDeviceToDevice, s), "copy b"))
    return VIBE_C_ERR_DEVICE;
  return set_coef_dev(h, s);
}

int vibe_helmholtz_solve(vibe_helmholtz* h, const double* a, const double* b, const double* f, double* x) {
  if (!h || !f || !x || ((a == nullptr) != (b == nullptr))) {
    g_herr = "vibe_helmholtz_solve: bad argument";
    return VIBE_C_ERR_BAD_ARG;
  }
  if (a) {
    const int rc = vibe_helmholtz_set_coefficients(h, a, b);
    if (rc) return rc;
  }
  if (!upload(h, f, h->f)) return VIBE_C_ERR_DEVICE;
  const int rc = solve_dev(h, h->f, h->x, h->stream);
  if (rc != VIBE_C_OK && rc != VIBE_C_ERR_SINGULAR) return rc;
  if (!download(h, h->x, x)) return VIBE_C_ERR_DEVICE;
  return rc;
}

int vibe_helmholtz_solve_dev(vibe_helmholtz* h, const double* f, double* x, vibe_stream_t stream) {
  if (!h || !f || !x) {
    g_herr = "vibe_helmholtz_solve_dev: NULL argument";
    return VIBE_C_ERR_BAD_ARG;
  }
  return solve_dev(h, f, x, (cudaStream_t)stream);
}

int vibe_helmholtz_apply_dev(vibe_helmholtz* h, const double* x, double* y, vibe_stream_t stream) {
  if (!h || !x || !y || !h->coef) {
    g_herr = "vibe_helmholtz_apply_dev: bad argument or coefficients not set";
    return VIBE_C_ERR_BAD_ARG;
  }
  hz_apply_ref(h->g, h->a, h->b, x, y, (cudaStream_t)stream);
  return ok(cudaGetLastError(), "apply") ? VIBE_C_OK : VIBE_C_ERR_DEVICE;
}

int vibe_helmholtz_iterations(const vibe_helmholtz* h) { return h ? h->iterations : 0; }
double vibe_helmholtz_residual(const vibe_helmholtz* h) { return h ? h->residual : 0.0; }
const char* vibe_helmholtz_name(const vibe_helmholtz* h) {
  static const char* names[] = {"vertical_tridiagonal", "refinement", "krylov_jacobi", "mg_bicgstab_fp64",
                                "mg_bicgstab_mixed"};
  return h ? names[h->kind] : "";
}
int vibe_helmholtz_set_iterative_refinement(vibe_helmholtz* h, int on, int precision) {
  (void)precision;
  if (!h) return VIBE_C_ERR_BAD_ARG;
  h->refine = on != 0;
  return VIBE_C_OK;
}
int vibe_helmholtz_levels(const vibe_helmholtz* h) {
  if (!h) return 0;
  if (h->mg32) return mg_levels(h->mg32);
  if (h->mg64) return mg_levels(h->mg64);
  return 0;
}

double vibe_helmholtz_residual_l2(vibe_helmholtz* h, const double* f, const double* x) {
  if (!h || !f || !x || !h->coef) return 0.0;
  if (!upload(h, f, h->f) || !upload(h, x, h->x)) return 0.0;
  double* r = h->w[8];
  hz_residual_ref(h->g, h->a, h->b, h->f, h->x, r, h->stream);
  double rr = 0.0;
  if (!hdot(h, r, r, h->stream, rr)) return 0.0;
  return std::sqrt(rr);
}

}  // extern "C"
