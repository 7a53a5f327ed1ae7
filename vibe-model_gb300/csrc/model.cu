// vibe-model_gb300/csrc/model.cu
//
// Host side of the GB300 dynamics step: case set-up (grid metrics,
// reference state, initial state -- computed once on the host with the
// reference's formulas), device buffers, the per-step kernel schedule for
// both precisions, and the C ABI declared in include/vibe_gb300.h.
// Nothing here computes the step on the CPU: every state update is a kernel.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "step_kernels.cuh"
#include "vibe_gb300.h"
#include "vibe_helmholtz.h"
#include "vibe_nest.h"
#include "vibe_tlad.h"
#include "tlad_internal.cuh"
#include <array>

using namespace vgb;

namespace {
thread_local std::string g_err;
int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}
#define CUDA_OK(call)                                                                          \
  do {                                                                                         \
    cudaError_t e_ = (call);                                                                   \
    if (e_ != cudaSuccess) return fail(VIBE_GB300_EDEVICE, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

constexpr int H = 4;  // halo width of the reference's FieldT (driver.cpp:157-159)

struct HostSetup {
  std::vector<double> zeta, zs, sponge;
  std::vector<double> ref[5];  // FieldT storage of theta0, pi0, rho0, p0, qv0
  std::vector<double> st[NSPECIES];
};
}  // namespace

// FP64 launchers of one build variant (FMA-contracted or bit-exact)
struct Fp64Ops {
  decltype(&fp64_slow_tendency) slow_tendency;
  decltype(&fp64_stage_update) stage_update;
  decltype(&fp64_fb_substep) fb_substep;
  decltype(&fp64_ref_hevi_substep) ref_hevi_substep;
  decltype(&fp64_cons_hevi_substep) cons_hevi_substep;
  decltype(&fp64_sponge) sponge;
  decltype(&fp64_nonfinite) nonfinite;
  decltype(&fp64_fb_substep_ad) fb_substep_ad;
  decltype(&fp64_hevi_substep_ad) hevi_substep_ad;
};
static const Fp64Ops kFp64Fast = {fp64_slow_tendency, fp64_stage_update, fp64_fb_substep, fp64_ref_hevi_substep,
                                  fp64_cons_hevi_substep, fp64_sponge, fp64_nonfinite, fp64_fb_substep_ad,
                                  fp64_hevi_substep_ad};
static const Fp64Ops kFp64Exact = {fp64_slow_tendency_exact, fp64_stage_update_exact, fp64_fb_substep_exact,
                                   fp64_ref_hevi_substep_exact, fp64_cons_hevi_substep_exact, fp64_sponge_exact,
                                   fp64_nonfinite_exact, fp64_fb_substep_ad_exact, fp64_hevi_substep_ad_exact};

struct vibe_gb300_model {
  vibe_gb300_setup su{};
  const Fp64Ops* f64 = &kFp64Fast;
  int precision = 0;
  Dims d{};
  Metric met{};
  Flags fl{};
  Tab tab{};
  cudaStream_t stream = nullptr;
  HostSetup hs;
  int nsx[NSPECIES], nsy[NSPECIES], nsz[NSPECIES];
  bool uniform = true;
  // device memory (one allocation per buffer)
  std::vector<void*> allocs;
  double* S[2][NSPECIES] = {};
  int cur = 0;
  double* tend[NSPECIES] = {};
  double* tmp[NSPECIES] = {};
  double* lin[5] = {};  // u, v, w, rho, pi perturbations of the acoustic TL/AD (allocated on first use)
  float* lin32[2][5] = {};         // FP32 acoustic TL/AD (mixed models): ping-pong perturbations
  float* lin32_dh = nullptr;       // FP32 HEVI AD: bar of the horizontal divergence
  float* lin32_scr = nullptr;      // FP32 HEVI AD: per-column work
  double* lin_tmp[3] = {};         // HEVI TL: the column solve's w, rho, pi outputs
  double* lin_scr = nullptr;       // HEVI TL/AD: per-column work
  double* lin_dh = nullptr;        // HEVI AD: bar of the horizontal divergence
  // TL/AD of the model's own step (allocated on first use): six perturbation
  // states of 12 fields, the WENO face fluxes (9 fields), one cell field and
  // a zero field (the reference of the sponge's linear part)
  double* stl[6][NSPECIES] = {};
  double* stl_face = nullptr;
  double* stl_cell = nullptr;
  double* stl_zero = nullptr;
  // while set, a step copies its second and third stages' input states here
  double* const* rec_stage[2] = {nullptr, nullptr};
  // physics package (vibe_gb300_set_physics) and its tendency accumulators
  vibe_gb300_physics_fn phys_fn = nullptr;
  void* phys_user = nullptr;
  unsigned phys_written = 0;  // accumulators the package wrote in its last call (they need zeroing)
  void* pt[NSPECIES] = {};  // u, v, theta, qv..qg: double (FP64) or float (mixed)
  double* d_zmid = nullptr;
  double* d_zs = nullptr;
  double* scratch = nullptr;
  double* wface = nullptr;  // FP64 path: WENO face fluxes of one scalar
  double *d_dzeta = nullptr, *d_scale = nullptr, *d_sponge = nullptr;
  double *d_th0 = nullptr, *d_pi0 = nullptr, *d_rho0 = nullptr;
  double* d_stage_in = nullptr;   // staging for FieldT <-> device layout
  double* d_tri = nullptr;        // reference HEVI coefficients (3*nz)
  float* W0[NSPECIES] = {};
  float* WSt[2][NSPECIES] = {};
  float* WA[NSPECIES] = {};
  float* WB[NSPECIES] = {};
  float* WR[NSPECIES] = {};       // last stage's FP32 tendency
  float* d_ftab = nullptr;        // FP32 tables
  double* d_dtab = nullptr;       // FP64 tables
  float* d_lu = nullptr;          // 3 stages x 3*nz
  double* d_spid = nullptr;       // identity sponge tables (nz+1 weights, nz+1 zeros)
  float* d_spif = nullptr;
  unsigned* d_err = nullptr;
  unsigned* h_err = nullptr;      // pinned
  double* h_pin = nullptr;        // pinned staging
  size_t pin_n = 0;
  double cfg_dt = -1.0;
  int cfg_nsub = -1;
  int kmin = 0;
  std::vector<float> ftab_host;
  std::vector<double> dtab_host;
  // optional per-kernel-class timing with CUDA events on the model stream
  bool timing = false;
  static constexpr int kClasses = 4;  // 0 stage, 1 substep (all kernels), 2 finish/sponge, 3 other
  std::vector<cudaEvent_t> ev_pool;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> ev_open;
  double class_ms[kClasses] = {};
  long class_n[kClasses] = {};
  // semi-implicit step: Helmholtz solver and its problem (nx*ny*nz each)
  vibe_helmholtz* hz = nullptr;
  int hz_kind = -1, hz_max_iter = 0;
  double hz_tol = 0.0;
  double *hz_a = nullptr, *hz_b = nullptr, *hz_f = nullptr, *hz_x = nullptr;
  int hz_iterations = 0;
  double hz_residual = 0.0;
  double hz_ms = 0.0;
  double cfl_rate = 0.0;  // max over cells of 1/dx + 1/dy + 1/dz
  cudaEvent_t hz_ev[2] = {nullptr, nullptr};
  // CUDA graphs of one mixed step, per state parity
  bool use_graph = true, graph_warm = false;
  cudaGraphExec_t gexec[2] = {nullptr, nullptr};
  double graph_dt = -1.0;
  int graph_nsub = -1;
  // device copy of the prognostic state (vibe_gb300_snapshot), made on first save
  double* snap[NSPECIES] = {};
  bool has_snap = false;
  // pipelined host I/O (vibe_gb300_step_io): copy streams, double-buffered
  // FieldT staging on the device, events ordering the three streams
  struct IoPipe {
    cudaStream_t sin = nullptr, sout = nullptr;
    double* in[2][NSPECIES] = {};
    double* out[2][NSPECIES] = {};
    cudaEvent_t start = nullptr, in_done[2] = {}, packed[2] = {}, unpacked[2] = {}, out_done[2] = {};
    long n = 0;
    bool idle = true;  // no call since the last join: the next uploads start after the model's stream
  };
  IoPipe* io = nullptr;
};

namespace {
void io_release(vibe_gb300_model* m);
}  // namespace

namespace {

size_t storage_count(const vibe_gb300_model* m, int q) {
  return (size_t)m->nsx[q] * m->nsy[q] * m->nsz[q];
}
__host__ __device__ inline size_t soff(int nsx, int nsy, int i, int j, int k) {
  return ((size_t)(k + H) * nsy + (size_t)(j + H)) * nsx + (size_t)(i + H);
}

// ---- host set-up, same formulas as the reference --------------------------

// make_stretched_zeta, src/grid/geometry.cpp:39-60
void make_zeta(int nz, double first, double stretch, std::vector<double>& zeta) {
  std::vector<double> dz(nz);
  double total = 0.0, h = first, acc = 0.0;
  for (int k = 0; k < nz; ++k) { dz[k] = h; total += h; h *= stretch; }
  zeta.assign(nz + 1, 0.0);
  for (int k = 0; k < nz; ++k) { acc += dz[k]; zeta[k + 1] = acc / total; }
  zeta[nz] = 1.0;
}

struct Geo {
  const vibe_gb300_setup* s;
  const std::vector<double>* zeta;
  const std::vector<double>* zs;
  double terrain(int i, int j) const {  // geometry.cpp:247-253
    return (*zs)[(size_t)iclamp(j, 0, s->ny - 1) * s->nx + iclamp(i, 0, s->nx - 1)];
  }
  double zeta_at(double kk) const {  // geometry.cpp:20-31
    const int nz = s->nz;
    if (kk <= 0.0) return (*zeta)[0];
    if (kk >= (double)nz) return (*zeta)[nz];
    const int k0 = (int)std::floor(kk);
    const double frac = kk - (double)k0;
    if (frac == 0.0) return (*zeta)[k0];
    if (std::fabs(frac - 0.5) < 1e-12) return 0.5 * ((*zeta)[k0] + (*zeta)[k0 + 1]);
    return (*zeta)[k0] + frac * ((*zeta)[k0 + 1] - (*zeta)[k0]);
  }
  double height(int i, int j, double kk) const {  // geometry.cpp:260-263
    const double z0 = terrain(i, j);
    return z0 + zeta_at(kk) * (s->z_top - z0);
  }
  double zc(int i, int j, int k) const { return height(i, j, (double)k + 0.5); }
};

double density_from(double pi0, double th0) { return kP0 * std::pow(pi0, kCv / kRd) / (kRd * th0); }  // reference_state.cpp:26-28
double pressure_from(double pi0) { return kP0 * std::pow(pi0, kCp / kRd); }                            // :31

void host_setup(vibe_gb300_model* m) {
  const vibe_gb300_setup& s = m->su;
  const int nx = s.nx, ny = s.ny, nz = s.nz;
  HostSetup& hs = m->hs;
  make_zeta(nz, s.zeta_first, s.zeta_stretch, hs.zeta);
  hs.zs.assign((size_t)nx * ny, 0.0);
  if (s.terrain_kind == 1)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const double x = ((double)i + 0.5) * s.dx - s.hill_xc;
        const double y = ((double)j + 0.5) * s.dy - s.hill_yc;
        hs.zs[(size_t)j * nx + i] = s.hill_h * std::exp(-(x * x + y * y) / (s.hill_a * s.hill_a));
      }
  Geo g{&s, &hs.zeta, &hs.zs};
  const int cx = m->nsx[RHO], cy = m->nsy[RHO];
  for (auto& r : hs.ref) r.assign(storage_count(m, RHO), 0.0);
  auto R = [&](int w, int i, int j, int k) -> double& { return hs.ref[w][soff(cx, cy, i, j, k)]; };
  const double pi_surf = std::pow(s.p_surf / kP0, kRd / kCp);
  if (s.ref_kind == 1) {  // ReferenceState::from_profile, reference_state.cpp:61-110
    const int np = (int)std::ceil(s.z_top / s.profile_dz) + 2;
    std::vector<double> z(np), th(np), zi(nz + 1);
    for (int p = 0; p < np; ++p) {
      z[p] = (double)p * s.profile_dz;
      th[p] = s.theta0 * std::exp(s.bv_n * s.bv_n * z[p] / kG);
    }
    auto theta_at = [&](double zz) {
      if (zz <= z.front()) return th.front();
      if (zz >= z.back()) return th.back();
      size_t k = 0;
      while (k + 2 < z.size() && z[k + 1] < zz) ++k;
      const double w = (z[k + 1] - z[k] > 0.0) ? (zz - z[k]) / (z[k + 1] - z[k]) : 0.0;
      return th[k] + w * (th[k + 1] - th[k]);
    };
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        for (int k = 0; k <= nz; ++k) zi[k] = g.height(i, j, (double)k);
        double pi = pi_surf;
        R(0, i, j, 0) = theta_at(zi[0]);
        for (int k = 0; k < nz; ++k) {
          const double th_lo = theta_at(zi[k]), th_hi = theta_at(zi[k + 1]);
          const double th_mid = 0.5 * (th_lo + th_hi);
          const double dz = zi[k + 1] - zi[k];
          pi -= kG * dz / (kCp * th_mid);
          const double th_c = 0.5 * (th_lo + th_hi);
          R(0, i, j, k) = th_c;
          R(1, i, j, k) = pi;
          R(3, i, j, k) = pressure_from(pi);
          R(2, i, j, k) = density_from(pi, th_c);
          R(4, i, j, k) = 0.0;
        }
      }
  } else {  // ReferenceState::isothermal, reference_state.cpp:35-59
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
          const double z = g.zc(i, j, k);
          const double pi = pi_surf - kG * z / (kCp * s.theta0);
          R(0, i, j, k) = s.theta0;
          R(1, i, j, k) = pi;
          R(3, i, j, k) = pressure_from(pi);
          R(2, i, j, k) = density_from(pi, s.theta0);
          R(4, i, j, k) = 0.0;
        }
  }
  // Damping constructor sponge profile, damping.cpp:24-41
  hs.sponge.assign(nz, 0.0);
  {
    const double zs0 = s.sponge_start_fraction * s.z_top;
    for (int k = 0; k < nz; ++k) {
      const double z = g.zc(0, 0, k);
      if (z <= zs0) continue;
      const double t = (z - zs0) / dmax(s.z_top - zs0, 1.0);
      const double sn = std::sin(0.5 * kPi * (t < 0.0 ? 0.0 : (t > 1.0 ? 1.0 : t)));
      hs.sponge[k] = s.sponge_alpha * sn * sn;
    }
  }
  // init_warm_bubble, initial_conditions.cpp:136-159 (fill_base_state :66-91,
  // apply_shear :94-102, enforce_state_equation :110-121)
  for (int q = 0; q < NSPECIES; ++q) hs.st[q].assign(storage_count(m, q), 0.0);
  auto S = [&](int q, int i, int j, int k) -> double& { return hs.st[q][soff(m->nsx[q], m->nsy[q], i, j, k)]; };
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const double z = g.zc(i, j, k);
        S(THETA, i, j, k) = R(0, i, j, k);
        S(PI, i, j, k) = R(1, i, j, k);
        S(RHO, i, j, k) = R(2, i, j, k);
        S(QV, i, j, k) = s.qv_surface * std::exp(-dmax(z, 0.0) / s.qv_decay_height);
      }
  const double xc = (s.bubble_xc != 0.0) ? s.bubble_xc : 0.5 * 0.0 + 0.5 * (double)nx * s.dx;
  const double yc = (s.bubble_yc != 0.0) ? s.bubble_yc : 0.5 * (double)ny * s.dy;
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const double x = (0 + (double)i + 0.5) * s.dx, y = (0 + (double)j + 0.5) * s.dy;
        const double z = g.zc(i, j, k);
        const double ax = (x - xc) / s.bubble_radius_x, ay = (y - yc) / s.bubble_radius_x,
                     az = (z - s.bubble_zc) / s.bubble_radius_z;
        const double r2 = ax * ax + ay * ay + az * az;
        if (r2 < 1.0) {
          const double c = std::cos(0.5 * kPi * std::sqrt(r2));
          S(THETA, i, j, k) += s.bubble_amplitude * c * c;
        }
      }
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i <= nx; ++i) S(U, i, j, k) = s.u_background + s.shear_u * g.zc(imin(i, nx - 1), j, k);
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const double qv = dmax(S(QV, i, j, k), 0.0);
        const double gamma_f = (1.0 + qv / kEpsVap) / (1.0 + qv);
        const double val = S(RHO, i, j, k) * kRd * S(THETA, i, j, k) * gamma_f / kP0;
        if (val > 0.0) S(PI, i, j, k) = std::pow(val, kRd / kCv);
      }
}

// ---- device buffers -------------------------------------------------------
template <class T>
int dalloc(vibe_gb300_model* m, T** p, size_t n) {
  void* v = nullptr;
  CUDA_OK(cudaMalloc(&v, n * sizeof(T) + 256));
  CUDA_OK(cudaMemsetAsync(v, 0, n * sizeof(T) + 256, m->stream));
  m->allocs.push_back(v);
  *p = (T*)v;
  return 0;
}

// FieldT storage <-> device layout
__global__ void k_pack(Dims d, int nsx, int nsy, int ni, int nj, int nk, const double* __restrict__ src,
                       double* __restrict__ dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
  if (i >= ni || j >= nj || k >= nk) return;
  dst[d.idx(i, j, k)] = src[soff(nsx, nsy, i, j, k)];
}
// device layout (FP64 or FP32) -> FP64 FieldT storage, zeros outside the
// box i < ni, j < nj, k < nk: one thread per storage point of a 3-D grid
// (no index divisions), coalesced along i on both sides
template <class T>
__global__ void k_unpack_t(Dims d, int nsx, int nsy, int ni, int nj, int nk, const T* __restrict__ src,
                           double* __restrict__ dst) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y, z = blockIdx.z;
  if (x >= nsx || y >= nsy) return;
  const int ii = x - H, jj = y - H, kk = z - H;
  double v = 0.0;
  if (ii >= 0 && ii < ni && jj >= 0 && jj < nj && kk >= 0 && kk < nk) v = (double)src[d.idx(ii, jj, kk)];
  dst[((size_t)z * nsy + y) * nsx + x] = v;
}
template <class T>
void unpack(const Dims& d, int nsx, int nsy, int nsz, int ni, int nj, int nk, const T* src, double* dst,
            cudaStream_t s) {
  k_unpack_t<T><<<dim3((nsx + 31) / 32, (nsy + 7) / 8, nsz), dim3(32, 8), 0, s>>>(d, nsx, nsy, ni, nj, nk, src, dst);
}

// rigid ground and lid (w_rigid): w = 0 on the k = 0 and k = nz faces
__global__ void k_rigid_w(Dims d, double* __restrict__ w) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= d.nx || j >= d.ny) return;
  w[d.idx(i, j, 0)] = 0.0;
  w[d.idx(i, j, d.nz)] = 0.0;
}

// zero every point of a field outside the box i < ni, j < nj, k < nk
__global__ void k_keep_box(Dims d, int ni, int nj, int nk, double* __restrict__ f) {
  const size_t n = d.plane * (size_t)(d.nz + 1);
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(e / d.plane);
    const size_t r = e - (size_t)k * d.plane;
    const int j = (int)(r / d.P), i = (int)(r - (size_t)j * d.P);
    if (i >= ni || j >= nj || k >= nk) f[e] = 0.0;
  }
}

void box_of(const vibe_gb300_model* m, int q, int& ni, int& nj, int& nk) {
  ni = m->d.nx + 1;
  nj = m->d.ny + 1;
  nk = m->d.nz + (q == W);
}

int upload_storage(vibe_gb300_model* m, int q, const double* host, double* const* dsts, int ndst) {
  const size_t n = storage_count(m, q);
  CUDA_OK(cudaMemcpyAsync(m->d_stage_in, host, n * sizeof(double), cudaMemcpyHostToDevice, m->stream));
  int ni, nj, nk;
  box_of(m, q, ni, nj, nk);
  const dim3 b(32, 4);
  for (int t = 0; t < ndst; ++t)
    k_pack<<<dim3((ni + 31) / 32, (nj + 3) / 4, nk), b, 0, m->stream>>>(m->d, m->nsx[q], m->nsy[q], ni, nj, nk,
                                                                         m->d_stage_in, dsts[t]);
  CUDA_OK(cudaGetLastError());
  return 0;
}

// ---- FP32 tables of the mixed path / stage coefficients ---------------------
int build_tables(vibe_gb300_model* m) {
  const int nz = m->d.nz;
  const auto& hs = m->hs;
  const int cx = m->nsx[RHO], cy = m->nsy[RHO];
  auto R = [&](int w, int k) { return hs.ref[w][soff(cx, cy, 0, 0, k)]; };
  std::vector<double> r0(nz), t0(nz), p0(nz);
  for (int k = 0; k < nz; ++k) { t0[k] = R(0, k); p0[k] = R(1, k); r0[k] = R(2, k); }
  const double zt = m->su.z_top;
  auto dzeta = [&](int k) { const int kk = iclamp(k, 0, nz - 1); return hs.zeta[kk + 1] - hs.zeta[kk]; };
  std::vector<float>& f = m->ftab_host;
  f.assign((size_t)20 * (nz + 1) + 6 * (size_t)nz + 64, 0.f);
  size_t o = 0;
  auto put = [&](const float** dst, size_t n) { size_t at = o; o += n; return at; };
  size_t o_r0c = put(nullptr, nz), o_rfz = put(nullptr, nz + 1), o_t0c = put(nullptr, nz), o_tfz = put(nullptr, nz + 1);
  size_t o_kap = put(nullptr, nz), o_idzc = put(nullptr, nz), o_idzw = put(nullptr, nz + 1), o_idza = put(nullptr, nz);
  size_t o_thi = put(nullptr, nz), o_t0d = put(nullptr, 6 * (size_t)nz), o_spw = put(nullptr, nz + 1);
  for (int k = 0; k < nz; ++k) {
    f[o_r0c + k] = (float)r0[k];
    f[o_t0c + k] = (float)t0[k];
    f[o_kap + k] = (float)((kRd / kCv) * (p0[k] / dmax(r0[k], 1e-8)));
    f[o_idzc + k] = (float)(1.0 / dmax(dzeta(k) * zt, 1.0));
    f[o_idza + k] = (float)(1.0 / (dzeta(k) * zt));
    f[o_thi + k] = (float)(1.0 / dmax(t0[k], 1.0));
    for (int mm = -3; mm <= 2; ++mm) f[o_t0d + 6 * (size_t)k + (mm + 3)] = (float)(t0[iclamp(k + mm, 0, nz - 1)] - t0[k]);
  }
  for (int k = 0; k <= nz; ++k) {
    const int kc = imin(k, nz - 1), km = imax(k - 1, 0);
    f[o_rfz + k] = (float)(0.5 * (r0[km] + r0[kc]));
    f[o_tfz + k] = (float)(0.5 * (t0[km] + t0[kc]));
    f[o_idzw + k] = (float)(1.0 / dmax(dzeta(kc) * zt, 1.0));
    f[o_spw + k] = 1.f;
  }
  const size_t nft = o;
  if (dalloc(m, &m->d_ftab, nft)) return VIBE_GB300_EDEVICE;
  CUDA_OK(cudaMemcpy(m->d_ftab, f.data(), nft * sizeof(float), cudaMemcpyHostToDevice));
  Tab& t = m->tab;
  t.r0c = m->d_ftab + o_r0c; t.rfz = m->d_ftab + o_rfz; t.t0c = m->d_ftab + o_t0c; t.tfz = m->d_ftab + o_tfz;
  t.kap = m->d_ftab + o_kap; t.idzc = m->d_ftab + o_idzc; t.idzw = m->d_ftab + o_idzw; t.idza = m->d_ftab + o_idza;
  t.th0inv = m->d_ftab + o_thi; t.t0d = m->d_ftab + o_t0d; t.spw = m->d_ftab + o_spw;
  // FP64: spwd(nz+1), spdt(nz+1), r0, t0, p0 (nz each)
  std::vector<double>& dt = m->dtab_host;
  dt.assign(2 * (size_t)(nz + 1) + 3 * (size_t)nz, 0.0);
  for (int k = 0; k <= nz; ++k) dt[k] = 1.0;
  for (int k = 0; k < nz; ++k) {
    dt[2 * (nz + 1) + k] = r0[k];
    dt[2 * (nz + 1) + nz + k] = t0[k];
    dt[2 * (nz + 1) + 2 * nz + k] = p0[k];
  }
  if (dalloc(m, &m->d_dtab, dt.size())) return VIBE_GB300_EDEVICE;
  CUDA_OK(cudaMemcpy(m->d_dtab, dt.data(), dt.size() * sizeof(double), cudaMemcpyHostToDevice));
  t.spwd = m->d_dtab;
  t.spdt = m->d_dtab + (nz + 1);
  t.r0d = m->d_dtab + 2 * (nz + 1);
  t.t0dd = t.r0d + nz;
  t.p0d = t.r0d + 2 * nz;
  t.dx_inv = (float)(1.0 / m->su.dx);
  t.dy_inv = (float)(1.0 / m->su.dy);
  t.f0 = (float)m->met.f0;
  t.beta = (float)m->met.beta;
  t.dy = (float)m->su.dy;
  // identity sponge tables for single substep folds
  std::vector<double> idt(2 * (size_t)(nz + 1), 0.0);
  for (int k = 0; k <= nz; ++k) idt[k] = 1.0;
  if (dalloc(m, &m->d_spid, idt.size())) return VIBE_GB300_EDEVICE;
  CUDA_OK(cudaMemcpy(m->d_spid, idt.data(), idt.size() * sizeof(double), cudaMemcpyHostToDevice));
  std::vector<float> idf(nz + 1, 1.f);
  if (dalloc(m, &m->d_spif, idf.size())) return VIBE_GB300_EDEVICE;
  CUDA_OK(cudaMemcpy(m->d_spif, idf.data(), idf.size() * sizeof(float), cudaMemcpyHostToDevice));
  return 0;
}

// dt/n_sub dependent coefficients: sponge weights (damping.cpp:94,98), the
// LU factors of the consistent HEVI matrix for the three stage substep
// lengths, and the reference HEVI coefficients are built per call.
int configure_dt(vibe_gb300_model* m, double dt, int n_sub) {
  if (dt == m->cfg_dt && n_sub == m->cfg_nsub) return 0;
  const int nz = m->d.nz;
  const auto& sp = m->hs.sponge;
  std::vector<double>& d = m->dtab_host;
  std::vector<float>& f = m->ftab_host;
  const size_t o_spw = (size_t)nz + (nz + 1) + nz + (nz + 1) + nz + nz + (nz + 1) + nz + nz + 6 * (size_t)nz;
  if (m->uniform) {  // per-level sponge tables of the mixed path
    for (int k = 0; k <= nz; ++k) {
      const double a = sp[imin(k, nz - 1)];
      const double w = (a > 0.0) ? 1.0 / (1.0 + dt * a) : 1.0;
      d[k] = w;
      d[nz + 1 + k] = (a > 0.0) ? dt * a : 0.0;
      f[o_spw + k] = (float)w;
    }
    CUDA_OK(cudaMemcpyAsync(m->d_dtab, d.data(), 2 * (size_t)(nz + 1) * sizeof(double), cudaMemcpyHostToDevice,
                            m->stream));
    CUDA_OK(cudaMemcpyAsync(m->d_ftab + o_spw, f.data() + o_spw, (nz + 1) * sizeof(float), cudaMemcpyHostToDevice,
                            m->stream));
    CUDA_OK(cudaStreamSynchronize(m->stream));
  }
  m->kmin = nz + 1;
  for (int k = 0; k < nz; ++k)
    if (sp[k] > 0.0) { m->kmin = k; break; }
  if (m->precision == VIBE_GB300_MIXED) {
    // consistent HEVI matrix (uniform column): a_k = -c_k T_k,
    // c_k = -c_k T_{k+1}, b_k = 1 + c_k (T_k + T_{k+1}) with
    // c_k = (dtau*beta)^2 kappa_k / dz_k, T_f = rho0_f cp theta0_f / dzf_f
    const auto& hs = m->hs;
    const int cx = m->nsx[RHO], cy = m->nsy[RHO];
    auto R = [&](int w, int k) { return hs.ref[w][soff(cx, cy, 0, 0, k)]; };
    auto dzeta = [&](int k) { const int kk = iclamp(k, 0, nz - 1); return hs.zeta[kk + 1] - hs.zeta[kk]; };
    const double zt = m->su.z_top, b = m->su.hevi_beta;
    std::vector<double> T(nz + 1, 0.0);
    for (int k = 1; k < nz; ++k) {
      const double rf = 0.5 * (R(2, k - 1) + R(2, k)), tf = 0.5 * (R(0, k - 1) + R(0, k));
      T[k] = rf * kCp * tf / dmax(dzeta(k) * zt, 1.0);
    }
    std::vector<float> lu(9 * (size_t)nz, 0.f);
    const double dts[3] = {dt / 3.0, dt / 2.0, dt};
    for (int s = 0; s < 3; ++s) {
      const double dtau = dts[s] / (double)(n_sub > 1 ? n_sub : 1);
      double cprev = 0.0;
      for (int k = 0; k < nz; ++k) {
        const double kap = (kRd / kCv) * (R(1, k) / dmax(R(2, k), 1e-8));
        const double ck = (dtau * b) * (dtau * b) * kap / dmax(dzeta(k) * zt, 1.0);
        const double a = -ck * T[k], c = -ck * T[k + 1], bb = 1.0 + ck * (T[k] + T[k + 1]);
        const double den = (k == 0) ? bb : bb - a * cprev;
        cprev = (k < nz - 1) ? c / den : 0.0;
        lu[s * 3 * (size_t)nz + k] = (float)a;
        lu[s * 3 * (size_t)nz + nz + k] = (float)cprev;
        lu[s * 3 * (size_t)nz + 2 * nz + k] = (float)(1.0 / den);
      }
    }
    CUDA_OK(cudaMemcpyAsync(m->d_lu, lu.data(), lu.size() * sizeof(float), cudaMemcpyHostToDevice, m->stream));
    CUDA_OK(cudaStreamSynchronize(m->stream));
  }
  m->cfg_dt = dt;
  m->cfg_nsub = n_sub;
  return 0;
}

// reference HEVI coefficients from column (0,0), acoustic_substep.cpp:38-65
int ref_hevi_coefficients(vibe_gb300_model* m, double dtau) {
  const int nz = m->d.nz;
  const auto& hs = m->hs;
  const int cx = m->nsx[RHO], cy = m->nsy[RHO];
  auto R = [&](int w, int k) { return hs.ref[w][soff(cx, cy, 0, 0, k)]; };
  std::vector<double> tri(3 * (size_t)nz, 0.0);
  double* ta = tri.data();
  double* tb = ta + nz;
  double* tc = tb + nz;
  const double half = 0.5 * dtau;
  for (int k = 0; k < nz; ++k) {
    const double scale = m->su.z_top - hs.zs[0];
    const double dz = dmax((hs.zeta[k + 1] - hs.zeta[k]) * scale, 1.0);
    const double rho0 = R(2, k), th0 = R(0, k);
    const double cs2 = (kCp / kCv) * kRd * R(0, k) * R(1, k);
    const double a_k = half * half * kCp * th0 * rho0 / (dz * dz);
    const double a_kp1 = (k < nz - 1) ? half * half * kCp * R(0, k + 1) * R(2, k + 1) / (dz * dz) : a_k;
    const double b0 = 1.0 / dmax(rho0 * cs2, 1e-12);
    tb[k] = b0 + a_k + a_kp1;
    if (k < nz - 1) tc[k] = -a_kp1;
    if (k > 0) ta[k - 1] = -a_k;
  }
  CUDA_OK(cudaMemcpyAsync(m->d_tri, tri.data(), tri.size() * sizeof(double), cudaMemcpyHostToDevice, m->stream));
  CUDA_OK(cudaStreamSynchronize(m->stream));
  return 0;
}

WS ws_of(float* const* a) {
  WS w;
  for (int q = 0; q < NSPECIES; ++q) w.f[q] = a[q];
  return w;
}
// the fields the acoustic substeps update (u, v, w, rho, pi); theta sits
// between rho and pi in the species order, so a range test would be wrong
inline bool acoustic_field(int q) { return q == U || q == V || q == W || q == RHO || q == PI; }
// acoustic fields from `sub`, the rest from `stage`
WS ws_compose(float* const* sub, float* const* stage) {
  WS w;
  for (int q = 0; q < NSPECIES; ++q) w.f[q] = acoustic_field(q) ? sub[q] : stage[q];
  return w;
}

cudaEvent_t take_event(vibe_gb300_model* m) {
  cudaEvent_t e;
  if (!m->ev_pool.empty()) {
    e = m->ev_pool.back();
    m->ev_pool.pop_back();
  } else {
    cudaEventCreate(&e);
  }
  return e;
}
struct Span {  // brackets the launches of one kernel class with two events
  vibe_gb300_model* m;
  int cls;
  cudaEvent_t a = nullptr;
  Span(vibe_gb300_model* mm, int c) : m(mm), cls(c) {
    if (!m->timing) return;
    a = take_event(m);
    cudaEventRecord(a, m->stream);
  }
  ~Span() {
    if (!a) return;
    cudaEvent_t b = take_event(m);
    cudaEventRecord(b, m->stream);
    m->ev_open.push_back({cls, {a, b}});
  }
};
void collect_timing(vibe_gb300_model* m) {  // after a stream sync
  for (auto& o : m->ev_open) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, o.second.first, o.second.second);
    m->class_ms[o.first] += ms;
    m->class_n[o.first] += 1;
    m->ev_pool.push_back(o.second.first);
    m->ev_pool.push_back(o.second.second);
  }
  m->ev_open.clear();
}

// ---- physics coupling (runge_kutta.cpp:46-63) -------------------------------
constexpr int kPhysFields[9] = {U, V, THETA, QV, QC, QR, QI, QS, QG};

// d += pt over whole buffers (FP64 path): State's add_scaled(1, pt) per field
__global__ void k_add_pt64(size_t n, const double* __restrict__ pt, double* __restrict__ d) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x)
    d[e] = d[e] + pt[e];
}
// mixed path: the stage kernel has written s = s0 + dt_s R; add dt_s pt, and
// pt to the stage-3 tendency R the finish kernel folds into the FP64 state
__global__ void k_add_pt32(size_t n, const float* __restrict__ pt, float* __restrict__ s, float dts,
                           float* __restrict__ r) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const float p = pt[e];
    s[e] = s[e] + dts * p;
    if (r) r[e] = r[e] + p;
  }
}

// zero the accumulators and let the package enqueue its work for this stage
int physics_stage(vibe_gb300_model* m, int stage, double dt, const void* const* state) {
  const bool mixed = m->precision == VIBE_GB300_MIXED;
  const size_t n = m->d.plane * (size_t)(m->d.nz + 1), es = mixed ? sizeof(float) : sizeof(double);
  vibe_gb300_physics_args a{};
  a.precision = mixed ? VIBE_GB300_MIXED : VIBE_GB300_FP64;
  a.stage = stage;
  a.dt = dt;
  a.nx = m->d.nx;
  a.ny = m->d.ny;
  a.nz = m->d.nz;
  a.pitch = m->d.P;
  a.moist = m->fl.moist ? 1 : 0;
  for (int q = 0; q < NSPECIES; ++q) a.state[q] = state[q];
  unsigned all = 0;
  for (int q : kPhysFields) {
    all |= 1u << q;
    if (m->phys_written & (1u << q)) CUDA_OK(cudaMemsetAsync(m->pt[q], 0, n * es, m->stream));
    a.tend[q] = m->pt[q];
  }
  a.written = all;
  a.ref_theta = m->d_th0;
  a.ref_pi = m->d_pi0;
  a.ref_rho = m->d_rho0;
  a.zeta_mid = m->d_zmid;
  a.terrain = m->d_zs;
  a.depth = m->d_scale;
  a.stream = m->stream;
  if (int rc = m->phys_fn(m->phys_user, &a)) return fail(rc < 0 ? rc : VIBE_GB300_EDEVICE, "physics package failed");
  CUDA_OK(cudaGetLastError());
  m->phys_written = a.written & all;
  return 0;
}

// One step's launches on the model stream (the state ping-pong m->cur flips).
int enqueue_one_step(vibe_gb300_model* m, double dt, int n_sub) {
  const double dts[3] = {dt / 3.0, dt / 2.0, dt};
  const Dims& d = m->d;
  {
    double** S0 = m->S[m->cur];
    double** S1 = m->S[1 - m->cur];
    if (m->precision == VIBE_GB300_FP64) {
      for (int stage = 0; stage < 3; ++stage) {
        double** src = (stage == 0) ? S0 : S1;
        {
          Span sp(m, 0);
          m->f64->slow_tendency(d, m->met, m->fl, src, m->tend, m->scratch, m->wface, m->stream);
          if (m->phys_fn) {
            if (int rc = physics_stage(m, stage, dt, (const void* const*)src)) return rc;
            const size_t n = d.plane * (size_t)(d.nz + 1);
            for (int q : kPhysFields)
              if (m->phys_written & (1u << q))
                k_add_pt64<<<1024, 256, 0, m->stream>>>(n, (const double*)m->pt[q], m->tend[q]);
          }
          m->f64->stage_update(d, S0, m->tend, dts[stage], S1, m->stream);
        }
        const double dtau = dts[stage] / (double)n_sub;
        if (m->fl.acoustic_mode == 1)
          if (int rc = ref_hevi_coefficients(m, dtau)) return rc;
        for (int n = 0; n < n_sub; ++n) {
          Span sp(m, 1);
          if (m->fl.acoustic_mode == 0) m->f64->fb_substep(d, m->met, m->fl, S1, dtau, m->stream);
          else if (m->fl.acoustic_mode == 1)
            m->f64->ref_hevi_substep(d, m->met, S1, dtau, m->d_tri, m->d_tri + d.nz, m->d_tri + 2 * d.nz, m->scratch,
                                  m->d_err, m->stream);
          else m->f64->cons_hevi_substep(d, m->met, m->fl, S1, m->tmp, m->scratch, dtau, m->d_err, m->stream);
        }
        Span sp(m, 2);
        m->f64->nonfinite(d, S1, m->d_err, m->stream);
        if (stage < 2 && m->rec_stage[stage])
          for (int q = 0; q < NSPECIES; ++q)
            CUDA_OK(cudaMemcpyAsync(m->rec_stage[stage][q], S1[q], d.plane * (size_t)(d.nz + 1) * sizeof(double),
                                    cudaMemcpyDeviceToDevice, m->stream));
      }
      Span sp(m, 2);
      m->f64->sponge(d, m->met, S1, m->kmin, dt, m->stream);
      if (m->fl.w_rigid) {
        const dim3 b(32, 8);
        k_rigid_w<<<dim3((d.nx + 31) / 32, (d.ny + 7) / 8), b, 0, m->stream>>>(d, S1[W]);
      }
    } else {
      const WS w0 = ws_of(m->W0);
      float** final_sub = nullptr;
      float last_dtau = 0.f;
      for (int stage = 0; stage < 3; ++stage) {
        float** st_out = m->WSt[stage & 1];
        const WS win = (stage == 0) ? w0 : ws_compose(final_sub, m->WSt[(stage - 1) & 1]);
        {
          Span sp(m, 0);
          const WS wr = ws_of(m->WR);
          if (m->phys_fn) {  // on the stage input, before the stage kernel overwrites nothing it reads
            const void* st[NSPECIES];
            for (int q = 0; q < NSPECIES; ++q) st[q] = win.f[q];
            if (int rc = physics_stage(m, stage, dt, st)) return rc;
          }
          if (mixed_stage(d, m->tab, m->fl, win, w0, ws_of(st_out), stage == 2 ? &wr : nullptr, dts[stage],
                          m->d_err, m->stream))
            return fail(VIBE_GB300_EDEVICE, "TMA descriptor creation failed (cuTensorMapEncodeTiled)");
          if (m->phys_fn) {
            const size_t n = d.plane * (size_t)(d.nz + 1);
            for (int q : kPhysFields)
              if (m->phys_written & (1u << q))
                k_add_pt32<<<1024, 256, 0, m->stream>>>(n, (const float*)m->pt[q], st_out[q], (float)dts[stage],
                                                        stage == 2 ? m->WR[q] : nullptr);
          }
        }
        const float dtau = (float)(dts[stage] / (double)n_sub);
        float** in = st_out;
        for (int n = 0; n < n_sub; ++n) {
          float** out = (n & 1) ? m->WB : m->WA;
          if (m->fl.acoustic_mode == 2) {
            // the u/v update of substep n-1 is applied inside substep n's column kernel
            Span sp(m, 1);
            if (mixed_hevi_column(d, m->tab, m->fl, ws_of(in), ws_of(out), dtau, m->d_lu + (size_t)stage * 3 * d.nz,
                                  n > 0, m->d_err, m->stream))
              return fail(VIBE_GB300_EDEVICE, "TMA descriptor creation failed (cuTensorMapEncodeTiled)");
          } else {
            Span sp(m, 1);
            mixed_fb_substep(d, m->tab, m->fl, ws_of(in), ws_of(out), dtau, m->stream);
          }
          in = out;
        }
        if (m->fl.acoustic_mode == 2 && stage < 2) {  // the last substep's u/v update, in place
          Span sp(m, 3);
          if (mixed_hevi_defers(d)) mixed_uv_fix(d, m->tab, m->fl, ws_of(in), dtau, m->stream);
          else mixed_uv_backward(d, m->tab, ws_of(in), ws_of(in), dtau, m->stream);
        }
        final_sub = in;
        last_dtau = dtau;
        if (stage < 2 && m->rec_stage[stage]) {
          // the next stage's input as FP64 totals; what the working copy does
          // not hold (inactive species, points off the boxes) from the step's start
          for (int q = 0; q < NSPECIES; ++q)
            CUDA_OK(cudaMemcpyAsync(m->rec_stage[stage][q], S0[q], d.plane * (size_t)(d.nz + 1) * sizeof(double),
                                    cudaMemcpyDeviceToDevice, m->stream));
          WS next = ws_compose(in, m->WSt[stage & 1]);
          if (!m->fl.moist)
            for (int q = QV + 1; q < NSPECIES; ++q) next.f[q] = nullptr;
          working_to_f64(d, m->tab, next, m->rec_stage[stage], m->stream);
        }
      }
      Span sp(m, 2);
      const WS wr = ws_of(m->WR);
      // stage 3's last u/v update is folded into the finish kernel
      mixed_finish(d, m->tab, m->fl, ws_of(final_sub), ws_of(m->WSt[0]), w0, &wr, dt, S0, S1, m->d_err, m->stream,
                   m->fl.acoustic_mode == 2 ? last_dtau : 0.f, m->fl.acoustic_mode == 2 && mixed_hevi_defers(d));
    }
    m->cur = 1 - m->cur;
  }
  CUDA_OK(cudaGetLastError());
  return 0;
}

void drop_graphs(vibe_gb300_model* m) {
  for (int p = 0; p < 2; ++p) {
    if (m->gexec[p]) cudaGraphExecDestroy(m->gexec[p]);
    m->gexec[p] = nullptr;
  }
  m->graph_dt = -1.0;
  m->graph_nsub = -1;
}

// The mixed step as a CUDA graph: one graph per state parity (the step reads
// S[cur] and writes S[1-cur]), captured from the same launches the eager
// path enqueues, after one eager step with the same dt/n_sub has set every
// kernel attribute. Replayed with one cudaGraphLaunch per step.
int enqueue_steps(vibe_gb300_model* m, double dt, int n_sub_in, int n_steps) {
  const int n_sub = n_sub_in > 1 ? n_sub_in : 1;
  if (int rc = configure_dt(m, dt, n_sub)) return rc;
  const bool graph = m->use_graph && !m->timing && m->precision == VIBE_GB300_MIXED;
  if (graph && (m->graph_dt != dt || m->graph_nsub != n_sub)) {
    drop_graphs(m);
    m->graph_dt = dt;
    m->graph_nsub = n_sub;
    m->graph_warm = false;
  }
  for (int step = 0; step < n_steps; ++step) {
    if (!graph || !m->graph_warm) {
      if (int rc = enqueue_one_step(m, dt, n_sub)) return rc;
      m->graph_warm = true;
      continue;
    }
    const int parity = m->cur;
    if (!m->gexec[parity]) {
      cudaGraph_t g = nullptr;
      CUDA_OK(cudaStreamBeginCapture(m->stream, cudaStreamCaptureModeThreadLocal));
      const int rc = enqueue_one_step(m, dt, n_sub);
      const cudaError_t e = cudaStreamEndCapture(m->stream, &g);
      m->cur = parity;  // capture enqueues nothing: undo the flip
      if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
      }
      CUDA_OK(e);
      const cudaError_t ei = cudaGraphInstantiate(&m->gexec[parity], g, 0);
      cudaGraphDestroy(g);
      CUDA_OK(ei);
    }
    CUDA_OK(cudaGraphLaunch(m->gexec[parity], m->stream));
    m->cur = 1 - m->cur;
  }
  CUDA_OK(cudaGetLastError());
  return 0;
}

int read_status(vibe_gb300_model* m) {
  CUDA_OK(cudaMemcpyAsync(m->h_err, m->d_err, sizeof(unsigned), cudaMemcpyDeviceToHost, m->stream));
  CUDA_OK(cudaStreamSynchronize(m->stream));
  collect_timing(m);
  const unsigned e = *m->h_err;
  CUDA_OK(cudaMemsetAsync(m->d_err, 0, sizeof(unsigned), m->stream));
  if (e & kErrWaitTimeout) return fail(VIBE_GB300_EDEVICE, "a TMA box of the stage kernel did not arrive (bounded wait)");
  if (e & kErrSingular) return fail(VIBE_GB300_ESINGULAR, "tridiagonal pivot below 1e-300");
  if (e & kErrNonFinite) return fail(VIBE_GB300_ENONFINITE, "non-finite value in the state");
  return 0;
}

// the FP32 working copy's targets: moisture species beyond qv only when they
// are prognostic (no kernel of a dry model reads them)
WS working_targets(const vibe_gb300_model* m, float* const* w) {
  WS t = ws_of(w);
  if (!m->fl.moist)
    for (int q = QV + 1; q < NSPECIES; ++q) t.f[q] = nullptr;
  return t;
}

int sync_working(vibe_gb300_model* m) {
  if (m->precision != VIBE_GB300_MIXED) return 0;
  mixed_to_working(m->d, m->tab, m->S[m->cur], working_targets(m, m->W0), m->stream);
  CUDA_OK(cudaGetLastError());
  return 0;
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

const char* vibe_gb300_last_error(void) { return g_err.c_str(); }

void vibe_gb300_setup_defaults(vibe_gb300_setup* s) {
  std::memset(s, 0, sizeof(*s));
  s->nx = 64; s->ny = 64; s->nz = 40;
  s->dx = 250.0; s->dy = 250.0; s->z_top = 10000.0;
  s->zeta_first = 1.0; s->zeta_stretch = 1.0;
  s->ref_kind = 0; s->theta0 = 300.0; s->p_surf = 100000.0; s->bv_n = 0.01; s->profile_dz = 250.0;
  s->bubble_amplitude = 2.0; s->bubble_radius_x = 2000.0; s->bubble_radius_z = 2000.0;
  s->bubble_xc = 8000.0; s->bubble_yc = 8000.0; s->bubble_zc = 2000.0;
  s->qv_surface = 0.014; s->qv_decay_height = 3000.0;
  s->advection = 5; s->weno_scalars = 1; s->moist = 0; s->coriolis = 0; s->latitude = 45.0;
  s->sponge_alpha = 0.2; s->sponge_start_fraction = 0.8;
  s->divergence_damping = 0.0; s->divergence_order = 2;
  s->pgf_perturbation = 1; s->acoustic_mode = 0; s->hevi_beta = 0.5; s->split_fast = 1; s->weno_advective = 1;
}

int vibe_gb300_model_create(const vibe_gb300_setup* s, int precision, vibe_gb300_model** out) {
  if (!s || !out) return fail(VIBE_GB300_EBADARG, "null argument");
  *out = nullptr;
  if (s->nx < 1 || s->ny < 1 || s->nz < 1 || !(s->dx > 0) || !(s->dy > 0) || !(s->z_top > 0))
    return fail(VIBE_GB300_EBADARG, "grid sizes and spacings must be positive");
  if (precision != VIBE_GB300_FP64 && precision != VIBE_GB300_MIXED && precision != VIBE_GB300_FP64_EXACT)
    return fail(VIBE_GB300_EBADARG, "precision must be VIBE_GB300_FP64, _MIXED or _FP64_EXACT");
  if (s->acoustic_mode < 0 || s->acoustic_mode > 2) return fail(VIBE_GB300_EBADARG, "acoustic_mode must be 0, 1 or 2");
  auto* m = new vibe_gb300_model();
  m->su = *s;
  m->f64 = (precision == VIBE_GB300_FP64_EXACT) ? &kFp64Exact : &kFp64Fast;
  if (precision == VIBE_GB300_FP64_EXACT) precision = VIBE_GB300_FP64;  // same buffers and schedule
  m->precision = precision;
  auto bail = [&](int rc) { vibe_gb300_model_destroy(m); return rc; };
  const int nx = s->nx, ny = s->ny, nz = s->nz;
  for (int q = 0; q < NSPECIES; ++q) {
    m->nsx[q] = nx + 2 * H + (q == U);
    m->nsy[q] = ny + 2 * H + (q == V);
    m->nsz[q] = nz + 2 * H + (q == W);
  }
  m->d.nx = nx; m->d.ny = ny; m->d.nz = nz;
  m->d.P = ((nx + 1) + 7) / 8 * 8;
  m->d.NY1 = ny + 1;
  m->d.plane = (size_t)m->d.NY1 * m->d.P;
  Flags& fl = m->fl;
  fl.advection = s->advection; fl.weno_scalars = s->weno_scalars; fl.weno_advective = s->weno_advective;
  fl.moist = s->moist; fl.coriolis = s->coriolis; fl.div_damp = s->divergence_damping;
  fl.div_order = s->divergence_order; fl.pgf_pert = s->pgf_perturbation; fl.split_fast = s->split_fast;
  fl.w_rigid = s->w_rigid;
  fl.acoustic_mode = s->acoustic_mode; fl.hevi_beta = s->hevi_beta;
  host_setup(m);
  // horizontally uniform reference state on flat terrain?
  {
    const int cx = m->nsx[RHO], cy = m->nsy[RHO];
    for (size_t e = 0; e < m->hs.zs.size() && m->uniform; ++e) m->uniform = (m->hs.zs[e] == 0.0);
    for (int w = 0; w < 3 && m->uniform; ++w)
      for (int k = 0; k < nz && m->uniform; ++k)
        for (int j = 0; j < ny && m->uniform; ++j)
          for (int i = 0; i < nx && m->uniform; ++i)
            m->uniform = (m->hs.ref[w][soff(cx, cy, i, j, k)] == m->hs.ref[w][soff(cx, cy, 0, 0, k)]);
  }
  if (precision == VIBE_GB300_MIXED) {
    if (!m->uniform) return bail(fail(VIBE_GB300_EUNSUPPORTED, "mixed path needs flat terrain and a horizontally uniform reference state"));
    if (!s->pgf_perturbation || !s->split_fast)
      return bail(fail(VIBE_GB300_EUNSUPPORTED, "mixed path needs pgf_perturbation=1 and split_fast=1"));
    if (s->acoustic_mode == 1) return bail(fail(VIBE_GB300_EUNSUPPORTED, "mixed path supports acoustic_mode 0 and 2"));
    if (s->divergence_damping > 0.0 && s->divergence_order > 2)
      return bail(fail(VIBE_GB300_EUNSUPPORTED, "mixed path supports 2nd-order divergence damping only"));
    // the mixed kernels index a field with 32-bit offsets (any grid whose
    // state fits in device memory is far below this)
    if (m->d.plane * (size_t)(nz + 1) >= ((size_t)1 << 32))
      return bail(fail(VIBE_GB300_EUNSUPPORTED, "mixed path needs fewer than 2^32 elements per field"));
  }
  m->met.f0 = 2.0 * kOmega * std::sin(s->latitude * (kPi / 180.0));
  m->met.beta = 2.0 * kOmega * std::cos(s->latitude * (kPi / 180.0)) / kEarthRadius;
  if (cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) != cudaSuccess)
    return bail(fail(VIBE_GB300_EDEVICE, "cudaStreamCreate failed (no CUDA device?)"));
  const size_t nfield = m->d.plane * (size_t)(nz + 1);
  size_t max_storage = 0;
  for (int q = 0; q < NSPECIES; ++q) max_storage = std::max(max_storage, storage_count(m, q));
  int rc = 0;
  for (int b = 0; b < 2 && !rc; ++b)
    for (int q = 0; q < NSPECIES && !rc; ++q) rc = dalloc(m, &m->S[b][q], nfield);
  rc = rc ? rc : dalloc(m, &m->d_stage_in, max_storage);
  rc = rc ? rc : dalloc(m, &m->d_dzeta, (size_t)nz);
  rc = rc ? rc : dalloc(m, &m->d_scale, (size_t)nx * ny);
  rc = rc ? rc : dalloc(m, &m->d_sponge, (size_t)nz);
  rc = rc ? rc : dalloc(m, &m->d_th0, nfield);
  rc = rc ? rc : dalloc(m, &m->d_pi0, nfield);
  rc = rc ? rc : dalloc(m, &m->d_rho0, nfield);
  rc = rc ? rc : dalloc(m, &m->d_err, (size_t)1);
  rc = rc ? rc : dalloc(m, &m->d_tri, 3 * (size_t)nz);
  if (!rc && precision == VIBE_GB300_FP64) {
    for (int q = 0; q < NSPECIES && !rc; ++q) rc = dalloc(m, &m->tend[q], nfield);
    for (int q = 0; q < NSPECIES && !rc; ++q) rc = (q == W || q == RHO || q == PI) ? dalloc(m, &m->tmp[q], nfield) : 0;
    const size_t scr = std::max(m->d.plane * (size_t)nz + (size_t)nx * ny * 2 * nz, (size_t)nx * ny * (6 * (size_t)nz + 6));
    rc = rc ? rc : dalloc(m, &m->scratch, std::max(scr, nfield));
    rc = rc ? rc : dalloc(m, &m->wface, 3 * nfield);  // WENO face fluxes of one scalar (x, y, z faces)
  }
  if (!rc && precision == VIBE_GB300_MIXED) {
    for (int q = 0; q < NSPECIES && !rc; ++q) rc = dalloc(m, &m->W0[q], nfield);
    for (int b = 0; b < 2 && !rc; ++b)
      for (int q = 0; q < NSPECIES && !rc; ++q) rc = dalloc(m, &m->WSt[b][q], nfield);
    for (int q = 0; q < NSPECIES && !rc; ++q) rc = acoustic_field(q) ? dalloc(m, &m->WA[q], nfield) : 0;
    for (int q = 0; q < NSPECIES && !rc; ++q) rc = acoustic_field(q) ? dalloc(m, &m->WB[q], nfield) : 0;
    for (int q = 0; q < NSPECIES && !rc; ++q) rc = dalloc(m, &m->WR[q], nfield);
    rc = rc ? rc : dalloc(m, &m->d_lu, 9 * (size_t)nz);
  }
  if (rc) return bail(rc);
  if (cudaMallocHost(&m->h_err, sizeof(unsigned)) != cudaSuccess) return bail(fail(VIBE_GB300_EDEVICE, "cudaMallocHost failed"));
  *m->h_err = 0;
  // metrics
  std::vector<double> dz(nz), sc((size_t)nx * ny);
  for (int k = 0; k < nz; ++k) dz[k] = m->hs.zeta[k + 1] - m->hs.zeta[k];
  for (size_t e = 0; e < sc.size(); ++e) sc[e] = s->z_top - m->hs.zs[e];
  if (cudaMemcpy(m->d_dzeta, dz.data(), nz * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(m->d_scale, sc.data(), sc.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(m->d_sponge, m->hs.sponge.data(), nz * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess)
    return bail(fail(VIBE_GB300_EDEVICE, "metric upload failed"));
  m->met.dx = s->dx; m->met.dy = s->dy; m->met.z_top = s->z_top;
  m->met.inv_dx = 1.0 / s->dx; m->met.inv_dy = 1.0 / s->dy;
  m->met.dzeta = m->d_dzeta; m->met.scale = m->d_scale; m->met.sponge = m->d_sponge;
  m->met.th0 = m->d_th0; m->met.pi0 = m->d_pi0; m->met.rho0 = m->d_rho0;
  {
    double* dst[1];
    dst[0] = m->d_th0;
    if ((rc = upload_storage(m, RHO, m->hs.ref[0].data(), dst, 1))) return bail(rc);
    CUDA_OK(cudaStreamSynchronize(m->stream));
    dst[0] = m->d_pi0;
    if ((rc = upload_storage(m, RHO, m->hs.ref[1].data(), dst, 1))) return bail(rc);
    CUDA_OK(cudaStreamSynchronize(m->stream));
    dst[0] = m->d_rho0;
    if ((rc = upload_storage(m, RHO, m->hs.ref[2].data(), dst, 1))) return bail(rc);
    CUDA_OK(cudaStreamSynchronize(m->stream));
  }
  if (m->uniform)
    if ((rc = build_tables(m))) return bail(rc);
  for (int q = 0; q < NSPECIES; ++q)
    if ((rc = vibe_gb300_set_field(m, q, m->hs.st[q].data()))) return bail(rc);
  *out = m;
  return 0;
}

void vibe_gb300_model_destroy(vibe_gb300_model* m) {
  if (m && m->hz) vibe_helmholtz_destroy(m->hz);
  if (m && m->hz_ev[0]) { cudaEventDestroy(m->hz_ev[0]); cudaEventDestroy(m->hz_ev[1]); }
  if (m) drop_graphs(m);
  if (!m) return;
  if (m->stream) cudaStreamSynchronize(m->stream);
  io_release(m);
  collect_timing(m);
  for (cudaEvent_t e : m->ev_pool) cudaEventDestroy(e);
  for (void* p : m->allocs) cudaFree(p);
  if (m->h_err) cudaFreeHost(m->h_err);
  if (m->h_pin) cudaFreeHost(m->h_pin);
  if (m->stream) cudaStreamDestroy(m->stream);
  delete m;
}

size_t vibe_gb300_storage_size(const vibe_gb300_model* m, int species) {
  if (!m || species < 0 || species >= NSPECIES) return 0;
  return storage_count(m, species);
}

int vibe_gb300_set_field(vibe_gb300_model* m, int q, const double* host) {
  if (!m || !host || q < 0 || q >= NSPECIES) return fail(VIBE_GB300_EBADARG, "bad argument");
  double* dst[2] = {m->S[0][q], m->S[1][q]};
  if (int rc = upload_storage(m, q, host, dst, 2)) return rc;
  if (int rc = sync_working(m)) return rc;
  CUDA_OK(cudaStreamSynchronize(m->stream));
  if (m->precision == VIBE_GB300_MIXED) {
    // every FP32 buffer starts from the same values (ghost line included)
    const size_t n = m->d.plane * (size_t)(m->d.nz + 1) * sizeof(float);
    for (int b = 0; b < 2; ++b) CUDA_OK(cudaMemcpyAsync(m->WSt[b][q], m->W0[q], n, cudaMemcpyDeviceToDevice, m->stream));
    if (acoustic_field(q)) {
      CUDA_OK(cudaMemcpyAsync(m->WA[q], m->W0[q], n, cudaMemcpyDeviceToDevice, m->stream));
      CUDA_OK(cudaMemcpyAsync(m->WB[q], m->W0[q], n, cudaMemcpyDeviceToDevice, m->stream));
    }
    CUDA_OK(cudaStreamSynchronize(m->stream));
  }
  return 0;
}

int vibe_gb300_get_field(vibe_gb300_model* m, int q, double* host) {
  if (!m || !host || q < 0 || q >= NSPECIES) return fail(VIBE_GB300_EBADARG, "bad argument");
  const size_t n = storage_count(m, q);
  int ni, nj, nk;
  box_of(m, q, ni, nj, nk);
  unpack<double>(m->d, m->nsx[q], m->nsy[q], m->nsz[q], ni, nj, nk, m->S[m->cur][q],
                                        m->d_stage_in, m->stream);
  CUDA_OK(cudaGetLastError());
  CUDA_OK(cudaMemcpyAsync(host, m->d_stage_in, n * sizeof(double), cudaMemcpyDeviceToHost, m->stream));
  CUDA_OK(cudaStreamSynchronize(m->stream));
  return 0;
}

int vibe_gb300_get_reffield(const vibe_gb300_model* m, int which, double* host) {
  if (!m || !host || which < 0 || which > 4) return fail(VIBE_GB300_EBADARG, "bad argument");
  std::memcpy(host, m->hs.ref[which].data(), m->hs.ref[which].size() * sizeof(double));
  return 0;
}
int vibe_gb300_get_zeta(const vibe_gb300_model* m, double* host) {
  if (!m || !host) return fail(VIBE_GB300_EBADARG, "bad argument");
  std::memcpy(host, m->hs.zeta.data(), m->hs.zeta.size() * sizeof(double));
  return 0;
}
int vibe_gb300_get_terrain(const vibe_gb300_model* m, double* host) {
  if (!m || !host) return fail(VIBE_GB300_EBADARG, "bad argument");
  std::memcpy(host, m->hs.zs.data(), m->hs.zs.size() * sizeof(double));
  return 0;
}
int vibe_gb300_get_sponge(const vibe_gb300_model* m, double* host) {
  if (!m || !host) return fail(VIBE_GB300_EBADARG, "bad argument");
  std::memcpy(host, m->hs.sponge.data(), m->hs.sponge.size() * sizeof(double));
  return 0;
}

int vibe_gb300_step_async(vibe_gb300_model* m, double dt, int n_sub, int n_steps) {
  if (!m || n_steps < 0 || !(dt > 0)) return fail(VIBE_GB300_EBADARG, "bad argument");
  return enqueue_steps(m, dt, n_sub, n_steps);
}

int vibe_gb300_sync(vibe_gb300_model* m) {
  if (!m) return fail(VIBE_GB300_EBADARG, "bad argument");
  if (int rc = vibe_gb300_io_join(m)) return rc;
  return read_status(m);
}

int vibe_gb300_step(vibe_gb300_model* m, double dt, int n_sub, int n_steps) {
  if (int rc = vibe_gb300_step_async(m, dt, n_sub, n_steps)) return rc;
  return read_status(m);
}

int vibe_gb300_slow_tendency(vibe_gb300_model* m, double* const* host_out) {
  if (!m || !host_out) return fail(VIBE_GB300_EBADARG, "bad argument");
  if (m->precision == VIBE_GB300_MIXED) {
    // the stage kernel with no base state writes the raw FP32 tendency
    if (int rc = sync_working(m)) return rc;
    WS none;
    for (int q = 0; q < NSPECIES; ++q) none.f[q] = nullptr;
    if (mixed_stage(m->d, m->tab, m->fl, ws_of(m->W0), none, ws_of(m->WSt[1]), nullptr, 1.0, m->d_err, m->stream))
      return fail(VIBE_GB300_EDEVICE, "TMA descriptor creation failed (cuTensorMapEncodeTiled)");
    for (int q = 0; q < NSPECIES; ++q) {
      int ni = m->d.nx + (q == U), nj = m->d.ny + (q == V), nk = m->d.nz + (q == W);
      const bool active = q <= QV || m->fl.moist;
      if (!active) { ni = 0; }
      mixed_unpack_f32(m->d, m->nsx[q], m->nsy[q], m->nsz[q], ni, nj, nk, m->WSt[1][q], m->d_stage_in, m->stream);
      CUDA_OK(cudaMemcpyAsync(host_out[q], m->d_stage_in, storage_count(m, q) * sizeof(double), cudaMemcpyDeviceToHost,
                              m->stream));
      CUDA_OK(cudaStreamSynchronize(m->stream));
    }
    // WSt[1] now holds tendencies: restore its ghost line / inactive species
    const size_t n = m->d.plane * (size_t)(m->d.nz + 1) * sizeof(float);
    for (int q = 0; q < NSPECIES; ++q) CUDA_OK(cudaMemcpyAsync(m->WSt[1][q], m->W0[q], n, cudaMemcpyDeviceToDevice, m->stream));
    CUDA_OK(cudaStreamSynchronize(m->stream));
    return read_status(m);
  }
  m->f64->slow_tendency(m->d, m->met, m->fl, m->S[m->cur], m->tend, m->scratch, m->wface, m->stream);
  for (int q = 0; q < NSPECIES; ++q) {
    int ni, nj, nk;
    box_of(m, q, ni, nj, nk);
    if (q == U) nj = m->d.ny;
    else if (q == V) ni = m->d.nx;
    else if (q == W) { ni = m->d.nx; nj = m->d.ny; }
    else { ni = m->d.nx; nj = m->d.ny; }
    unpack<double>(m->d, m->nsx[q], m->nsy[q], m->nsz[q], ni, nj, nk, m->tend[q], m->d_stage_in, m->stream);
    CUDA_OK(cudaMemcpyAsync(host_out[q], m->d_stage_in, storage_count(m, q) * sizeof(double), cudaMemcpyDeviceToHost,
                            m->stream));
    CUDA_OK(cudaStreamSynchronize(m->stream));
  }
  CUDA_OK(cudaGetLastError());
  return 0;
}

int vibe_gb300_acoustic_substep(vibe_gb300_model* m, double dtau) {
  if (!m) return fail(VIBE_GB300_EBADARG, "bad argument");
  if (m->precision == VIBE_GB300_FP64) {
    m->f64->fb_substep(m->d, m->met, m->fl, m->S[m->cur], dtau, m->stream);
  } else {
    if (int rc = sync_working(m)) return rc;
    mixed_fb_substep(m->d, m->tab, m->fl, ws_of(m->W0), ws_of(m->WA), (float)dtau, m->stream);
    Tab id = m->tab;
    id.spwd = m->d_spid; id.spdt = m->d_spid + (m->d.nz + 1); id.spw = m->d_spif;
    mixed_finish(m->d, id, m->fl, ws_compose(m->WA, m->W0), ws_of(m->W0), ws_of(m->WSt[1]), nullptr, 0.0,
                 m->S[m->cur], m->S[m->cur], m->d_err, m->stream);
  }
  CUDA_OK(cudaGetLastError());
  return read_status(m);
}

// FieldT storage -> device layout over the staggered box (inverse of k_pack);
// points outside the box keep what dst holds
__global__ void k_scatter(Dims d, int nsx, int nsy, int ni, int nj, int nk, const double* __restrict__ src,
                          double* __restrict__ dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
  if (i >= ni || j >= nj || k >= nk) return;
  dst[soff(nsx, nsy, i, j, k)] = src[d.idx(i, j, k)];
}

namespace {
constexpr int kLinField[5] = {U, V, W, RHO, PI};

// hevi: the consistent HEVI substep (k_chevi_column + k_uv_backward) instead
// of the explicit forward-backward one
int acoustic_linear(vibe_gb300_model* m, double dtau, int n_sub, const double* const* in, double* const* out,
                    bool adjoint, bool hevi = false) {
  if (!m || !in || !out || n_sub < 0) return fail(VIBE_GB300_EBADARG, "bad argument");
  for (int f = 0; f < 5; ++f)
    if (!in[f] || !out[f]) return fail(VIBE_GB300_EBADARG, "bad argument");
  const size_t nfield = m->d.plane * (size_t)(m->d.nz + 1);
  if (!m->lin[0]) {
    for (int f = 0; f < 5; ++f)
      if (int rc = dalloc(m, &m->lin[f], nfield)) return rc;
  }
  if (hevi && !m->lin_scr) {
    for (int f = 0; f < 3; ++f)
      if (int rc = dalloc(m, &m->lin_tmp[f], nfield)) return rc;
    if (int rc = dalloc(m, &m->lin_dh, nfield)) return rc;
    if (int rc = dalloc(m, &m->lin_scr, (size_t)m->d.nx * m->d.ny * (6 * (size_t)m->d.nz + 6))) return rc;
  }
  double* st[NSPECIES] = {};  // the substep kernels see the perturbation as their state
  for (int f = 0; f < 5; ++f) {
    st[kLinField[f]] = m->lin[f];
    if (int rc = upload_storage(m, kLinField[f], in[f], &m->lin[f], 1)) return rc;
  }
  Flags lf = m->fl;
  lf.pgf_pert = 0;  // gradient of pi' itself: the substep is linear
  double* tmp[NSPECIES] = {};
  tmp[W] = m->lin_tmp[0];
  tmp[RHO] = m->lin_tmp[1];
  tmp[PI] = m->lin_tmp[2];
  for (int n = 0; n < n_sub; ++n) {
    if (hevi) {
      if (adjoint) m->f64->hevi_substep_ad(m->d, m->met, lf, st, m->lin_dh, m->lin_scr, dtau, m->d_err, m->stream);
      else m->f64->cons_hevi_substep(m->d, m->met, lf, st, tmp, m->lin_scr, dtau, m->d_err, m->stream);
    } else {
      if (adjoint) m->f64->fb_substep_ad(m->d, m->met, st, dtau, m->stream);
      else m->f64->fb_substep(m->d, m->met, lf, st, dtau, m->stream);
    }
  }
  CUDA_OK(cudaGetLastError());
  const dim3 b(32, 4);
  for (int f = 0; f < 5; ++f) {
    const int q = kLinField[f];
    int ni, nj, nk;
    box_of(m, q, ni, nj, nk);
    const size_t n = storage_count(m, q);
    CUDA_OK(cudaMemcpyAsync(m->d_stage_in, in[f], n * sizeof(double), cudaMemcpyHostToDevice, m->stream));
    k_scatter<<<dim3((ni + 31) / 32, (nj + 3) / 4, nk), b, 0, m->stream>>>(m->d, m->nsx[q], m->nsy[q], ni, nj, nk,
                                                                            m->lin[f], m->d_stage_in);
    CUDA_OK(cudaGetLastError());
    CUDA_OK(cudaMemcpyAsync(out[f], m->d_stage_in, n * sizeof(double), cudaMemcpyDeviceToHost, m->stream));
    CUDA_OK(cudaStreamSynchronize(m->stream));
  }
  return read_status(m);
}
}  // namespace

// FieldT storage (double) <-> FP32 device layout over the staggered box
__global__ void k_pack_to_f32(Dims d, int nsx, int nsy, int ni, int nj, int nk, const double* __restrict__ src,
                              float* __restrict__ dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
  if (i >= ni || j >= nj || k >= nk) return;
  dst[d.idx(i, j, k)] = (float)src[soff(nsx, nsy, i, j, k)];
}
__global__ void k_scatter_from_f32(Dims d, int nsx, int nsy, int ni, int nj, int nk, const float* __restrict__ src,
                                   double* __restrict__ dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
  if (i >= ni || j >= nj || k >= nk) return;
  dst[soff(nsx, nsy, i, j, k)] = (double)src[d.idx(i, j, k)];
}

namespace {
// the mixed model's own FP32 forward-backward substep (mixed_fb_substep) on
// perturbations of (u, v, w, rho', pi'), and its adjoint
int acoustic_linear_f32(vibe_gb300_model* m, double dtau, int n_sub, const double* const* in, double* const* out,
                        bool adjoint, bool hevi = false) {
  if (!m || !in || !out || n_sub < 0) return fail(VIBE_GB300_EBADARG, "bad argument");
  if (m->precision != VIBE_GB300_MIXED) return fail(VIBE_GB300_EUNSUPPORTED, "the FP32 form needs a mixed model");
  for (int f = 0; f < 5; ++f)
    if (!in[f] || !out[f]) return fail(VIBE_GB300_EBADARG, "bad argument");
  const size_t nfield = m->d.plane * (size_t)(m->d.nz + 1);
  if (!m->lin32[0][0])
    for (int b = 0; b < 2; ++b)
      for (int f = 0; f < 5; ++f)
        if (int rc = dalloc(m, &m->lin32[b][f], nfield)) return rc;
  if (hevi && !m->lin32_dh) {
    if (int rc = dalloc(m, &m->lin32_dh, nfield)) return rc;
    if (int rc = dalloc(m, &m->lin32_scr, (size_t)m->d.nx * m->d.ny * (4 * (size_t)m->d.nz + 2))) return rc;
  }
  if (hevi) {  // the column factors for this dtau in stage slot 0, as vibe_gb300_hevi_substep sets them
    m->cfg_dt = -1.0;
    if (int rc = configure_dt(m, 3.0 * dtau, 1)) return rc;
  }
  const dim3 bl(32, 4);
  auto ws_lin = [&](int b) {
    WS w;
    for (int q = 0; q < NSPECIES; ++q) w.f[q] = nullptr;
    for (int f = 0; f < 5; ++f) w.f[kLinField[f]] = m->lin32[b][f];
    return w;
  };
  for (int f = 0; f < 5; ++f) {
    const int q = kLinField[f];
    int ni, nj, nk;
    box_of(m, q, ni, nj, nk);
    CUDA_OK(cudaMemcpyAsync(m->d_stage_in, in[f], storage_count(m, q) * sizeof(double), cudaMemcpyHostToDevice,
                            m->stream));
    k_pack_to_f32<<<dim3((ni + 31) / 32, (nj + 3) / 4, nk), bl, 0, m->stream>>>(m->d, m->nsx[q], m->nsy[q], ni, nj,
                                                                                nk, m->d_stage_in, m->lin32[0][f]);
    CUDA_OK(cudaMemcpyAsync(m->lin32[1][f], m->lin32[0][f], nfield * sizeof(float), cudaMemcpyDeviceToDevice,
                            m->stream));
  }
  int cur = 0;
  for (int n = 0; n < n_sub; ++n) {
    if (hevi) {
      if (adjoint) {
        mixed_hevi_substep_ad(m->d, m->tab, m->fl, ws_lin(0), m->d_lu, m->lin32_dh, m->lin32_scr, (float)dtau,
                              m->stream);
      } else {
        if (mixed_hevi_substep(m->d, m->tab, m->fl, ws_lin(cur), ws_lin(1 - cur), (float)dtau, m->d_lu, m->d_err,
                               m->stream))
          return fail(VIBE_GB300_EDEVICE, "TMA descriptor creation failed (cuTensorMapEncodeTiled)");
        cur = 1 - cur;
      }
    } else if (adjoint) {
      mixed_fb_substep_ad(m->d, m->tab, ws_lin(0), (float)dtau, m->stream);
    } else {
      mixed_fb_substep(m->d, m->tab, m->fl, ws_lin(cur), ws_lin(1 - cur), (float)dtau, m->stream);
      cur = 1 - cur;
    }
  }
  CUDA_OK(cudaGetLastError());
  for (int f = 0; f < 5; ++f) {
    const int q = kLinField[f];
    int ni, nj, nk;
    box_of(m, q, ni, nj, nk);
    const size_t n = storage_count(m, q);
    CUDA_OK(cudaMemcpyAsync(m->d_stage_in, in[f], n * sizeof(double), cudaMemcpyHostToDevice, m->stream));
    k_scatter_from_f32<<<dim3((ni + 31) / 32, (nj + 3) / 4, nk), bl, 0, m->stream>>>(
        m->d, m->nsx[q], m->nsy[q], ni, nj, nk, m->lin32[cur][f], m->d_stage_in);
    CUDA_OK(cudaGetLastError());
    CUDA_OK(cudaMemcpyAsync(out[f], m->d_stage_in, n * sizeof(double), cudaMemcpyDeviceToHost, m->stream));
    CUDA_OK(cudaStreamSynchronize(m->stream));
  }
  return read_status(m);
}
}  // namespace

int vibe_gb300_acoustic_tl_f32(vibe_gb300_model* m, double dtau, int n_sub, const double* const* in,
                               double* const* out) {
  return acoustic_linear_f32(m, dtau, n_sub, in, out, false);
}

int vibe_gb300_acoustic_ad_f32(vibe_gb300_model* m, double dtau, int n_sub, const double* const* in,
                               double* const* out) {
  return acoustic_linear_f32(m, dtau, n_sub, in, out, true);
}

int vibe_gb300_hevi_tl_f32(vibe_gb300_model* m, double dtau, int n_sub, const double* const* in, double* const* out) {
  return acoustic_linear_f32(m, dtau, n_sub, in, out, false, true);
}

int vibe_gb300_hevi_ad_f32(vibe_gb300_model* m, double dtau, int n_sub, const double* const* in, double* const* out) {
  return acoustic_linear_f32(m, dtau, n_sub, in, out, true, true);
}

int vibe_gb300_acoustic_tl(vibe_gb300_model* m, double dtau, int n_sub, const double* const* in, double* const* out) {
  return acoustic_linear(m, dtau, n_sub, in, out, false);
}

int vibe_gb300_acoustic_ad(vibe_gb300_model* m, double dtau, int n_sub, const double* const* in, double* const* out) {
  return acoustic_linear(m, dtau, n_sub, in, out, true);
}

int vibe_gb300_hevi_tl(vibe_gb300_model* m, double dtau, int n_sub, const double* const* in, double* const* out) {
  return acoustic_linear(m, dtau, n_sub, in, out, false, true);
}

int vibe_gb300_hevi_ad(vibe_gb300_model* m, double dtau, int n_sub, const double* const* in, double* const* out) {
  return acoustic_linear(m, dtau, n_sub, in, out, true, true);
}

int vibe_gb300_hevi_substep(vibe_gb300_model* m, double dtau) {
  if (!m) return fail(VIBE_GB300_EBADARG, "bad argument");
  if (m->fl.acoustic_mode == 0) return fail(VIBE_GB300_EBADARG, "acoustic_mode 0 has no HEVI substep");
  if (m->precision == VIBE_GB300_FP64) {
    if (m->fl.acoustic_mode == 1) {
      if (int rc = ref_hevi_coefficients(m, dtau)) return rc;
      m->f64->ref_hevi_substep(m->d, m->met, m->S[m->cur], dtau, m->d_tri, m->d_tri + m->d.nz, m->d_tri + 2 * m->d.nz,
                            m->scratch, m->d_err, m->stream);
    } else {
      m->f64->cons_hevi_substep(m->d, m->met, m->fl, m->S[m->cur], m->tmp, m->scratch, dtau, m->d_err, m->stream);
    }
  } else {
    // single substep: factors for this dtau in stage slot 0
    const double dt_equiv = 3.0 * dtau;  // stage 0 uses dt/3 with n_sub = 1
    m->cfg_dt = -1.0;
    if (int rc = configure_dt(m, dt_equiv, 1)) return rc;
    if (int rc = sync_working(m)) return rc;
    if (mixed_hevi_substep(m->d, m->tab, m->fl, ws_of(m->W0), ws_of(m->WA), (float)dtau, m->d_lu, m->d_err, m->stream))
      return fail(VIBE_GB300_EDEVICE, "TMA descriptor creation failed (cuTensorMapEncodeTiled)");
    Tab id = m->tab;
    id.spwd = m->d_spid; id.spdt = m->d_spid + (m->d.nz + 1); id.spw = m->d_spif;
    mixed_finish(m->d, id, m->fl, ws_compose(m->WA, m->W0), ws_of(m->W0), ws_of(m->WSt[1]), nullptr, 0.0,
                 m->S[m->cur], m->S[m->cur], m->d_err, m->stream);
    m->cfg_dt = -1.0;
  }
  CUDA_OK(cudaGetLastError());
  return read_status(m);
}

// ---- autotuner: time the launch shapes of the mixed step that give the
// same bits (column kernel variant, then the stage kernel's levels per
// block) on this model's grid and keep the fastest for the process.
int vibe_gb300_autotune(vibe_gb300_model* m, double dt, int n_sub, vibe_gb300_tuning* out) {
  if (!m || !(dt > 0.0) || !out) return fail(VIBE_GB300_EBADARG, "bad argument");
  if (m->precision != VIBE_GB300_MIXED) return fail(VIBE_GB300_EUNSUPPORTED, "the autotuner tunes the mixed path");
  CUDA_OK(cudaStreamSynchronize(m->stream));
  const int cur0 = m->cur;  // the trials' steps flip the state parity; it is put back with the state
  const size_t n = m->d.plane * (size_t)(m->d.nz + 1);
  std::vector<void*> keep(NSPECIES, nullptr);
  auto release = [&]() {
    for (void* p : keep)
      if (p) cudaFree(p);
  };
  for (int q = 0; q < NSPECIES; ++q) {
    if (cudaMalloc(&keep[q], n * sizeof(double)) != cudaSuccess) {
      release();
      return fail(VIBE_GB300_EDEVICE, "autotune state copy");
    }
    CUDA_OK(cudaMemcpyAsync(keep[q], m->S[m->cur][q], n * sizeof(double), cudaMemcpyDeviceToDevice, m->stream));
  }
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int kSteps = 3;
  auto trial = [&](const MixedTune& tn, double* ms) -> int {
    mixed_set_tune(m->d, tn);
    drop_graphs(m);
    for (int q = 0; q < NSPECIES; ++q)
      CUDA_OK(cudaMemcpyAsync(m->S[m->cur][q], keep[q], n * sizeof(double), cudaMemcpyDeviceToDevice, m->stream));
    if (int rc = sync_working(m)) return rc;
    if (int rc = enqueue_steps(m, dt, n_sub, 2)) return rc;  // eager step + graph capture
    CUDA_OK(cudaEventRecord(e0, m->stream));
    if (int rc = enqueue_steps(m, dt, n_sub, kSteps)) return rc;
    CUDA_OK(cudaEventRecord(e1, m->stream));
    if (int rc = read_status(m)) return rc;
    float t = 0.f;
    CUDA_OK(cudaEventElapsedTime(&t, e0, e1));
    *ms = t / kSteps;
    return 0;
  };
  MixedTune best, cur;
  double best_ms = 0.0, default_ms = 0.0, ms = 0.0;
  int rc = trial(MixedTune{}, &default_ms), tried = 1;
  best_ms = default_ms;
  // column kernel: 0 register ring, 1 cp.async ring, 2/3 two columns per thread, 4 TMA-fed two columns,
  // 5 the same with the w/rho' corrections deferred to the reader
  for (int c = 0; c <= 5 && !rc; ++c) {
    cur = MixedTune{};
    cur.column = c;
    rc = trial(cur, &ms);
    ++tried;
    if (!rc && ms < best_ms) { best_ms = ms; best = cur; }
  }
  // stage levels per block around the built-in choice
  const int base = mixed_stage_levels(m->d);
  // the chunk sizes that split the column evenly, the built-in one halved and
  // doubled, and the short chunks around it (wave quantisation of the grid)
  const int cand[] = {m->d.nz, (m->d.nz + 1) / 2, (m->d.nz + 2) / 3, (m->d.nz + 3) / 4, base / 2, base * 2,
                      base - 2, base - 1, base + 1, base + 2, base + 3};
  std::vector<int> seen;
  for (int v : cand) {
    if (rc || v < 4 || v > m->d.nz || v == base || std::find(seen.begin(), seen.end(), v) != seen.end()) continue;
    seen.push_back(v);
    cur = best;
    cur.stage_levels = v;
    rc = trial(cur, &ms);
    ++tried;
    if (!rc && ms < best_ms) { best_ms = ms; best = cur; }
  }
  mixed_set_tune(m->d, rc ? MixedTune{} : best);
  drop_graphs(m);
  m->cur = cur0;
  for (int q = 0; q < NSPECIES; ++q)
    cudaMemcpyAsync(m->S[m->cur][q], keep[q], n * sizeof(double), cudaMemcpyDeviceToDevice, m->stream);
  const int rs = sync_working(m);
  cudaStreamSynchronize(m->stream);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  release();
  if (rc) return rc;
  if (rs) return rs;
  out->stage_levels = best.stage_levels > 0 ? best.stage_levels : base;
  out->column_kernel = best.column;
  out->ms_per_step = best_ms;
  out->default_ms_per_step = default_ms;
  out->candidates = tried;
  return 0;
}

int vibe_gb300_set_physics(vibe_gb300_model* m, vibe_gb300_physics_fn fn, void* user) {
  if (!m) return fail(VIBE_GB300_EBADARG, "bad argument");
  if (fn && !m->pt[THETA]) {
    const size_t n = m->d.plane * (size_t)(m->d.nz + 1);
    for (int q : kPhysFields) {
      int rc = 0;
      if (m->precision == VIBE_GB300_MIXED) rc = dalloc(m, (float**)&m->pt[q], n);
      else rc = dalloc(m, (double**)&m->pt[q], n);
      if (rc) return rc;
    }
    const int nz = m->d.nz;
    std::vector<double> zmid(nz);
    for (int k = 0; k < nz; ++k) zmid[k] = 0.5 * (m->hs.zeta[k] + m->hs.zeta[k + 1]);  // geometry.cpp:20-31 at k + 1/2
    if (int rc = dalloc(m, &m->d_zmid, (size_t)nz)) return rc;
    if (int rc = dalloc(m, &m->d_zs, m->hs.zs.size())) return rc;
    CUDA_OK(cudaMemcpyAsync(m->d_zmid, zmid.data(), nz * sizeof(double), cudaMemcpyHostToDevice, m->stream));
    CUDA_OK(cudaMemcpyAsync(m->d_zs, m->hs.zs.data(), m->hs.zs.size() * sizeof(double), cudaMemcpyHostToDevice,
                            m->stream));
    CUDA_OK(cudaStreamSynchronize(m->stream));
  }
  // accumulators a package may have written are zero again before the next one's first call
  if (m->pt[THETA] && m->phys_written) {
    const size_t n = m->d.plane * (size_t)(m->d.nz + 1);
    const size_t es = m->precision == VIBE_GB300_MIXED ? sizeof(float) : sizeof(double);
    for (int q : kPhysFields)
      if (m->phys_written & (1u << q)) CUDA_OK(cudaMemsetAsync(m->pt[q], 0, n * es, m->stream));
    CUDA_OK(cudaStreamSynchronize(m->stream));
  }
  m->phys_fn = fn;
  m->phys_user = user;
  m->phys_written = 0;
  drop_graphs(m);
  return 0;
}

int vibe_gb300_physics_tendency(vibe_gb300_model* m, double dt, double* const* out) {
  if (!m || !out) return fail(VIBE_GB300_EBADARG, "bad argument");
  if (!m->phys_fn) return fail(VIBE_GB300_EBADARG, "no physics package installed");
  const void* st[NSPECIES];
  if (m->precision == VIBE_GB300_MIXED) {
    if (int rc = sync_working(m)) return rc;
    for (int q = 0; q < NSPECIES; ++q) st[q] = m->W0[q];
  } else {
    for (int q = 0; q < NSPECIES; ++q) st[q] = m->S[m->cur][q];
  }
  if (int rc = physics_stage(m, 0, dt, st)) return rc;
  for (int f = 0; f < 9; ++f) {
    const int q = kPhysFields[f];
    if (!out[f]) continue;
    int ni, nj, nk;
    box_of(m, q, ni, nj, nk);
    if (m->precision == VIBE_GB300_MIXED)
      unpack<float>(m->d, m->nsx[q], m->nsy[q], m->nsz[q], ni, nj, nk,
                                                (const float*)m->pt[q], m->d_stage_in, m->stream);
    else
      unpack<double>(m->d, m->nsx[q], m->nsy[q], m->nsz[q], ni, nj, nk,
                                            (const double*)m->pt[q], m->d_stage_in, m->stream);
    CUDA_OK(cudaGetLastError());
    CUDA_OK(cudaMemcpyAsync(out[f], m->d_stage_in, storage_count(m, q) * sizeof(double), cudaMemcpyDeviceToHost,
                            m->stream));
    CUDA_OK(cudaStreamSynchronize(m->stream));
  }
  return read_status(m);
}

int vibe_gb300_set_tuning(vibe_gb300_model* m, const vibe_gb300_tuning* t) {
  if (!m || !t || t->stage_levels < 0 || t->stage_levels > m->d.nz || t->column_kernel < -1 || t->column_kernel > 5)
    return fail(VIBE_GB300_EBADARG, "bad argument");
  MixedTune tn;
  tn.stage_levels = t->stage_levels;
  tn.column = t->column_kernel;
  mixed_set_tune(m->d, tn);
  drop_graphs(m);
  return 0;
}

// ---- restart files of the device state in the reference's .vibebin
// format (io::write_restart / read_restart, src/io/field_io.cpp:207-250;
// byte layout src/io/binary_writer.cpp:1-20 and 271-320): "VIBEBIN1",
// int32 nx ny nz, int32 real_kind (0), float64 time, int32 nvars, int32
// nlevels (= nz); then per variable char name[32] and float64 values over
// the stagger's points, i fastest; "__restart_info__" holds [time, step].
// Integers and doubles little-endian, assembled byte by byte.
}  // extern "C"

namespace {
const char* const kVbName[NSPECIES] = {"u", "v", "w", "rho", "theta", "pi", "qv", "qc", "qr", "qi", "qs", "qg"};

void vb_i32(std::vector<unsigned char>& b, int v) {
  const uint32_t u = (uint32_t)v;
  for (int s = 0; s < 32; s += 8) b.push_back((unsigned char)((u >> s) & 0xFFu));
}
void vb_f64(std::vector<unsigned char>& b, double v) {
  uint64_t u;
  std::memcpy(&u, &v, 8);
  for (int s = 0; s < 64; s += 8) b.push_back((unsigned char)((u >> s) & 0xFFu));
}
void vb_name(std::vector<unsigned char>& b, const char* name) {
  char n[32] = {};
  std::strncpy(n, name, 31);
  b.insert(b.end(), n, n + 32);
}
uint32_t rd_u32(const unsigned char* p) {
  return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}
double rd_f64(const unsigned char* p) {
  uint64_t u = 0;
  for (int i = 0; i < 8; ++i) u |= (uint64_t)p[i] << (8 * i);
  double v;
  std::memcpy(&v, &u, 8);
  return v;
}
// stagger implied by a variable name (binary_writer.cpp:100-118): 1 x-face, 2 y-face, 3 z-face, 0 cell
int vb_stagger(const std::string& n) {
  if (n == "u" || n == "u_facex") return 1;
  if (n == "v" || n == "v_facey") return 2;
  if (n == "w" || n == "zeta" || n == "w_facez") return 3;
  return 0;
}
}  // namespace

extern "C" {

int vibe_gb300_write_restart(vibe_gb300_model* m, const char* path, double time, int step) {
  if (!m || !path) return fail(VIBE_GB300_EBADARG, "bad argument");
  const int nx = m->d.nx, ny = m->d.ny, nz = m->d.nz;
  std::vector<unsigned char> b;
  b.insert(b.end(), {'V', 'I', 'B', 'E', 'B', 'I', 'N', '1'});
  vb_i32(b, nx);
  vb_i32(b, ny);
  vb_i32(b, nz);
  vb_i32(b, 0);
  vb_f64(b, time);
  vb_i32(b, 1 + NSPECIES);
  vb_i32(b, nz);
  vb_name(b, "__restart_info__");
  vb_f64(b, time);
  vb_f64(b, (double)step);
  std::vector<double> h;
  for (int q = 0; q < NSPECIES; ++q) {
    h.resize(storage_count(m, q));
    if (int rc = vibe_gb300_get_field(m, q, h.data())) return rc;
    vb_name(b, kVbName[q]);
    const int ni = nx + (q == U), nj = ny + (q == V), nk = nz + (q == W);
    for (int k = 0; k < nk; ++k)
      for (int j = 0; j < nj; ++j)
        for (int i = 0; i < ni; ++i) vb_f64(b, h[soff(m->nsx[q], m->nsy[q], i, j, k)]);
  }
  std::FILE* f = std::fopen(path, "wb");
  if (!f) return fail(VIBE_GB300_EBADARG, std::string("cannot write ") + path);
  const bool ok = std::fwrite(b.data(), 1, b.size(), f) == b.size();
  if (std::fclose(f) != 0 || !ok) return fail(VIBE_GB300_EDEVICE, std::string("write failed: ") + path);
  return 0;
}

int vibe_gb300_read_restart(vibe_gb300_model* m, const char* path, double* time, int* step) {
  if (!m || !path) return fail(VIBE_GB300_EBADARG, "bad argument");
  std::FILE* f = std::fopen(path, "rb");
  if (!f) return fail(VIBE_GB300_EBADARG, std::string("cannot read ") + path);
  std::vector<unsigned char> b;
  unsigned char chunk[1 << 16];
  size_t got;
  while ((got = std::fread(chunk, 1, sizeof chunk, f)) > 0) b.insert(b.end(), chunk, chunk + got);
  std::fclose(f);
  if (b.size() < 40 || std::memcmp(b.data(), "VIBEBIN1", 8) != 0) return fail(VIBE_GB300_EBADARG, "not a .vibebin file");
  const int nx = (int)rd_u32(&b[8]), ny = (int)rd_u32(&b[12]), nz = (int)rd_u32(&b[16]);
  const int nvars = (int)rd_u32(&b[32]);
  if (nx != m->d.nx || ny != m->d.ny || nz != m->d.nz)
    return fail(VIBE_GB300_EBADARG, "restart grid differs from the model's");
  // start from the current state so points the file does not hold (halo,
  // ghost lines, species not in the file) keep their values
  std::vector<std::vector<double>> st(NSPECIES);
  const double* ptrs[NSPECIES] = {};
  double rinfo[2] = {0.0, 0.0};
  size_t at = 40;
  for (int v = 0; v < nvars; ++v) {
    if (at + 32 > b.size()) return fail(VIBE_GB300_EBADARG, "truncated .vibebin file");
    char nm[33] = {};
    std::memcpy(nm, &b[at], 32);
    at += 32;
    const std::string name(nm);
    if (name == "__restart_info__") {
      if (at + 16 > b.size()) return fail(VIBE_GB300_EBADARG, "truncated .vibebin file");
      rinfo[0] = rd_f64(&b[at]);
      rinfo[1] = rd_f64(&b[at + 8]);
      at += 16;
      continue;
    }
    const int sg = vb_stagger(name);
    const int ni = nx + (sg == 1), nj = ny + (sg == 2), nk = nz + (sg == 3);
    const size_t cnt = (size_t)ni * nj * nk;
    if (at + 8 * cnt > b.size()) return fail(VIBE_GB300_EBADARG, "truncated .vibebin file");
    int q = -1;
    for (int s = 0; s < NSPECIES; ++s)
      if (name == kVbName[s]) q = s;
    if (q >= 0) {
      st[q].resize(storage_count(m, q));
      if (int rc = vibe_gb300_get_field(m, q, st[q].data())) return rc;
      size_t e = at;
      for (int k = 0; k < nk; ++k)
        for (int j = 0; j < nj; ++j)
          for (int i = 0; i < ni; ++i, e += 8) st[q][soff(m->nsx[q], m->nsy[q], i, j, k)] = rd_f64(&b[e]);
      ptrs[q] = st[q].data();
    }
    at += 8 * cnt;
  }
  if (int rc = vibe_gb300_set_state(m, ptrs, NSPECIES)) return rc;
  CUDA_OK(cudaStreamSynchronize(m->stream));
  if (time) *time = rinfo[0];
  if (step) *step = (int)std::llround(rinfo[1]);
  return 0;
}

// ---- global energy and mass budget (dyn::energy_budget,
// src/dyn/diagnostics.cpp:255-277) in FP64 on the device: per cell with
// dv = dx dy ((H - zs)/H) dzeta(k) H and z = zs + zeta(k + 1/2) (H - zs),
// mass += rho dv, kinetic += 0.5 rho |u_c|^2 dv (face averages), internal +=
// rho cv theta pi dv, potential += rho g z dv, latent += rho Lv max(qv, 0) dv.
// Each thread sums with Neumaier compensation, blocks merge their partials in
// shared memory and one block merges the blocks in order (deterministic).
}  // extern "C"

namespace {
constexpr int kBudgetBlocks = 304, kBudgetThreads = 256;
struct StatePtrs {
  const double* f[NSPECIES];
};
constexpr double kLatentVap = 2.501e6;  // constants.hpp:29

struct Comp {
  double s = 0.0, c = 0.0;
  __device__ void add(double x) {
    const double t = s + x;
    if (fabs(s) >= fabs(x)) c += (s - t) + x;
    else c += (x - t) + s;
    s = t;
  }
  __device__ void merge(const Comp& o) {
    add(o.s);
    c += o.c;
  }
};

__device__ void budget_block_merge(Comp (&v)[5], double* out) {
  __shared__ double sh[kBudgetThreads][10];
  for (int q = 0; q < 5; ++q) {
    sh[threadIdx.x][2 * q] = v[q].s;
    sh[threadIdx.x][2 * q + 1] = v[q].c;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    Comp r[5];
    for (int t = 0; t < (int)blockDim.x; ++t)
      for (int q = 0; q < 5; ++q) {
        Comp o;
        o.s = sh[t][2 * q];
        o.c = sh[t][2 * q + 1];
        r[q].merge(o);
      }
    for (int q = 0; q < 5; ++q) {
      out[2 * q] = r[q].s;
      out[2 * q + 1] = r[q].c;
    }
  }
}

__global__ void k_budget(Dims d, double dx, double dy, double ztop, const double* __restrict__ scale,
                         const double* __restrict__ dzeta, const double* __restrict__ zc, StatePtrs s,
                         double* __restrict__ part) {
  Comp v[5];  // mass, kinetic, internal, potential, latent
  const size_t ncol = (size_t)d.nx * d.ny, n = ncol * d.nz;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(e / ncol);
    const size_t col = e % ncol;
    const int j = (int)(col / d.nx), i = (int)(col % d.nx);
    const size_t c = d.idx(i, j, k);
    const double sc = scale[col], zs = ztop - sc;
    const double dv = dx * dy * (sc / ztop) * dzeta[k] * ztop;
    const double rho = s.f[RHO][c];
    const double uc = 0.5 * (s.f[U][c] + s.f[U][c + 1]);
    const double vc = 0.5 * (s.f[V][c] + s.f[V][c + d.P]);
    const double wc = 0.5 * (s.f[W][c] + s.f[W][c + d.plane]);
    const double T = s.f[THETA][c] * s.f[PI][c];
    const double z = zs + zc[k] * sc;
    v[0].add(rho * dv);
    v[1].add(0.5 * rho * (uc * uc + vc * vc + wc * wc) * dv);
    v[2].add(rho * kCv * T * dv);
    v[3].add(rho * kG * z * dv);
    v[4].add(rho * kLatentVap * fmax(s.f[QV][c], 0.0) * dv);
  }
  budget_block_merge(v, part + (size_t)blockIdx.x * 10);
}

__global__ void k_budget_final(const double* __restrict__ part, int nb, double* __restrict__ out) {
  Comp v[5];
  for (int b = threadIdx.x; b < nb; b += blockDim.x)
    for (int q = 0; q < 5; ++q) {
      Comp o;
      o.s = part[(size_t)b * 10 + 2 * q];
      o.c = part[(size_t)b * 10 + 2 * q + 1];
      v[q].merge(o);
    }
  budget_block_merge(v, out);
}
}  // namespace

extern "C" {

int vibe_gb300_energy_budget(vibe_gb300_model* m, double* out6) {
  if (!m || !out6) return fail(VIBE_GB300_EBADARG, "bad argument");
  const int nz = m->d.nz;
  // zeta at the level centres (Grid::z_center, geometry.hpp:135-137, with
  // zeta_at's half-level branch, geometry.cpp:20-31)
  std::vector<double> zc(nz);
  for (int k = 0; k < nz; ++k) zc[k] = 0.5 * (m->hs.zeta[k] + m->hs.zeta[k + 1]);
  double* buf = nullptr;
  CUDA_OK(cudaMallocAsync((void**)&buf, ((size_t)nz + (size_t)kBudgetBlocks * 10 + 10) * sizeof(double), m->stream));
  double* dzc = buf;
  double* part = buf + nz;
  double* dout = part + (size_t)kBudgetBlocks * 10;
  CUDA_OK(cudaMemcpyAsync(dzc, zc.data(), nz * sizeof(double), cudaMemcpyHostToDevice, m->stream));
  StatePtrs sp;
  for (int q = 0; q < NSPECIES; ++q) sp.f[q] = m->S[m->cur][q];
  k_budget<<<kBudgetBlocks, kBudgetThreads, 0, m->stream>>>(m->d, m->met.dx, m->met.dy, m->met.z_top, m->met.scale,
                                                             m->met.dzeta, dzc, sp, part);
  k_budget_final<<<1, kBudgetThreads, 0, m->stream>>>(part, kBudgetBlocks, dout);
  double r[10];
  CUDA_OK(cudaMemcpyAsync(r, dout, sizeof r, cudaMemcpyDeviceToHost, m->stream));
  CUDA_OK(cudaFreeAsync(buf, m->stream));
  CUDA_OK(cudaStreamSynchronize(m->stream));
  const double mass = r[0] + r[1], ke = r[2] + r[3], ie = r[4] + r[5], pe = r[6] + r[7], le = r[8] + r[9];
  out6[0] = ke;
  out6[1] = ie;
  out6[2] = pe;
  out6[3] = le;
  out6[4] = ke + ie + pe + le;
  out6[5] = mass;
  return 0;
}

int vibe_gb300_snapshot(vibe_gb300_model* m, int op) {
  if (!m || op < 0 || op > 1) return fail(VIBE_GB300_EBADARG, "bad argument");
  const size_t n = m->d.plane * (size_t)(m->d.nz + 1);
  if (op == 0) {
    if (!m->snap[0])
      for (int q = 0; q < NSPECIES; ++q)
        if (int rc = dalloc(m, &m->snap[q], n)) return rc;
    for (int q = 0; q < NSPECIES; ++q)
      CUDA_OK(cudaMemcpyAsync(m->snap[q], m->S[m->cur][q], n * sizeof(double), cudaMemcpyDeviceToDevice, m->stream));
    m->has_snap = true;
    return 0;
  }
  if (!m->has_snap) return fail(VIBE_GB300_EBADARG, "no snapshot saved");
  for (int q = 0; q < NSPECIES; ++q)
    CUDA_OK(cudaMemcpyAsync(m->S[m->cur][q], m->snap[q], n * sizeof(double), cudaMemcpyDeviceToDevice, m->stream));
  return sync_working(m);
}

int vibe_gb300_sponge(vibe_gb300_model* m, double dt) {
  if (!m) return fail(VIBE_GB300_EBADARG, "bad argument");
  int kmin = m->d.nz + 1;
  for (int k = 0; k < m->d.nz; ++k)
    if (m->hs.sponge[k] > 0.0) { kmin = k; break; }
  m->f64->sponge(m->d, m->met, m->S[m->cur], kmin, dt, m->stream);
  if (int rc = sync_working(m)) return rc;
  CUDA_OK(cudaGetLastError());
  return read_status(m);
}

// SemiImplicitIntegrator::step (src/time/semi_implicit.cpp:167-226) as the
// reference's code computes it (O-SI). The shipped step solves for pi' and
// writes the solution with update_from_pressure into its local copy
// s_explicit, which it then drops; that copy has no effect on the state and
// is not formed here. No physics driver; the RA filter is off (default).
int vibe_gb300_si_step(vibe_gb300_model* m, double dt, int kind, int max_iter, double tol, int* iterations,
                       double* residual, double* pi_new) {
  if (!m || !(dt > 0.0) || kind < 0 || kind > 4 || max_iter < 1) return fail(VIBE_GB300_EBADARG, "bad argument");
  if (m->precision == VIBE_GB300_MIXED)
    return fail(VIBE_GB300_EUNSUPPORTED, "the semi-implicit step runs on the FP64 precisions");
  const Dims& d = m->d;
  const size_t n = (size_t)d.nx * d.ny * d.nz;
  if (!m->hz || m->hz_kind != kind || m->hz_max_iter != max_iter || m->hz_tol != tol) {
    if (m->hz) vibe_helmholtz_destroy(m->hz);
    m->hz = nullptr;
    std::vector<double> dz(d.nz);
    for (int k = 0; k < d.nz; ++k) dz[k] = m->hs.zeta[k + 1] - m->hs.zeta[k];
    if (vibe_helmholtz_create(kind, d.nx, d.ny, d.nz, m->su.dx, m->su.dy, m->su.z_top, dz.data(), m->hs.zs.data(),
                              max_iter, tol, &m->hz) != VIBE_C_OK)
      return fail(VIBE_GB300_EDEVICE, std::string("helmholtz solver: ") + vibe_helmholtz_last_error());
    m->hz_kind = kind;
    m->hz_max_iter = max_iter;
    m->hz_tol = tol;
    if (!m->hz_a) {
      int rc = dalloc(m, &m->hz_a, n);
      rc = rc ? rc : dalloc(m, &m->hz_b, n);
      rc = rc ? rc : dalloc(m, &m->hz_f, n);
      rc = rc ? rc : dalloc(m, &m->hz_x, n);
      if (rc) return rc;
    }
  }
  double* const* st = m->S[m->cur];
  m->f64->slow_tendency(d, m->met, m->fl, st, m->tend, m->scratch, m->wface, m->stream);
  si_assemble(d, m->met, st, m->tend, dt, m->hz_a, m->hz_b, m->hz_f, m->stream);
  CUDA_OK(cudaGetLastError());
  if (!m->hz_ev[0]) {
    CUDA_OK(cudaEventCreate(&m->hz_ev[0]));
    CUDA_OK(cudaEventCreate(&m->hz_ev[1]));
  }
  CUDA_OK(cudaEventRecord(m->hz_ev[0], m->stream));
  if (vibe_helmholtz_set_coefficients_dev(m->hz, m->hz_a, m->hz_b, (vibe_stream_t)m->stream) != VIBE_C_OK)
    return fail(VIBE_GB300_EDEVICE, std::string("helmholtz coefficients: ") + vibe_helmholtz_last_error());
  const int hrc = vibe_helmholtz_solve_dev(m->hz, m->hz_f, m->hz_x, (vibe_stream_t)m->stream);
  CUDA_OK(cudaEventRecord(m->hz_ev[1], m->stream));
  CUDA_OK(cudaEventSynchronize(m->hz_ev[1]));
  {
    float ms = 0.f;
    CUDA_OK(cudaEventElapsedTime(&ms, m->hz_ev[0], m->hz_ev[1]));
    m->hz_ms = ms;
  }
  m->hz_iterations = vibe_helmholtz_iterations(m->hz);
  m->hz_residual = vibe_helmholtz_residual(m->hz);
  if (iterations) *iterations = m->hz_iterations;
  if (residual) *residual = m->hz_residual;
  if (hrc == VIBE_C_ERR_SINGULAR) return fail(VIBE_GB300_ESINGULAR, "singular Helmholtz column");
  if (hrc != VIBE_C_OK) return fail(VIBE_GB300_EDEVICE, std::string("helmholtz solve: ") + vibe_helmholtz_last_error());
  if (pi_new) {
    si_to_cells(d, m->hz_x, m->tmp[PI], m->stream);
    unpack<double>(d, m->nsx[RHO], m->nsy[RHO], m->nsz[RHO], d.nx, d.ny, d.nz, m->tmp[PI],
                                          m->d_stage_in, m->stream);
    CUDA_OK(cudaMemcpyAsync(pi_new, m->d_stage_in, storage_count(m, RHO) * sizeof(double), cudaMemcpyDeviceToHost,
                            m->stream));
  }
  const int upd[] = {THETA, QV, RHO, QC, QR, QI, QS, QG};
  for (int q : upd) si_cells_add_scaled(d, st[q], m->tend[q], dt, m->stream);
  int kmin = d.nz + 1;
  for (int k = 0; k < d.nz; ++k)
    if (m->hs.sponge[k] > 0.0) { kmin = k; break; }
  m->f64->sponge(d, m->met, st, kmin, dt, m->stream);
  m->f64->nonfinite(d, st, m->d_err, m->stream);
  CUDA_OK(cudaGetLastError());
  return read_status(m);
}

int vibe_gb300_set_graph(vibe_gb300_model* m, int enable) {
  if (!m) return fail(VIBE_GB300_EBADARG, "bad argument");
  if (m->stream) cudaStreamSynchronize(m->stream);
  drop_graphs(m);
  m->use_graph = enable != 0;
  return 0;
}

int vibe_gb300_cfl(vibe_gb300_model* m, double dt, double dtau, double* adv_cfl, double* max_sound_speed,
                   double* acoustic_cfl) {
  if (!m) return fail(VIBE_GB300_EBADARG, "bad argument");
  unsigned long long* dv = nullptr;
  CUDA_OK(cudaMallocAsync((void**)&dv, 4 * sizeof(unsigned long long), m->stream));
  diag_cfl(m->d, m->met, m->S[m->cur], dt, dtau, dv, m->stream);
  unsigned long long hv[4] = {0, 0, 0, 0};
  CUDA_OK(cudaMemcpyAsync(hv, dv, sizeof(hv), cudaMemcpyDeviceToHost, m->stream));
  CUDA_OK(cudaFreeAsync(dv, m->stream));
  CUDA_OK(cudaStreamSynchronize(m->stream));
  double r[4];
  for (int q = 0; q < 4; ++q) std::memcpy(&r[q], &hv[q], sizeof(double));
  if (adv_cfl) *adv_cfl = r[0];
  if (max_sound_speed) *max_sound_speed = r[1];
  if (acoustic_cfl) *acoustic_cfl = r[2];
  m->cfl_rate = r[3];
  return 0;
}

// RungeKutta3Integrator::max_stable_dt (runge_kutta.cpp:121-140):
// min(0.8 / cfl_number(s, 1), 2 / (max sound speed * max(1/dx + 1/dy + 1/dz)))
int vibe_gb300_max_stable_dt(vibe_gb300_model* m, double* dt_out) {
  if (!m || !dt_out) return fail(VIBE_GB300_EBADARG, "bad argument");
  double adv = 0.0, cs = 0.0;
  if (int rc = vibe_gb300_cfl(m, 1.0, 1.0, &adv, &cs, nullptr)) return rc;
  const double rate = cs * m->cfl_rate;
  const double dt_adv = (adv > 0.0) ? 0.8 / adv : 1e9;
  const double dt_ac = (rate > 0.0) ? 2.0 / rate : 1e9;
  *dt_out = std::min(dt_adv, dt_ac);
  return 0;
}

int vibe_gb300_si_stats(const vibe_gb300_model* m, int* iterations, double* residual, double* solve_ms) {
  if (!m) return fail(VIBE_GB300_EBADARG, "bad argument");
  if (iterations) *iterations = m->hz_iterations;
  if (residual) *residual = m->hz_residual;
  if (solve_ms) *solve_ms = m->hz_ms;
  return 0;
}

// ---- groups: several mixed models advanced together, one launch per kernel
// for all of them (work-list over the domains' blocks), each step replayed as
// a CUDA graph per state parity.
}  // extern "C"

struct vibe_gb300_group {
  std::vector<vibe_gb300_model*> ms;
  cudaStream_t stream = nullptr;
  unsigned *d_err = nullptr, *h_err = nullptr;
  MixedBatch* batch[2] = {nullptr, nullptr};
  cudaGraphExec_t g[2] = {nullptr, nullptr};
  double dt = -1.0;
  int nsub = -1;
};

namespace {
void group_drop(vibe_gb300_group* g) {
  for (int p = 0; p < 2; ++p) {
    if (g->g[p]) cudaGraphExecDestroy(g->g[p]);
    g->g[p] = nullptr;
    mixed_batch_destroy(g->batch[p]);
    g->batch[p] = nullptr;
  }
}
}  // namespace

extern "C" {

int vibe_gb300_group_create(vibe_gb300_model* const* models, int n, vibe_gb300_group** out) {
  if (!models || n < 1 || !out) return fail(VIBE_GB300_EBADARG, "bad argument");
  for (int q = 0; q < n; ++q) {
    vibe_gb300_model* m = models[q];
    if (!m || m->precision != VIBE_GB300_MIXED || m->fl.acoustic_mode != 2)
      return fail(VIBE_GB300_EUNSUPPORTED, "a group holds mixed-precision models with acoustic_mode 2");
    if (m->phys_fn)  // the work-list launches have no physics call
      return fail(VIBE_GB300_EUNSUPPORTED, "group members cannot have a physics package installed");
    if (m->d.nz != models[0]->d.nz || m->fl.moist != models[0]->fl.moist ||
        m->fl.weno_scalars != models[0]->fl.weno_scalars || m->fl.advection != models[0]->fl.advection ||
        m->fl.weno_advective != models[0]->fl.weno_advective || m->fl.coriolis != models[0]->fl.coriolis ||
        m->fl.div_damp != models[0]->fl.div_damp || m->fl.hevi_beta != models[0]->fl.hevi_beta)
      return fail(VIBE_GB300_EUNSUPPORTED, "group members need the same nz and numerics flags");
  }
  auto* g = new vibe_gb300_group();
  g->ms.assign(models, models + n);
  if (cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMalloc(&g->d_err, sizeof(unsigned)) != cudaSuccess || cudaMallocHost(&g->h_err, sizeof(unsigned)) != cudaSuccess ||
      cudaMemset(g->d_err, 0, sizeof(unsigned)) != cudaSuccess) {
    vibe_gb300_group_destroy(g);
    return fail(VIBE_GB300_EDEVICE, "group allocation failed");
  }
  *out = g;
  return 0;
}

void vibe_gb300_group_destroy(vibe_gb300_group* g) {
  if (!g) return;
  if (g->stream) cudaStreamSynchronize(g->stream);
  group_drop(g);
  cudaFree(g->d_err);
  if (g->h_err) cudaFreeHost(g->h_err);
  if (g->stream) cudaStreamDestroy(g->stream);
  delete g;
}

}  // extern "C"

namespace {
// (re)build the work lists of a group for (dt, n_sub); members idle
int group_prepare(vibe_gb300_group* g, double dt, int n_sub) {
  const int parity0 = g->ms[0]->cur;
  for (auto* m : g->ms) {
    if (m->cur != parity0) return fail(VIBE_GB300_EUNSUPPORTED, "group members must share the state parity");
    CUDA_OK(cudaStreamSynchronize(m->stream));  // nothing of theirs in flight
  }
  // A member stepped alone, or run through a substep / TL-AD entry point, may
  // have rebuilt its per-model dt tables (HEVI LU factors, sponge weights)
  // for another dt since the group last ran: put them back for the group's
  // (dt, n_sub) on every call. The tables are rewritten in place (same device
  // pointers), so the work lists and captured graphs below stay valid; the
  // call is free when a member's tables already match.
  CUDA_OK(cudaStreamSynchronize(g->stream));
  for (auto* m : g->ms)
    if (int rc = configure_dt(m, dt, n_sub)) return rc;
  if (g->dt == dt && g->nsub == n_sub) return 0;
  group_drop(g);
  for (int p = 0; p < 2; ++p) {
    std::vector<MixedDomain> doms;
    for (auto* m : g->ms) {
      MixedDomain md;
      md.d = m->d;
      md.t = m->tab;
      md.lu = m->d_lu;
      md.W0 = m->W0;
      md.WSt0 = m->WSt[0];
      md.WSt1 = m->WSt[1];
      md.WA = m->WA;
      md.WB = m->WB;
      md.WR = m->WR;
      md.S0 = m->S[p];
      md.S1 = m->S[1 - p];
      doms.push_back(md);
    }
    g->batch[p] = mixed_batch_build(doms, g->ms[0]->fl, dt, n_sub, g->d_err);
    if (!g->batch[p]) return fail(VIBE_GB300_EDEVICE, "group launch set-up failed");
  }
  g->dt = dt;
  g->nsub = n_sub;
  return 0;
}

// wait for the group's stream, then read and clear its error word
int group_check(vibe_gb300_group* g) {
  CUDA_OK(cudaMemcpyAsync(g->h_err, g->d_err, sizeof(unsigned), cudaMemcpyDeviceToHost, g->stream));
  CUDA_OK(cudaStreamSynchronize(g->stream));
  const unsigned e = *g->h_err;
  CUDA_OK(cudaMemsetAsync(g->d_err, 0, sizeof(unsigned), g->stream));
  CUDA_OK(cudaStreamSynchronize(g->stream));
  if (e & kErrWaitTimeout) return fail(VIBE_GB300_EDEVICE, "a TMA box of the stage kernel did not arrive (bounded wait)");
  if (e & kErrNonFinite) return fail(VIBE_GB300_ENONFINITE, "non-finite value in a group member's state");
  return 0;
}
}  // namespace

extern "C" {

int vibe_gb300_group_step(vibe_gb300_group* g, double dt, int n_sub_in, int n_steps) {
  if (!g || !(dt > 0.0) || n_steps < 0) return fail(VIBE_GB300_EBADARG, "bad argument");
  const int n_sub = n_sub_in > 1 ? n_sub_in : 1;
  if (int rc = group_prepare(g, dt, n_sub)) return rc;
  for (int step = 0; step < n_steps; ++step) {
    const int p = g->ms[0]->cur;
    if (!g->g[p]) {
      cudaGraph_t gr = nullptr;
      CUDA_OK(cudaStreamBeginCapture(g->stream, cudaStreamCaptureModeThreadLocal));
      mixed_batch_enqueue(g->batch[p], g->stream);
      const cudaError_t e = cudaStreamEndCapture(g->stream, &gr);
      CUDA_OK(e);
      const cudaError_t ei = cudaGraphInstantiate(&g->g[p], gr, 0);
      cudaGraphDestroy(gr);
      CUDA_OK(ei);
    }
    CUDA_OK(cudaGraphLaunch(g->g[p], g->stream));
    for (auto* m : g->ms) m->cur = 1 - m->cur;
  }
  return group_check(g);
}

int vibe_gb300_group_launches_per_step(const vibe_gb300_group* g) {
  return (g && g->batch[0]) ? mixed_batch_launches(g->batch[0]) : 0;
}

vibe_stream_t vibe_gb300_group_stream(vibe_gb300_group* g) { return g ? (vibe_stream_t)g->stream : nullptr; }

// ---- nested sets: parents advanced by one group with dt, their two-way
// nests by another group with r sub-steps of dt/r (the parent step; the
// parent state interpolated into a boundary buffer of every nest
// (Nest::interpolate_from_parent); r nest sub-steps, each followed by the
// Davies relaxation towards that buffer (apply_lateral_boundary); the nests
// restricted back onto their parents (restrict_to_parent, two-way)). One
// parent step is one CUDA graph, captured once per pair of state parities.
}  // extern "C"

struct vibe_gb300_nested {
  std::vector<vibe_gb300_model*> parents, children;
  std::vector<int> parent_of;
  std::vector<vibe_nest_placement> pl_interp, pl_restrict;
  vibe_gb300_group* gp = nullptr;
  vibe_gb300_group* gc = nullptr;
  std::vector<std::vector<double*>> buf;  // per nest: boundary buffer (FP64, model layout)
  std::vector<std::vector<double>> davies;  // per nest: the Davies weights of its zone
  std::vector<void*> allocs;
  cudaStream_t stream = nullptr;
  cudaGraphExec_t graph[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};  // [parent parity][nest parity]
  int nvars = 7;
  int launches = 0;
};

namespace {
// op 0: parent S[pp] -> boundary buffer; 1: nest S[cp] -> parent S[pp];
// 2: Davies blend of nest S[cp] with the buffer
int nested_transfer(vibe_gb300_nested* n, int op, int c, int pp, int cp) {
  vibe_gb300_model* ch = n->children[c];
  vibe_gb300_model* pa = n->parents[n->parent_of[c]];
  const vibe_nest_placement* pl = (op == 1) ? &n->pl_restrict[c] : &n->pl_interp[c];
  const double* pin[NSPECIES];
  double* pout[NSPECIES];
  const double* cin[NSPECIES];
  double* cout[NSPECIES];
  for (int q = 0; q < n->nvars; ++q) {
    pin[q] = pa->S[pp][q];
    pout[q] = pa->S[pp][q];
    cin[q] = (op == 2) ? n->buf[c][q] : ch->S[cp][q];
    cout[q] = (op == 0) ? n->buf[c][q] : ch->S[cp][q];
  }
  // (the boundary buffer is read only in the Davies zone: op 0 fills just that)
  const int rc = nest_model_layout(op, pl, n->nvars, pa->d.nx, pa->d.ny, pa->d.nz, pin, pa->d.P, pa->d.plane,
                                   ch->d.nx, ch->d.ny, ch->d.nz, cin, op == 1 ? pout : cout, ch->d.P, ch->d.plane,
                                   n->stream, op == 0);
  ++n->launches;
  return rc == VIBE_C_OK ? 0 : fail(VIBE_GB300_EDEVICE, "nest transfer failed");
}

// The FP32 working copy after a transfer changed the FP64 state, on the
// points it changed: a nest's Davies frame (in the relaxation's own launch),
// the restriction box of a parent after the feedback. Elsewhere the working
// copy the finish kernel wrote stands, as after any step.
int relax_nest(vibe_gb300_nested* n, int c, int parity) {
  vibe_gb300_model* m = n->children[c];
  ++n->launches;
  if (mixed_nest_relax(m->d, m->tab, m->S[parity], n->buf[c].data(), n->nvars, n->davies[c].data(),
                       n->pl_interp[c].boundary_zone, working_targets(m, m->W0), n->stream))
    return fail(VIBE_GB300_EBADARG, "bad Davies zone");
  return 0;
}
void to_working_box(vibe_gb300_nested* n, int c, int parity) {
  vibe_gb300_model* m = n->parents[n->parent_of[c]];
  const vibe_nest_placement& q = n->pl_restrict[c];
  mixed_to_working_region(m->d, m->tab, m->S[parity], working_targets(m, m->W0), q.i0, q.j0, q.iext, q.jext,
                          n->stream);
  ++n->launches;
}

// one parent step from parities (pp, cp), enqueued on the nested stream
int nested_enqueue(vibe_gb300_nested* n, int pp, int cp, int r) {
  n->launches = mixed_batch_launches(n->gp->batch[pp]) + r * mixed_batch_launches(n->gc->batch[0]);
  mixed_batch_enqueue(n->gp->batch[pp], n->stream);
  const int pn = 1 - pp;
  const int nc = (int)n->children.size();
  for (int c = 0; c < nc; ++c)
    if (int rc = nested_transfer(n, 0, c, pn, cp)) return rc;
  int cc = cp;
  for (int sub = 0; sub < r; ++sub) {
    mixed_batch_enqueue(n->gc->batch[cc], n->stream);
    cc = 1 - cc;
    for (int c = 0; c < nc; ++c)
      if (int rc = relax_nest(n, c, cc)) return rc;
  }
  for (int c = 0; c < nc; ++c)
    if (int rc = nested_transfer(n, 1, c, pn, cc)) return rc;
  for (int c = 0; c < nc; ++c) to_working_box(n, c, pn);
  return 0;
}

void nested_drop(vibe_gb300_nested* n) {
  for (auto& row : n->graph)
    for (auto& g : row) {
      if (g) cudaGraphExecDestroy(g);
      g = nullptr;
    }
}
}  // namespace

extern "C" {

int vibe_gb300_nested_create(vibe_gb300_model* const* parents, int np, vibe_gb300_model* const* children, int nc,
                             const int* parent_of, const vibe_nest_placement* interp_pl,
                             const vibe_nest_placement* restrict_pl, vibe_gb300_nested** out) {
  if (!parents || np < 1 || !children || nc < 1 || !parent_of || !interp_pl || !restrict_pl || !out)
    return fail(VIBE_GB300_EBADARG, "bad argument");
  for (int c = 0; c < nc; ++c) {
    if (parent_of[c] < 0 || parent_of[c] >= np) return fail(VIBE_GB300_EBADARG, "parent index out of range");
    if (interp_pl[c].ratio != interp_pl[0].ratio || restrict_pl[c].ratio != interp_pl[0].ratio || interp_pl[0].ratio < 2)
      return fail(VIBE_GB300_EBADARG, "every nest needs the same ratio r >= 2 (time sub-cycling)");
    const vibe_gb300_model* pa = parents[parent_of[c]];
    if (children[c]->d.nz != pa->d.nz) return fail(VIBE_GB300_EBADARG, "nests share their parent's levels");
    const vibe_nest_placement& q = restrict_pl[c];
    if (q.i0 < 0 || q.j0 < 0 || q.iext < 0 || q.jext < 0 || q.i0 + q.iext > pa->d.nx + 1 ||
        q.j0 + q.jext > pa->d.ny + 1)
      return fail(VIBE_GB300_EBADARG, "restriction box outside the parent");
    if (interp_pl[c].boundary_zone < 1 || interp_pl[c].boundary_zone > 64)
      return fail(VIBE_GB300_EBADARG, "boundary zone must be 1..64 points");
    if (children[c]->precision != VIBE_GB300_MIXED || pa->precision != VIBE_GB300_MIXED)
      return fail(VIBE_GB300_EBADARG, "nested sets step mixed-precision models");
  }
  auto* n = new vibe_gb300_nested();
  n->parents.assign(parents, parents + np);
  n->children.assign(children, children + nc);
  n->parent_of.assign(parent_of, parent_of + nc);
  n->pl_interp.assign(interp_pl, interp_pl + nc);
  n->pl_restrict.assign(restrict_pl, restrict_pl + nc);
  n->nvars = parents[0]->fl.moist ? NSPECIES : QV + 1;
  int rc = vibe_gb300_group_create(parents, np, &n->gp);
  rc = rc ? rc : vibe_gb300_group_create(children, nc, &n->gc);
  if (!rc && cudaStreamCreateWithFlags(&n->stream, cudaStreamNonBlocking) != cudaSuccess)
    rc = fail(VIBE_GB300_EDEVICE, "stream");
  for (int c = 0; c < nc && !rc; ++c) {
    std::vector<double*> b(NSPECIES, nullptr);
    const size_t cnt = children[c]->d.plane * (size_t)(children[c]->d.nz + 1);
    for (int q = 0; q < n->nvars && !rc; ++q) {
      void* p = nullptr;
      if (cudaMalloc(&p, cnt * sizeof(double)) != cudaSuccess) {
        rc = fail(VIBE_GB300_EDEVICE, "buffer allocation");
      } else {
        n->allocs.push_back(p);
        b[q] = (double*)p;
        if (cudaMemset(p, 0, cnt * sizeof(double)) != cudaSuccess) rc = fail(VIBE_GB300_EDEVICE, "memset");
      }
    }
    n->buf.push_back(b);
    std::vector<double> dw(64, 0.0);
    if (!rc && vibe_davies_profile(interp_pl[c].boundary_zone, 1.0, dw.data()) != 0)
      rc = fail(VIBE_GB300_EBADARG, "Davies profile");
    n->davies.push_back(dw);
  }
  if (rc) {
    vibe_gb300_nested_destroy(n);
    return rc;
  }
  *out = n;
  return 0;
}

void vibe_gb300_nested_destroy(vibe_gb300_nested* n) {
  if (!n) return;
  if (n->stream) cudaStreamSynchronize(n->stream);
  nested_drop(n);
  vibe_gb300_group_destroy(n->gp);
  vibe_gb300_group_destroy(n->gc);
  for (void* p : n->allocs) cudaFree(p);
  if (n->stream) cudaStreamDestroy(n->stream);
  delete n;
}

int vibe_gb300_nested_launch(vibe_gb300_nested* n, double dt, int n_sub_in, int n_steps) {
  if (!n || !(dt > 0.0) || n_steps < 0) return fail(VIBE_GB300_EBADARG, "bad argument");
  const int n_sub = n_sub_in > 1 ? n_sub_in : 1;
  const int r = n->pl_interp[0].ratio;
  const double dtc = dt / r;
  const bool rebuild = n->gp->dt != dt || n->gp->nsub != n_sub || n->gc->dt != dtc || n->gc->nsub != n_sub;
  if (rebuild) {
    CUDA_OK(cudaStreamSynchronize(n->stream));
    nested_drop(n);
  }
  if (int rc = group_prepare(n->gp, dt, n_sub)) return rc;
  if (int rc = group_prepare(n->gc, dtc, n_sub)) return rc;
  for (int step = 0; step < n_steps; ++step) {
    const int pp = n->parents[0]->cur, cp = n->children[0]->cur;
    for (auto* m : n->parents)
      if (m->cur != pp) return fail(VIBE_GB300_EUNSUPPORTED, "parents must share the state parity");
    for (auto* m : n->children)
      if (m->cur != cp) return fail(VIBE_GB300_EUNSUPPORTED, "nests must share the state parity");
    if (!n->graph[pp][cp]) {
      cudaGraph_t gr = nullptr;
      CUDA_OK(cudaStreamBeginCapture(n->stream, cudaStreamCaptureModeThreadLocal));
      const int erc = nested_enqueue(n, pp, cp, r);
      const cudaError_t e = cudaStreamEndCapture(n->stream, &gr);
      if (erc) {
        if (gr) cudaGraphDestroy(gr);
        return erc;
      }
      CUDA_OK(e);
      const cudaError_t ei = cudaGraphInstantiate(&n->graph[pp][cp], gr, 0);
      cudaGraphDestroy(gr);
      CUDA_OK(ei);
    }
    CUDA_OK(cudaGraphLaunch(n->graph[pp][cp], n->stream));
    for (auto* m : n->parents) m->cur = 1 - m->cur;
    for (auto* m : n->children)
      if (r & 1) m->cur = 1 - m->cur;
  }
  CUDA_OK(cudaGetLastError());
  return 0;
}

int vibe_gb300_nested_wait(vibe_gb300_nested* n) {
  if (!n) return fail(VIBE_GB300_EBADARG, "bad argument");
  CUDA_OK(cudaStreamSynchronize(n->stream));
  const int rp = group_check(n->gp);
  const int rc = group_check(n->gc);
  return rp ? rp : rc;
}

int vibe_gb300_nested_step(vibe_gb300_nested* n, double dt, int n_sub, int n_steps) {
  if (int rc = vibe_gb300_nested_launch(n, dt, n_sub, n_steps)) return rc;
  return vibe_gb300_nested_wait(n);
}

int vibe_gb300_nested_launches_per_step(const vibe_gb300_nested* n) { return n ? n->launches : 0; }

vibe_stream_t vibe_gb300_nested_stream(vibe_gb300_nested* n) { return n ? (vibe_stream_t)n->stream : nullptr; }

// ---- assimilation windows: the TL/AD model linearised about the model's own
// trajectory, with checkpoints and recomputation (TangentLinearModel::
// propagate / record_trajectory, tangent_linear.cpp:679-716;
// AdjointModel::propagate_with_trajectory, :749-765; the Recompute
// checkpoint strategy, tangent_linear.hpp:56-61). The model state at step n
// is the linearisation point of TL/AD step n, read in place from the
// model's device buffers (same layout); every `every` steps the state is
// copied to a checkpoint; the adjoint sweep recomputes each segment's states
// from its checkpoint (double-buffered, so the recomputation of one segment
// overlaps the adjoint of the next).
}  // extern "C"

struct vibe_gb300_window {
  vibe_gb300_model* m = nullptr;
  vibe_tlad* t = nullptr;
  double dt = 0.0;
  int n_sub = 1, n_steps = 0, every = 10, tl_sub = 1;
  std::vector<std::array<double*, NSPECIES>> ckpt;
  std::vector<std::array<double*, NSPECIES>> seg[2];
  std::vector<void*> allocs;
  cudaEvent_t ev_model = nullptr, ev_seg[2] = {nullptr, nullptr}, e0 = nullptr, e1 = nullptr;
  double last_ms = 0.0;
};

namespace {
size_t state_count(const vibe_gb300_model* m) { return m->d.plane * (size_t)(m->d.nz + 1); }

int copy_state(vibe_gb300_model* m, double* const* dst, double* const* src) {
  for (int q = 0; q < NSPECIES; ++q)
    CUDA_OK(cudaMemcpyAsync(dst[q], src[q], state_count(m) * sizeof(double), cudaMemcpyDeviceToDevice, m->stream));
  return 0;
}

// checkpoint the current state; the FP32 working copy is rebuilt from it as a
// restart from the checkpoint will, so that recomputed states repeat the bits
int window_checkpoint(vibe_gb300_window* w, int c) {
  if (int rc = copy_state(w->m, w->ckpt[c].data(), w->m->S[w->m->cur])) return rc;
  return sync_working(w->m);
}
int window_restart(vibe_gb300_window* w, int c) {
  if (int rc = copy_state(w->m, w->m->S[w->m->cur], w->ckpt[c].data())) return rc;
  return sync_working(w->m);
}
int window_begin(vibe_gb300_window* w) {
  CUDA_OK(cudaEventRecord(w->e0, w->m->stream));
  return 0;
}
int window_end(vibe_gb300_window* w, cudaStream_t ts) {
  CUDA_OK(cudaEventRecord(w->ev_model, w->m->stream));
  CUDA_OK(cudaStreamWaitEvent(ts, w->ev_model, 0));
  CUDA_OK(cudaEventRecord(w->e1, ts));
  CUDA_OK(cudaStreamSynchronize(ts));
  float ms = 0.f;
  CUDA_OK(cudaEventElapsedTime(&ms, w->e0, w->e1));
  w->last_ms = ms;
  if (w->t) vgb::tlad_use_base(w->t, nullptr);
  return 0;
}

// ---- tangent-linear and adjoint of the model's own step ----------------------
// The step (runge_kutta.cpp:77-119 as this model composes it) is
//   x1 = A^n (x0 + dt/3 R(x0)),  x2 = A^n (x0 + dt/2 R(x1)),
//   x3 = A^n (x0 + dt R(x2)),     x_new = rigid(sponge(x3)),
// R the slow tendency, A one acoustic substep of the stage's dtau. A is
// affine in the state (its linear part is the substep applied to a
// perturbation with the gradient of pi itself), the sponge is affine (its
// linear part: the sponge toward a zero reference) and the rigid ground/lid
// is linear. The TL of a step needs the step's three stage inputs x0, x1,
// x2, which a step records when rec_stage is set. FP64 models: FP64 TL/AD;
// mixed models: the slow tendency's TL/AD in FP32 arithmetic and the model's
// own FP32 substep and its adjoint (perturbations stored in FP64).
int stl_supported(const vibe_gb300_model* m) {
  if (m->phys_fn) return fail(VIBE_GB300_EUNSUPPORTED, "the step's TL/AD has no physics package");
  if (m->fl.acoustic_mode == 1)
    return fail(VIBE_GB300_EUNSUPPORTED, "the reference HEVI substep (acoustic_mode 1) has no adjoint here");
  if (m->fl.div_damp > 0.0 && m->fl.div_order > 2)
    return fail(VIBE_GB300_EUNSUPPORTED, "fourth-order divergence damping has no TL/AD here");
  return 0;
}

int stl_ensure(vibe_gb300_model* m) {
  if (m->stl_zero) return 0;
  const size_t n = state_count(m);
  for (auto& st : m->stl)
    for (int q = 0; q < NSPECIES; ++q)
      if (int rc = dalloc(m, &st[q], n)) return rc;
  if (int rc = dalloc(m, &m->stl_face, 9 * n)) return rc;
  if (int rc = dalloc(m, &m->stl_cell, n)) return rc;
  if (m->precision == VIBE_GB300_FP64) {
    if (!m->lin_scr) {  // as the substep TL/AD entry points allocate them
      for (int f = 0; f < 3; ++f)
        if (int rc = dalloc(m, &m->lin_tmp[f], n)) return rc;
      if (int rc = dalloc(m, &m->lin_dh, n)) return rc;
      if (int rc = dalloc(m, &m->lin_scr, (size_t)m->d.nx * m->d.ny * (6 * (size_t)m->d.nz + 6))) return rc;
    }
  } else {
    if (!m->lin32[0][0])
      for (int b = 0; b < 2; ++b)
        for (int f = 0; f < 5; ++f)
          if (int rc = dalloc(m, &m->lin32[b][f], n)) return rc;
    if (!m->lin32_dh) {
      if (int rc = dalloc(m, &m->lin32_dh, n)) return rc;
      if (int rc = dalloc(m, &m->lin32_scr, (size_t)m->d.nx * m->d.ny * (4 * (size_t)m->d.nz + 2))) return rc;
    }
  }
  return dalloc(m, &m->stl_zero, n);  // last: it marks the set as allocated
}

// n_sub substeps of stage `stage` (or their adjoint) on the acoustic fields of x
int stl_substeps(vibe_gb300_model* m, int stage, double dtau, int n_sub, double* const* x, bool adjoint) {
  const Dims& d = m->d;
  const bool hevi = m->fl.acoustic_mode == 2;
  if (m->precision == VIBE_GB300_FP64) {
    Flags lf = m->fl;
    lf.pgf_pert = 0;  // the linear part: the gradient of the perturbation of pi
    double* tmp[NSPECIES] = {};
    tmp[W] = m->lin_tmp[0];
    tmp[RHO] = m->lin_tmp[1];
    tmp[PI] = m->lin_tmp[2];
    for (int n = 0; n < n_sub; ++n) {
      if (adjoint) {
        if (hevi) m->f64->hevi_substep_ad(d, m->met, lf, x, m->lin_dh, m->lin_scr, dtau, m->d_err, m->stream);
        else m->f64->fb_substep_ad(d, m->met, x, dtau, m->stream);
      } else {
        if (hevi) m->f64->cons_hevi_substep(d, m->met, lf, x, tmp, m->lin_scr, dtau, m->d_err, m->stream);
        else m->f64->fb_substep(d, m->met, lf, x, dtau, m->stream);
      }
    }
    CUDA_OK(cudaGetLastError());
    return 0;
  }
  const size_t n = state_count(m);
  for (int f = 0; f < 5; ++f) {
    lin_to_f32(n, x[kLinField[f]], m->lin32[0][f], m->stream);
    CUDA_OK(cudaMemcpyAsync(m->lin32[1][f], m->lin32[0][f], n * sizeof(float), cudaMemcpyDeviceToDevice, m->stream));
  }
  auto ws_lin = [&](int b) {
    WS w;
    for (int q = 0; q < NSPECIES; ++q) w.f[q] = nullptr;
    for (int f = 0; f < 5; ++f) w.f[kLinField[f]] = m->lin32[b][f];
    return w;
  };
  const float* lu = m->d_lu + (size_t)stage * 3 * d.nz;
  int cur = 0;
  for (int k = 0; k < n_sub; ++k) {
    if (hevi) {
      if (adjoint) {
        mixed_hevi_substep_ad(d, m->tab, m->fl, ws_lin(0), lu, m->lin32_dh, m->lin32_scr, (float)dtau, m->stream);
      } else {
        if (mixed_hevi_substep(d, m->tab, m->fl, ws_lin(cur), ws_lin(1 - cur), (float)dtau, lu, m->d_err, m->stream))
          return fail(VIBE_GB300_EDEVICE, "TMA descriptor creation failed (cuTensorMapEncodeTiled)");
        cur = 1 - cur;
      }
    } else if (adjoint) {
      mixed_fb_substep_ad(d, m->tab, ws_lin(0), (float)dtau, m->stream);
    } else {
      mixed_fb_substep(d, m->tab, m->fl, ws_lin(cur), ws_lin(1 - cur), (float)dtau, m->stream);
      cur = 1 - cur;
    }
  }
  for (int f = 0; f < 5; ++f) lin_to_f64(n, m->lin32[cur][f], x[kLinField[f]], m->stream);
  CUDA_OK(cudaGetLastError());
  return 0;
}

// the linear parts of the sponge and of the rigid ground and lid (both
// diagonal, so each is its own adjoint)
int stl_sponge_rigid(vibe_gb300_model* m, double dt, double* const* x) {
  Metric mz = m->met;
  mz.th0 = mz.pi0 = mz.rho0 = m->stl_zero;
  m->f64->sponge(m->d, mz, x, m->kmin, dt, m->stream);
  if (m->fl.w_rigid)
    k_rigid_w<<<dim3((m->d.nx + 31) / 32, (m->d.ny + 7) / 8), dim3(32, 8), 0, m->stream>>>(m->d, x[W]);
  CUDA_OK(cudaGetLastError());
  return 0;
}

// x: the perturbation of the step's input in, of its output out;
// base[s]: the input state of stage s of the trajectory step
int stl_step_tl(vibe_gb300_model* m, double dt, int n_sub, double* const* const* base, double* const* x) {
  const size_t n = state_count(m);
  const bool f32 = m->precision == VIBE_GB300_MIXED;
  double* const* x0 = m->stl[0];
  double* const* r = m->stl[2];
  if (int rc = copy_state(m, x0, x)) return rc;
  const double dts[3] = {dt / 3.0, dt / 2.0, dt};
  for (int st = 0; st < 3; ++st) {
    tend_tl(m->d, m->met, m->fl, base[st], st == 0 ? x0 : x, r, m->stl_face, f32, m->stream);
    for (int q = 0; q < NSPECIES; ++q) lin_axpy(n, x0[q], r[q], dts[st], x[q], m->stream);
    if (int rc = stl_substeps(m, st, dts[st] / n_sub, n_sub, x, false)) return rc;
  }
  return stl_sponge_rigid(m, dt, x);
}

// x: the bar of the step's output in, of its input out
int stl_step_ad(vibe_gb300_model* m, double dt, int n_sub, double* const* const* base, double* const* x) {
  const size_t n = state_count(m);
  const bool f32 = m->precision == VIBE_GB300_MIXED;
  double* const* acc = m->stl[0];
  double* const* r = m->stl[2];
  double* const* prev = m->stl[5];
  if (int rc = stl_sponge_rigid(m, dt, x)) return rc;
  for (int q = 0; q < NSPECIES; ++q) CUDA_OK(cudaMemsetAsync(acc[q], 0, n * sizeof(double), m->stream));
  const double dts[3] = {dt / 3.0, dt / 2.0, dt};
  for (int st = 2; st >= 0; --st) {
    if (int rc = stl_substeps(m, st, dts[st] / n_sub, n_sub, x, true)) return rc;
    for (int q = 0; q < NSPECIES; ++q) {
      lin_scale_add(n, x[q], 1.0, acc[q], m->stream);           // through x0 directly
      lin_axpy(n, m->stl_zero, x[q], dts[st], r[q], m->stream);  // bar of R = dt_stage * bar
      CUDA_OK(cudaMemsetAsync(prev[q], 0, n * sizeof(double), m->stream));
    }
    tend_ad(m->d, m->met, m->fl, base[st], r, prev, m->stl_face, m->stl_cell, f32, m->stream);
    if (st == 0) {
      for (int q = 0; q < NSPECIES; ++q) lin_scale_add(n, prev[q], 1.0, acc[q], m->stream);
    } else if (int rc = copy_state(m, x, prev)) {
      return rc;
    }
  }
  return copy_state(m, x, acc);
}

// one step from the model's current state that records its stage inputs;
// base[0] is the step's input (the model's buffer, intact until the next step)
int stl_record_step(vibe_gb300_model* m, double dt, int n_sub, double* const* rec1, double* const* rec2,
                    double* const** base) {
  base[0] = m->S[m->cur];
  base[1] = rec1;
  base[2] = rec2;
  m->rec_stage[0] = rec1;
  m->rec_stage[1] = rec2;
  const int rc = enqueue_one_step(m, dt, n_sub);
  m->rec_stage[0] = m->rec_stage[1] = nullptr;
  return rc;
}

// 12 FieldT host arrays -> device perturbation fields (zero off the boxes)
int stl_upload(vibe_gb300_model* m, const double* const* host, double* const* dev) {
  for (int q = 0; q < NSPECIES; ++q) {
    if (!host[q]) return fail(VIBE_GB300_EBADARG, "bad argument");
    CUDA_OK(cudaMemsetAsync(dev[q], 0, state_count(m) * sizeof(double), m->stream));
    if (int rc = upload_storage(m, q, host[q], &dev[q], 1)) return rc;
  }
  return 0;
}
// device -> FieldT: the boxes from dev, every other point from keep
int stl_download(vibe_gb300_model* m, double* const* dev, const double* const* keep, double* const* host) {
  const dim3 b(32, 4);
  for (int q = 0; q < NSPECIES; ++q) {
    if (!host[q]) return fail(VIBE_GB300_EBADARG, "bad argument");
    int ni, nj, nk;
    box_of(m, q, ni, nj, nk);
    const size_t n = storage_count(m, q);
    CUDA_OK(cudaMemcpyAsync(m->d_stage_in, keep[q], n * sizeof(double), cudaMemcpyHostToDevice, m->stream));
    k_scatter<<<dim3((ni + 31) / 32, (nj + 3) / 4, nk), b, 0, m->stream>>>(m->d, m->nsx[q], m->nsy[q], ni, nj, nk,
                                                                            dev[q], m->d_stage_in);
    CUDA_OK(cudaGetLastError());
    CUDA_OK(cudaMemcpyAsync(host[q], m->d_stage_in, n * sizeof(double), cudaMemcpyDeviceToHost, m->stream));
    CUDA_OK(cudaStreamSynchronize(m->stream));
  }
  return 0;
}
}  // namespace

extern "C" {

int vibe_gb300_window_plan(size_t free_bytes, size_t state_bytes, int n_steps, int seg_states, int* every) {
  if (!every || n_steps < 1 || seg_states < 1 || state_bytes == 0) return fail(VIBE_GB300_EBADARG, "bad argument");
  // store every step when n_steps checkpoints and a one-step segment fit in
  // 80 % of the free device memory; otherwise checkpoint every
  // ceil(sqrt(n_steps / seg_states)) steps, which minimises checkpoints +
  // segment states, and recompute each segment from its checkpoint
  const double st = (double)state_bytes, budget = 0.8 * (double)free_bytes;
  if ((n_steps + (double)seg_states) * st <= budget) {
    *every = 1;
    return 0;
  }
  const int e = std::max(1, (int)std::ceil(std::sqrt((double)n_steps / seg_states)));
  const int nck = (n_steps + e - 1) / e;
  if ((nck + (double)seg_states * e) * st > budget)
    return fail(VIBE_GB300_EDEVICE, "the window's checkpoints do not fit in device memory");
  *every = e;
  return 0;
}

int vibe_gb300_window_create(vibe_gb300_model* m, vibe_tlad* t, double dt, int n_sub, int n_steps, int every,
                             int tl_substeps, vibe_gb300_window** out) {
  if (!m || !out || !(dt > 0.0) || n_steps < 1 || every < 0 || tl_substeps < 1)
    return fail(VIBE_GB300_EBADARG, "bad argument");
  // t == NULL: the TL/AD of the model's own step; a segment then holds three
  // states per step (its input and its second and third stages' inputs)
  const bool own = (t == nullptr);
  if (own) {
    if (tl_substeps != 1) return fail(VIBE_GB300_EBADARG, "the model's own step TL/AD takes tl_substeps = 1");
    if (int rc = stl_supported(m)) return rc;
    if (int rc = stl_ensure(m)) return rc;
  } else {
    int nx, ny, nz;
    vgb::tlad_grid(t, &nx, &ny, &nz);
    if (nx != m->d.nx || ny != m->d.ny || nz != m->d.nz)
      return fail(VIBE_GB300_EBADARG, "the TL/AD grid differs from the model's");
  }
  const int seg_states = own ? 3 : 2;
  if (every == 0) {
    size_t free_b = 0, total_b = 0;
    CUDA_OK(cudaMemGetInfo(&free_b, &total_b));
    const size_t state_b = state_count(m) * sizeof(double) * NSPECIES;
    if (int rc = vibe_gb300_window_plan(free_b, state_b, n_steps, seg_states, &every)) return rc;
  }
  auto* w = new vibe_gb300_window();
  w->m = m;
  w->t = t;
  w->dt = dt;
  w->n_sub = n_sub;
  w->n_steps = n_steps;
  w->every = every;
  w->tl_sub = tl_substeps;
  const int nck = (n_steps + every - 1) / every, seg_len = std::min(every, n_steps);
  const size_t n = state_count(m);
  int rc = 0;
  auto alloc_state = [&](std::array<double*, NSPECIES>& a) {
    for (int q = 0; q < NSPECIES && !rc; ++q) {
      void* p = nullptr;
      if (cudaMalloc(&p, n * sizeof(double)) != cudaSuccess) {
        rc = fail(VIBE_GB300_EDEVICE, "window buffer allocation");
      } else {
        w->allocs.push_back(p);
        a[q] = (double*)p;
      }
    }
  };
  w->ckpt.resize(nck);
  for (auto& a : w->ckpt) alloc_state(a);
  if (own) {
    w->seg[0].resize(3 * (size_t)seg_len);
    for (auto& a : w->seg[0]) alloc_state(a);
  } else {
    for (int b = 0; b < 2; ++b) {
      w->seg[b].resize(seg_len);
      for (auto& a : w->seg[b]) alloc_state(a);
    }
  }
  if (!rc && (cudaEventCreateWithFlags(&w->ev_model, cudaEventDisableTiming) != cudaSuccess ||
              cudaEventCreateWithFlags(&w->ev_seg[0], cudaEventDisableTiming) != cudaSuccess ||
              cudaEventCreateWithFlags(&w->ev_seg[1], cudaEventDisableTiming) != cudaSuccess ||
              cudaEventCreate(&w->e0) != cudaSuccess || cudaEventCreate(&w->e1) != cudaSuccess))
    rc = fail(VIBE_GB300_EDEVICE, "events");
  if (rc) {
    vibe_gb300_window_destroy(w);
    return rc;
  }
  *out = w;
  return 0;
}

void vibe_gb300_window_destroy(vibe_gb300_window* w) {
  if (!w) return;
  if (w->m) cudaStreamSynchronize(w->m->stream);
  if (w->t) cudaStreamSynchronize(vgb::tlad_stream(w->t));
  for (cudaEvent_t e : {w->ev_model, w->ev_seg[0], w->ev_seg[1], w->e0, w->e1})
    if (e) cudaEventDestroy(e);
  for (void* p : w->allocs) cudaFree(p);
  delete w;
}

}  // extern "C"

namespace {
// the model's own step TL/AD over the window (t == NULL), on the model stream
int own_window_tl(vibe_gb300_window* w, const double* const* dx0, double* const* dx_out) {
  vibe_gb300_model* m = w->m;
  const int n_sub = std::max(w->n_sub, 1);
  if (int rc = configure_dt(m, w->dt, n_sub)) return rc;
  if (int rc = stl_upload(m, dx0, m->stl[1])) return rc;
  if (int rc = window_begin(w)) return rc;
  for (int n = 0; n < w->n_steps; ++n) {
    if (n % w->every == 0)
      if (int rc = window_checkpoint(w, n / w->every)) return rc;
    double* const* base[3];
    if (int rc = stl_record_step(m, w->dt, n_sub, m->stl[3], m->stl[4], base)) return rc;
    if (int rc = stl_step_tl(m, w->dt, n_sub, base, m->stl[1])) return rc;
  }
  if (int rc = window_end(w, m->stream)) return rc;
  if (int rc = stl_download(m, m->stl[1], dx0, dx_out)) return rc;
  if (int rc = read_status(m)) return rc;
  if (int rc = window_restart(w, 0)) return rc;
  return read_status(m);
}

int own_window_ad(vibe_gb300_window* w, const double* const* dy, double* const* dx0_adjoint) {
  vibe_gb300_model* m = w->m;
  const int n_sub = std::max(w->n_sub, 1);
  if (int rc = configure_dt(m, w->dt, n_sub)) return rc;
  if (int rc = stl_upload(m, dy, m->stl[1])) return rc;
  if (int rc = window_begin(w)) return rc;
  const int nck = (int)w->ckpt.size();
  const int last_ck = (nck - 1) * w->every;
  for (int n = 0; n <= last_ck; ++n) {  // forward sweep: checkpoints only
    if (n % w->every == 0)
      if (int rc = window_checkpoint(w, n / w->every)) return rc;
    if (n < last_ck)
      if (int rc = enqueue_one_step(m, w->dt, n_sub)) return rc;
  }
  auto& seg = w->seg[0];
  for (int sgm = nck - 1; sgm >= 0; --sgm) {  // backward over the segments
    const int first = sgm * w->every, last = std::min(w->n_steps, first + w->every);
    if (int rc = window_restart(w, sgm)) return rc;
    for (int n = first; n < last; ++n) {  // recompute: each step's three stage inputs
      const size_t o = 3 * (size_t)(n - first);
      if (int rc = copy_state(m, seg[o].data(), m->S[m->cur])) return rc;
      double* const* base[3];
      if (int rc = stl_record_step(m, w->dt, n_sub, seg[o + 1].data(), seg[o + 2].data(), base)) return rc;
    }
    for (int n = last - 1; n >= first; --n) {
      const size_t o = 3 * (size_t)(n - first);
      double* const* base[3] = {seg[o].data(), seg[o + 1].data(), seg[o + 2].data()};
      if (int rc = stl_step_ad(m, w->dt, n_sub, base, m->stl[1])) return rc;
    }
  }
  if (int rc = window_end(w, m->stream)) return rc;
  if (int rc = stl_download(m, m->stl[1], dy, dx0_adjoint)) return rc;
  if (int rc = read_status(m)) return rc;
  if (int rc = window_restart(w, 0)) return rc;
  return read_status(m);
}

int own_step_linear(vibe_gb300_model* m, double dt, int n_sub_in, const double* const* in, double* const* out,
                    bool adjoint) {
  if (!m || !in || !out || !(dt > 0.0)) return fail(VIBE_GB300_EBADARG, "bad argument");
  if (int rc = stl_supported(m)) return rc;
  if (int rc = stl_ensure(m)) return rc;
  const int n_sub = std::max(n_sub_in, 1);
  if (int rc = configure_dt(m, dt, n_sub)) return rc;
  if (int rc = stl_upload(m, in, m->stl[1])) return rc;
  const int c0 = m->cur;
  double* const* base[3];
  if (int rc = stl_record_step(m, dt, n_sub, m->stl[3], m->stl[4], base)) return rc;
  const int rc = adjoint ? stl_step_ad(m, dt, n_sub, base, m->stl[1]) : stl_step_tl(m, dt, n_sub, base, m->stl[1]);
  m->cur = c0;  // the linearisation point stays the model's state
  if (rc) return rc;
  if (int rc2 = sync_working(m)) return rc2;
  if (int rc2 = stl_download(m, m->stl[1], in, out)) return rc2;
  return read_status(m);
}
}  // namespace

extern "C" {

int vibe_gb300_window_tl(vibe_gb300_window* w, const double* const* dx0, double* const* dx_out) {
  if (!w || !dx0 || !dx_out) return fail(VIBE_GB300_EBADARG, "bad argument");
  if (!w->t) return own_window_tl(w, dx0, dx_out);
  vibe_gb300_model* m = w->m;
  vibe_tlad* t = w->t;
  cudaStream_t ts = vgb::tlad_stream(t);
  CUDA_OK(cudaStreamSynchronize(m->stream));
  double* const* v[2] = {vgb::tlad_work(t, 0), vgb::tlad_work(t, 1)};
  if (!vgb::tlad_upload(t, dx0, v[0])) return fail(VIBE_GB300_EBADARG, vibe_tlad_last_error());
  if (int rc = window_begin(w)) return rc;
  const double dtl = w->dt / w->tl_sub;
  int c = 0;
  for (int n = 0; n < w->n_steps; ++n) {
    if (n % w->every == 0)
      if (int rc = window_checkpoint(w, n / w->every)) return rc;
    CUDA_OK(cudaEventRecord(w->ev_model, m->stream));  // x_n is ready
    CUDA_OK(cudaStreamWaitEvent(ts, w->ev_model, 0));
    vgb::tlad_use_base(t, m->S[m->cur]);
    for (int j = 0; j < w->tl_sub; ++j, c = 1 - c) vgb::tlad_tl_step(t, v[c], v[1 - c], dtl);
    CUDA_OK(cudaEventRecord(w->ev_seg[0], ts));
    if (n + 1 < w->n_steps) {
      // step n reads x_n and writes the other buffer (overlaps the TL step);
      // step n + 1 overwrites x_n, so it waits for the TL step
      if (int rc = enqueue_steps(m, w->dt, w->n_sub, 1)) return rc;
      CUDA_OK(cudaStreamWaitEvent(m->stream, w->ev_seg[0], 0));
    }
  }
  if (int rc = window_end(w, ts)) return rc;
  if (!vgb::tlad_download(t, v[c], dx0, dx_out)) return fail(VIBE_GB300_EDEVICE, vibe_tlad_last_error());
  if (int rc = read_status(m)) return rc;
  if (int rc = window_restart(w, 0)) return rc;  // back to the window's initial state
  return read_status(m);
}

int vibe_gb300_window_ad(vibe_gb300_window* w, const double* const* dy, double* const* dx0_adjoint) {
  if (!w || !dy || !dx0_adjoint) return fail(VIBE_GB300_EBADARG, "bad argument");
  if (!w->t) return own_window_ad(w, dy, dx0_adjoint);
  vibe_gb300_model* m = w->m;
  vibe_tlad* t = w->t;
  cudaStream_t ts = vgb::tlad_stream(t);
  CUDA_OK(cudaStreamSynchronize(m->stream));
  double* const* v[2] = {vgb::tlad_work(t, 0), vgb::tlad_work(t, 1)};
  if (!vgb::tlad_upload(t, dy, v[0])) return fail(VIBE_GB300_EBADARG, vibe_tlad_last_error());
  if (int rc = window_begin(w)) return rc;
  // forward sweep: checkpoints only
  const int nck = (int)w->ckpt.size();
  const int last_ck = (nck - 1) * w->every;
  for (int n = 0; n <= last_ck; ++n) {
    if (n % w->every == 0)
      if (int rc = window_checkpoint(w, n / w->every)) return rc;
    if (n < last_ck)
      if (int rc = enqueue_steps(m, w->dt, w->n_sub, 1)) return rc;
  }
  // backward sweep over the segments, recomputing each from its checkpoint
  const double dtl = w->dt / w->tl_sub;
  int c = 0;
  for (int sgm = nck - 1; sgm >= 0; --sgm) {
    const int b = sgm & 1, first = sgm * w->every, last = std::min(w->n_steps, first + w->every);
    if (sgm <= nck - 3) CUDA_OK(cudaStreamWaitEvent(m->stream, w->ev_seg[b], 0));  // its buffers are free again
    if (int rc = window_restart(w, sgm)) return rc;
    for (int n = first; n < last; ++n) {
      if (int rc = copy_state(m, w->seg[b][n - first].data(), m->S[m->cur])) return rc;
      if (n + 1 < last)
        if (int rc = enqueue_steps(m, w->dt, w->n_sub, 1)) return rc;
    }
    CUDA_OK(cudaEventRecord(w->ev_model, m->stream));
    CUDA_OK(cudaStreamWaitEvent(ts, w->ev_model, 0));
    for (int n = last - 1; n >= first; --n) {
      vgb::tlad_use_base(t, w->seg[b][n - first].data());
      for (int j = 0; j < w->tl_sub; ++j, c = 1 - c) vgb::tlad_ad_step(t, v[c], v[1 - c], dtl);
    }
    CUDA_OK(cudaEventRecord(w->ev_seg[b], ts));
  }
  if (int rc = window_end(w, ts)) return rc;
  if (!vgb::tlad_download(t, v[c], dy, dx0_adjoint)) return fail(VIBE_GB300_EDEVICE, vibe_tlad_last_error());
  if (int rc = read_status(m)) return rc;
  if (int rc = window_restart(w, 0)) return rc;
  return read_status(m);
}

int vibe_gb300_tendency_tl(vibe_gb300_model* m, const double* const* dx, double* const* out) {
  if (!m || !dx || !out) return fail(VIBE_GB300_EBADARG, "bad argument");
  if (int rc = stl_supported(m)) return rc;
  if (int rc = stl_ensure(m)) return rc;
  if (int rc = stl_upload(m, dx, m->stl[1])) return rc;
  tend_tl(m->d, m->met, m->fl, m->S[m->cur], m->stl[1], m->stl[2], m->stl_face, m->precision == VIBE_GB300_MIXED,
          m->stream);
  CUDA_OK(cudaGetLastError());
  for (int q = 0; q < NSPECIES; ++q) {  // the tendency's boxes; zero elsewhere
    const int ni = m->d.nx + (q == U), nj = m->d.ny + (q == V), nk = m->d.nz + (q == W);
    unpack<double>(m->d, m->nsx[q], m->nsy[q], m->nsz[q], ni, nj, nk, m->stl[2][q],
                                          m->d_stage_in, m->stream);
    CUDA_OK(cudaMemcpyAsync(out[q], m->d_stage_in, storage_count(m, q) * sizeof(double), cudaMemcpyDeviceToHost,
                            m->stream));
    CUDA_OK(cudaStreamSynchronize(m->stream));
  }
  return read_status(m);
}

int vibe_gb300_tendency_ad(vibe_gb300_model* m, const double* const* bar_r, double* const* bar_x) {
  if (!m || !bar_r || !bar_x) return fail(VIBE_GB300_EBADARG, "bad argument");
  if (int rc = stl_supported(m)) return rc;
  if (int rc = stl_ensure(m)) return rc;
  if (int rc = stl_upload(m, bar_r, m->stl[2])) return rc;
  for (int q = 0; q < NSPECIES; ++q)  // only the tendency's boxes are its outputs
    k_keep_box<<<1024, 256, 0, m->stream>>>(m->d, m->d.nx + (q == U), m->d.ny + (q == V), m->d.nz + (q == W),
                                            m->stl[2][q]);
  for (int q = 0; q < NSPECIES; ++q)
    CUDA_OK(cudaMemsetAsync(m->stl[5][q], 0, state_count(m) * sizeof(double), m->stream));
  tend_ad(m->d, m->met, m->fl, m->S[m->cur], m->stl[2], m->stl[5], m->stl_face, m->stl_cell,
          m->precision == VIBE_GB300_MIXED, m->stream);
  CUDA_OK(cudaGetLastError());
  for (int q = 0; q < NSPECIES; ++q) {  // every uploaded point (the boxes incl. ghosts)
    int ni, nj, nk;
    box_of(m, q, ni, nj, nk);
    unpack<double>(m->d, m->nsx[q], m->nsy[q], m->nsz[q], ni, nj, nk, m->stl[5][q],
                                          m->d_stage_in, m->stream);
    CUDA_OK(cudaMemcpyAsync(bar_x[q], m->d_stage_in, storage_count(m, q) * sizeof(double), cudaMemcpyDeviceToHost,
                            m->stream));
    CUDA_OK(cudaStreamSynchronize(m->stream));
  }
  return read_status(m);
}

int vibe_gb300_step_tl(vibe_gb300_model* m, double dt, int n_sub, const double* const* dx, double* const* out) {
  return own_step_linear(m, dt, n_sub, dx, out, false);
}

int vibe_gb300_step_ad(vibe_gb300_model* m, double dt, int n_sub, const double* const* dy, double* const* out) {
  return own_step_linear(m, dt, n_sub, dy, out, true);
}

int vibe_gb300_window_stats(const vibe_gb300_window* w, double* last_ms, size_t* checkpoint_bytes,
                            size_t* segment_bytes) {
  if (!w) return fail(VIBE_GB300_EBADARG, "bad argument");
  const size_t st = state_count(w->m) * NSPECIES * sizeof(double);
  if (last_ms) *last_ms = w->last_ms;
  if (checkpoint_bytes) *checkpoint_bytes = st * w->ckpt.size();
  if (segment_bytes) *segment_bytes = st * (w->seg[0].size() + w->seg[1].size());
  return 0;
}

}  // extern "C"

namespace {
// after new FP64 state values of the species in `given` (others untouched):
// the FP32 working copy, and the ghost line of rho' and the inactive species
// in every FP32 buffer
int after_upload(vibe_gb300_model* m, const bool* given, int nspecies) {
  if (m->precision != VIBE_GB300_MIXED) return 0;
  if (int rc = sync_working(m)) return rc;
  const size_t n = m->d.plane * (size_t)(m->d.nz + 1) * sizeof(float);
  const int last = m->fl.moist ? QG : QV;
  for (int q = 0; q < nspecies; ++q) {
    if (!given[q] || !(q == RHO || q > last)) continue;
    for (int b = 0; b < 2; ++b) CUDA_OK(cudaMemcpyAsync(m->WSt[b][q], m->W0[q], n, cudaMemcpyDeviceToDevice, m->stream));
    if (acoustic_field(q)) {
      CUDA_OK(cudaMemcpyAsync(m->WA[q], m->W0[q], n, cudaMemcpyDeviceToDevice, m->stream));
      CUDA_OK(cudaMemcpyAsync(m->WB[q], m->W0[q], n, cudaMemcpyDeviceToDevice, m->stream));
    }
  }
  return 0;
}

// mixed models: one pass from the FieldT staging into the FP64 state (the
// buffer of the current parity) and the FP32 working copy (the conversion of
// to_working_body), plus the points that the step about to run does not
// write but reads later: in the other state buffer the ghost lines (i = nx for cell fields and w, j = ny for u,
// i = nx for v; the finish writes every other point of the next state) and
// all of a species it does not carry (beyond `last`); in rho's other working
// copies (stage outputs and substep buffers) its ghost lines
__global__ void k_pack_mixed(Dims d, int q, int last, int nsx, int nsy, int ni, int nj, int nk,
                             const double* __restrict__ ref, const double* __restrict__ src, double* __restrict__ s0,
                             double* __restrict__ s1, float* __restrict__ w0, float* __restrict__ c0,
                             float* __restrict__ c1, float* __restrict__ c2, float* __restrict__ c3) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
  if (i >= ni || j >= nj || k >= nk) return;
  const size_t c = d.idx(i, j, k);
  const double v = src[soff(nsx, nsy, i, j, k)];
  const bool ghost = (q == U) ? j == d.ny : (q == V) ? i == d.nx : (i == d.nx || j == d.ny);
  s0[c] = v;
  if (ghost || q > last) s1[c] = v;
  if (!w0) return;
  bool put;  // the points to_working_body converts
  if (q == U) put = j < d.ny && k < d.nz;
  else if (q == V) put = i < d.nx && k < d.nz;
  else if (q == W) put = i < d.nx && j < d.ny;
  else put = k < d.nz;
  if (!put) return;
  const float wv = ref ? (float)(v - ref[k]) : (float)v;
  w0[c] = wv;
  if (c0 && ghost) {
    c0[c] = wv;
    c1[c] = wv;
    c2[c] = wv;
    c3[c] = wv;
  }
}

void pack_mixed(vibe_gb300_model* m, int q, const double* src) {
  int ni, nj, nk;
  box_of(m, q, ni, nj, nk);
  const int last = m->fl.moist ? QG : QV;
  const double* ref = (q == RHO) ? m->tab.r0d : (q == THETA) ? m->tab.t0dd : (q == PI) ? m->tab.p0d : nullptr;
  float* w0 = (q > last) ? nullptr : m->W0[q];
  float *c0 = nullptr, *c1 = nullptr, *c2 = nullptr, *c3 = nullptr;
  if (q == RHO) {  // after_upload's copies of the working value
    c0 = m->WSt[0][q];
    c1 = m->WSt[1][q];
    c2 = m->WA[q];
    c3 = m->WB[q];
  }
  const dim3 b(32, 4);
  k_pack_mixed<<<dim3((ni + 31) / 32, (nj + 3) / 4, nk), b, 0, m->stream>>>(m->d, q, last, m->nsx[q], m->nsy[q], ni,
                                                                            nj, nk, ref, src, m->S[m->cur][q],
                                                                            m->S[1 - m->cur][q], w0, c0, c1, c2, c3);
}

void pack_both(vibe_gb300_model* m, int q, const double* src) {
  int ni, nj, nk;
  box_of(m, q, ni, nj, nk);
  const dim3 b(32, 4);
  for (int t = 0; t < 2; ++t)
    k_pack<<<dim3((ni + 31) / 32, (nj + 3) / 4, nk), b, 0, m->stream>>>(m->d, m->nsx[q], m->nsy[q], ni, nj, nk, src,
                                                                         m->S[t][q]);
}

int io_setup(vibe_gb300_model* m) {
  auto* io = new vibe_gb300_model::IoPipe();
  m->io = io;
  CUDA_OK(cudaStreamCreateWithFlags(&io->sin, cudaStreamNonBlocking));
  CUDA_OK(cudaStreamCreateWithFlags(&io->sout, cudaStreamNonBlocking));
  CUDA_OK(cudaEventCreateWithFlags(&io->start, cudaEventDisableTiming));
  for (int b = 0; b < 2; ++b) {
    for (cudaEvent_t* e : {&io->in_done[b], &io->packed[b], &io->unpacked[b], &io->out_done[b]})
      CUDA_OK(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    for (int q = 0; q < NSPECIES; ++q) {
      if (int rc = dalloc(m, &io->in[b][q], storage_count(m, q))) return rc;
      if (int rc = dalloc(m, &io->out[b][q], storage_count(m, q))) return rc;
    }
  }
  CUDA_OK(cudaStreamSynchronize(m->stream));
  return 0;
}

void io_release(vibe_gb300_model* m) {
  auto* io = m->io;
  if (!io) return;
  if (io->sin) cudaStreamSynchronize(io->sin);
  if (io->sout) cudaStreamSynchronize(io->sout);
  for (cudaEvent_t e : {io->start, io->in_done[0], io->in_done[1], io->packed[0], io->packed[1], io->unpacked[0],
                        io->unpacked[1], io->out_done[0], io->out_done[1]})
    if (e) cudaEventDestroy(e);
  if (io->sin) cudaStreamDestroy(io->sin);
  if (io->sout) cudaStreamDestroy(io->sout);
  delete io;  // staging buffers are in m->allocs
  m->io = nullptr;
}
}  // namespace

extern "C" {

int vibe_gb300_set_state(vibe_gb300_model* m, const double* const* host, int nspecies) {
  if (!m || !host || nspecies < 1 || nspecies > NSPECIES) return fail(VIBE_GB300_EBADARG, "bad argument");
  bool given[NSPECIES] = {};
  for (int q = 0; q < nspecies; ++q) {
    if (!host[q]) continue;
    given[q] = true;
    double* dst[2] = {m->S[0][q], m->S[1][q]};
    if (int rc = upload_storage(m, q, host[q], dst, 2)) return rc;
  }
  if (int rc = after_upload(m, given, nspecies)) return rc;
  CUDA_OK(cudaGetLastError());
  return 0;
}

// One step with host input and output, pipelined across calls: the input's
// host -> device copies run on one copy stream, the step on the model's
// stream, the result's device -> host copies on another; with two staging
// buffers each way, step n's download and step n+2's upload overlap step
// n+1's compute.
int vibe_gb300_step_io(vibe_gb300_model* m, const double* const* host_in, int n_in, double* const* host_out,
                       int n_out, double dt, int n_sub) {
  if (!m || n_in < 0 || n_in > NSPECIES || n_out < 0 || n_out > NSPECIES || (n_in && !host_in) ||
      (n_out && !host_out) || !(dt > 0.0))
    return fail(VIBE_GB300_EBADARG, "bad argument");
  if (!m->io)
    if (int rc = io_setup(m)) return rc;
  auto* io = m->io;
  const int b = (int)(io->n & 1);
  // the first call after a join starts its uploads after whatever is on the
  // model's stream (so an event recorded there before it brackets the
  // pipeline); later uploads only wait until their staging buffer was packed,
  // and so overlap the previous step
  if (io->idle) {
    CUDA_OK(cudaEventRecord(io->start, m->stream));
    CUDA_OK(cudaStreamWaitEvent(io->sin, io->start, 0));
    io->idle = false;
  }
  CUDA_OK(cudaStreamWaitEvent(io->sin, io->packed[b], 0));
  bool given[NSPECIES] = {};
  for (int q = 0; q < n_in; ++q) {
    if (!host_in[q]) continue;
    given[q] = true;
    CUDA_OK(cudaMemcpyAsync(io->in[b][q], host_in[q], storage_count(m, q) * sizeof(double), cudaMemcpyHostToDevice,
                            io->sin));
  }
  CUDA_OK(cudaEventRecord(io->in_done[b], io->sin));
  CUDA_OK(cudaStreamWaitEvent(m->stream, io->in_done[b], 0));
  if (m->precision == VIBE_GB300_MIXED) {  // state and working copy in one pass per field
    for (int q = 0; q < n_in; ++q)
      if (given[q]) pack_mixed(m, q, io->in[b][q]);
  } else {
    for (int q = 0; q < n_in; ++q)
      if (given[q]) pack_both(m, q, io->in[b][q]);
  }
  CUDA_OK(cudaEventRecord(io->packed[b], m->stream));
  if (int rc = enqueue_steps(m, dt, n_sub, 1)) return rc;
  CUDA_OK(cudaStreamWaitEvent(m->stream, io->out_done[b], 0));  // the staging buffer was read out
  for (int q = 0; q < n_out; ++q) {
    if (!host_out[q]) continue;
    int ni, nj, nk;
    box_of(m, q, ni, nj, nk);
    unpack<double>(m->d, m->nsx[q], m->nsy[q], m->nsz[q], ni, nj, nk, m->S[m->cur][q],
                                          io->out[b][q], m->stream);
  }
  CUDA_OK(cudaEventRecord(io->unpacked[b], m->stream));
  CUDA_OK(cudaStreamWaitEvent(io->sout, io->unpacked[b], 0));
  for (int q = 0; q < n_out; ++q)
    if (host_out[q])
      CUDA_OK(cudaMemcpyAsync(host_out[q], io->out[b][q], storage_count(m, q) * sizeof(double),
                              cudaMemcpyDeviceToHost, io->sout));
  CUDA_OK(cudaEventRecord(io->out_done[b], io->sout));
  ++io->n;
  CUDA_OK(cudaGetLastError());
  return 0;
}

// make the model's stream wait for every copy of the host-I/O pipeline (an
// event recorded on the model's stream after this covers all of it)
int vibe_gb300_io_join(vibe_gb300_model* m) {
  if (!m) return fail(VIBE_GB300_EBADARG, "bad argument");
  if (!m->io) return 0;
  for (int b = 0; b < 2; ++b) {
    CUDA_OK(cudaStreamWaitEvent(m->stream, m->io->in_done[b], 0));
    CUDA_OK(cudaStreamWaitEvent(m->stream, m->io->out_done[b], 0));
  }
  m->io->idle = true;
  return 0;
}

int vibe_gb300_get_state(vibe_gb300_model* m, double* const* host, int nspecies) {
  if (!m || !host || nspecies < 1 || nspecies > NSPECIES) return fail(VIBE_GB300_EBADARG, "bad argument");
  for (int q = 0; q < nspecies; ++q) {
    if (!host[q]) continue;
    int ni, nj, nk;
    box_of(m, q, ni, nj, nk);
    unpack<double>(m->d, m->nsx[q], m->nsy[q], m->nsz[q], ni, nj, nk, m->S[m->cur][q],
                                          m->d_stage_in, m->stream);
    CUDA_OK(cudaMemcpyAsync(host[q], m->d_stage_in, storage_count(m, q) * sizeof(double), cudaMemcpyDeviceToHost,
                            m->stream));
  }
  CUDA_OK(cudaGetLastError());
  return 0;
}

int vibe_gb300_set_kernel_timing(vibe_gb300_model* m, int enable) {
  if (!m) return fail(VIBE_GB300_EBADARG, "bad argument");
  CUDA_OK(cudaStreamSynchronize(m->stream));
  collect_timing(m);
  m->timing = enable != 0;
  for (int c = 0; c < vibe_gb300_model::kClasses; ++c) { m->class_ms[c] = 0.0; m->class_n[c] = 0; }
  return 0;
}

int vibe_gb300_kernel_times(vibe_gb300_model* m, double* ms, long* count, int nclass) {
  if (!m || !ms || !count) return fail(VIBE_GB300_EBADARG, "bad argument");
  CUDA_OK(cudaStreamSynchronize(m->stream));
  collect_timing(m);
  for (int c = 0; c < nclass && c < vibe_gb300_model::kClasses; ++c) { ms[c] = m->class_ms[c]; count[c] = m->class_n[c]; }
  return 0;
}

int vibe_gb300_device_field(vibe_gb300_model* m, int q, double** ptr, int* pitch) {
  if (!m || !ptr || q < 0 || q >= NSPECIES) return fail(VIBE_GB300_EBADARG, "bad argument");
  *ptr = m->S[m->cur][q];
  if (pitch) *pitch = m->d.P;
  return 0;
}

vibe_stream_t vibe_gb300_stream(vibe_gb300_model* m) { return m ? (vibe_stream_t)m->stream : nullptr; }

int vibe_gb300_launches_per_step(const vibe_gb300_model* m, int n_sub) {
  if (!m) return 0;
  n_sub = n_sub > 1 ? n_sub : 1;
  if (m->precision == VIBE_GB300_MIXED)
    return (m->fl.acoustic_mode == 2) ? 3 * (1 + n_sub) + 2 + 1 : 3 * (1 + 2 * n_sub) + 1;  // stage 3's u/v in finish
  const int tend = 4 + ((m->fl.div_damp > 0.0 && m->fl.div_order > 2) ? 1 : 0);
  const int sub = (m->fl.acoustic_mode == 0) ? 2 : (m->fl.acoustic_mode == 1 ? 4 : 2);
  return 3 * (tend + NSPECIES + n_sub * sub + 1) + 1;
}

}  // extern "C"
