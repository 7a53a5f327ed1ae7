// Kessler warm-rain microphysics as a physics package of the step
// (include/vibe_gb300.h: vibe_gb300_physics_kessler).
//
// Follows KesslerMicrophysics::step_column (src/physics/microphysics_kessler.
// cpp:269-331) with its helpers (saturation_adjust_point :100-144,
// rain_fall_speed :188-191, autoconversion / accretion :194-202,
// rain_evaporation_rate :213-227, sediment_rain :240-262; slope_parameter,
// ventilation_factor, particle_mass_rate :38-76; thermodynamics
// src/physics/physics_types.cpp:143-167 and physics_types.hpp:136-161), applied
// the way PhysicsDriver's microphysics step applies it: the column is built by
// state_to_column (physics_driver.cpp:95-128; layer depths by
// PhysicsColumn::diagnose_layer_depth, physics_types.cpp:257-284) and the
// tendencies are (after - before) / dt (physics_driver.cpp:271-288).
//
// One thread per column marching from the top level down. Every process of
// the scheme at level k depends only on level k and on the rain flux falling
// from level k+1, so the four passes of the column step (saturation
// adjustment, autoconversion + accretion, sedimentation from the top, rain
// evaporation) are done level by level in one top-down sweep with the same
// result. tgamma(1 + b) and cbrt(Sc) of the reference are constants, taken
// from the host's libm.
#include <cmath>

#include "vibe_gb300.h"
#include "vibe_internal.cuh"

namespace vgb {
namespace {

constexpr double kRv = 461.51, kKappaPhys = 0.28571, kT0 = 273.15;
constexpr double kRhoWater = 1000.0, kDvWater = 2.21e-5, kThermCondAir = 2.40e-2;
constexpr double kDynViscAir = 1.8e-5, kSchmidt = 0.6, kRainN0 = 8.0e6, kRainB = 3.0;

template <class R>
struct KesslerParams {
  R qc0, k1, k2, evap_coef, rain_a, rain_b;
  R rain_num;   // a N0 tgamma(1 + b), a = pi/6 rho_w
  R cbrt_sc;    // cbrt(Schmidt number)
  int positive_definite, exner_offset;
};

template <class R> __device__ __forceinline__ R rmax(R a, R b) { return a < b ? b : a; }  // std::max
template <class R> __device__ __forceinline__ R rmin(R a, R b) { return b < a ? b : a; }  // std::min
template <class R> __device__ __forceinline__ R rclamp(R v, R lo, R hi) { return v < lo ? lo : (hi < v ? hi : v); }
// FP64 models: the library functions (the reference's libm calls to an ulp
// or two). Mixed models: the FP32 hardware approximations, whose relative
// error (a few 1e-6 for these arguments) is far inside the FP32 path's
// tolerance against the FP64 scheme.
__device__ __forceinline__ double rpow(double a, double b) { return pow(a, b); }
__device__ __forceinline__ float rpow(float a, float b) { return __powf(a, b); }
__device__ __forceinline__ double rexp(double a) { return exp(a); }
__device__ __forceinline__ double rabs(double a) { return fabs(a); }
__device__ __forceinline__ float rabs(float a) { return fabsf(a); }
__device__ __forceinline__ float rexp(float a) { return __expf(a); }

template <class R> __device__ __forceinline__ R exner_of(R p) { return rpow(p / (R)kP0, (R)kKappaPhys); }
template <class R> __device__ __forceinline__ R latent_v(R t) { return ((R)2.501 - (R)0.00237 * (t - (R)kT0)) * (R)1.0e6; }
template <class R> __device__ __forceinline__ R qsat(R p, R t) {
  const R tc = rmax(t - (R)kT0, (R)-80.0);
  const R es = (R)611.2 * rexp((R)17.67 * tc / (tc + (R)243.5));
  return (R)kEpsVap * es / rmax(p - es, (R)1.0);
}
template <class R> __device__ __forceinline__ R fall_speed(const KesslerParams<R>& o, R rho, R qr) {
  const R load = rmax(rho * rmax(qr, (R)0), (R)0);
  return o.rain_a * rpow(load, o.rain_b);
}

// saturation_adjust_point (liquid phase, 10 Newton iterations, tol 1e-10)
template <class R>
__device__ void adjust(R& qv_io, R& qc_io, R& theta_io, R p) {
  R qv = rmax(qv_io, (R)0), qc = rmax(qc_io, (R)0), theta = theta_io;
  const R pi = exner_of(p);
  R t = rmax(theta * pi, (R)150);
  R qs = qsat(p, t);
  R l = latent_v(t);
  const R denom0 = (R)1 + l * l * qs / ((R)kCp * (R)kRv * t * t);
  R delta = rclamp((qv - qs) / denom0, -qc, qv);
  if (rabs(delta) < (R)1.0e-16) {
    qv_io = qv;
    qc_io = qc;
    return;
  }
  for (int it = 1; it <= 10; ++it) {
    t = theta * pi + (l / (R)kCp) * delta;
    t = rmax(t, (R)150);
    qs = qsat(p, t);
    l = latent_v(t);
    const R f = qv - delta - qs;
    const R dqsdT = l * qs / ((R)kRv * t * t);
    const R df = (R)-1 - (l / (R)kCp) * dqsdT;
    const R residual = rabs(f) / rmax(qs, (R)1.0e-12);
    if (residual <= (R)1.0e-10) break;
    const R step = -f / df;
    const R trial = rclamp(delta + rclamp(step, (R)-1.0, (R)1.0), -qc, qv);
    if (trial == delta) break;
    delta = trial;
  }
  qv -= delta;
  qc += delta;
  theta += l * delta / ((R)kCp * pi);
  qv_io = rmax(qv, (R)0);
  qc_io = rmax(qc, (R)0);
  theta_io = theta;
}

// rain_evaporation_rate with the exponential-spectrum helpers
template <class R>
__device__ R evap_rate(const KesslerParams<R>& o, R t, R rho, R qv, R qs, R qr) {
  if (!(qr > (R)0) || !(rho > (R)0)) return (R)0;
  const R qq = rmax(qr, (R)1.0e-14);
  const R den = rmax(rho * qq, (R)1.0e-20);
  const R lambda = rpow(o.rain_num / den, (R)1 / (R)kRainB);
  const R nr = (R)kRainN0 / rmax(lambda, (R)1.0e-8);
  const R r_mean = (R)0.5 / rmax(lambda, (R)1.0e-8);
  const R vt = fall_speed(o, rho, qr);
  R fv = (R)1;
  if (r_mean > (R)0) {
    const R re = (R)2 * r_mean * rmax(vt, (R)0) * rho / (R)kDynViscAir;
    fv = rmax((R)0.78 + (R)0.308 * o.cbrt_sc * sqrt(rmax(re, (R)0)), (R)1);
  }
  R dm = (R)0;
  if (r_mean > (R)0 && rho > (R)0 && t > (R)0) {
    const R rho_v = qv * rho, rho_vs = qs * rho;
    const R l = latent_v(t);
    const R dnm = (R)1 + l * l * (R)kDvWater * rho_vs / ((R)kThermCondAir * (R)kRv * t * t);
    dm = (R)4 * (R)kPi * r_mean * fv * (rho_v - rho_vs) / dnm;
  }
  const R rate = (-dm) * nr / rho;
  return rmax(o.evap_coef * rate, (R)0);
}

// state element -> compute type; departures (mixed) become totals
template <class R> __device__ __forceinline__ R tot(const double* s, const double*, size_t c) { return (R)s[c]; }
template <class R> __device__ __forceinline__ R tot(const float* s, const double* ref, size_t c) {
  return (R)s[c] + (R)ref[c];
}

template <class T, class R>
__global__ void k_kessler(const vibe_gb300_physics_args a, KesslerParams<R> o) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= a.nx || j >= a.ny) return;
  const int nz = a.nz;
  const R dt = (R)a.dt;
  const size_t plane = (size_t)a.pitch * (a.ny + 1), col = (size_t)j * a.pitch + i;
  const T* th_s = (const T*)a.state[THETA];
  const T* pi_s = (const T*)a.state[PI];
  const T* rho_s = (const T*)a.state[RHO];
  const T* qv_s = (const T*)a.state[QV];
  const T* qc_s = (const T*)a.state[QC];
  const T* qr_s = (const T*)a.state[QR];
  T* t_th = (T*)a.tend[THETA];
  T* t_qv = (T*)a.tend[QV];
  T* t_qc = (T*)a.tend[QC];
  T* t_qr = (T*)a.tend[QR];
  const bool mixed = sizeof(T) == sizeof(float);
  const R zs = (R)a.terrain[(size_t)j * a.nx + i], depth = (R)a.depth[(size_t)j * a.nx + i];
  auto zc = [&](int k) { return zs + (R)a.zeta_mid[k] * depth; };  // Grid::z_center
  R flux_in = (R)0;
  // level heights around the current level, carried down the column
  R z_up = (R)0, z_here = zc(nz - 1), z_dn = (nz > 1) ? zc(nz - 2) : (R)0;
  for (int k = nz - 1; k >= 0; --k) {
    const size_t c = (size_t)k * plane + col;
    // layer depth (diagnose_layer_depth): interfaces halfway between centres,
    // extrapolated at the bottom and top; 100 m for a single level
    R dz;
    if (nz == 1) {
      dz = rmax((z_here + (R)0.5 * (R)100) - (z_here - (R)0.5 * (R)100), (R)1.0e-6);
    } else {
      const R z = z_here;
      const R zlo = (k == 0) ? z - (R)0.5 * (z_up - z) : (R)0.5 * (z_dn + z);
      const R zhi = (k == nz - 1) ? z + (R)0.5 * (z - z_dn) : (R)0.5 * (z + z_up);
      dz = rmax(zhi - zlo, (R)1.0e-6);
    }
    z_up = z_here;
    z_here = z_dn;
    if (k >= 2) z_dn = zc(k - 2);
    // state_to_column
    const R pi0 = (R)a.ref_pi[c];
    const R pis = mixed ? tot<R>(pi_s, a.ref_pi, c) : (R)pi_s[c];
    const R pi = o.exner_offset ? pi0 + pis : pis;
    const R p = (R)kP0 * rpow(rmax(pi, (R)1.0e-3), (R)1 / (R)kKappaPhys);
    R theta = mixed ? tot<R>(th_s, a.ref_theta, c) : (R)th_s[c];
    R qv = rmax((R)qv_s[c], (R)0), qc = rmax((R)qc_s[c], (R)0), qr = rmax((R)qr_s[c], (R)0);
    R rho = mixed ? tot<R>(rho_s, a.ref_rho, c) : (R)rho_s[c];
    if (!(rho > (R)0)) {  // density from p and the virtual temperature
      const R qi = rmax((R)((const T*)a.state[QI])[c], (R)0), qsn = rmax((R)((const T*)a.state[QS])[c], (R)0),
              qg = rmax((R)((const T*)a.state[QG])[c], (R)0);
      const R tv = theta * exner_of(p) * ((R)1 + (R)0.608 * qv - qc - qi - qsn - qg);
      rho = p / ((R)kRd * tv);
    }
    const R th0 = theta, qv0 = qv, qc0 = qc, qr0 = qr;
    // 1. saturation adjustment
    adjust(qv, qc, theta, p);
    // 2. autoconversion + accretion
    {
      const R cq = rmax(qc, (R)0), rq = rmax(qr, (R)0);
      const R rate = o.k1 * rmax(cq - o.qc0, (R)0) + o.k2 * rmax(cq, (R)0) * rmax(rq, (R)0);
      const R dq = rmin(rate * dt, cq);
      qc = cq - dq;
      qr = rq + dq;
    }
    // 3. sedimentation: upstream flux from the level above, limited by the mass available
    {
      const R rh = rmax(rho, (R)1.0e-6), d = rmax(dz, (R)1.0e-6), rq = rmax(qr, (R)0);
      const R mass = rh * rq * d;
      const R vt = fall_speed(o, rh, rq);
      const R available = mass + flux_in * dt;
      const R out = rmin(rh * rq * vt * dt, rmax(available, (R)0));
      qr = rmax(available - out, (R)0) / (rh * d);
      flux_in = out / dt;
    }
    // 4. rain evaporation into subsaturated air
    {
      const R rq = rmax(qr, (R)0);
      if (rq > (R)0) {
        const R pk = exner_of(p);
        const R t = theta * pk;
        const R qs = qsat(p, t);
        const R v = rmax(qv, (R)0);
        if (v < qs) {
          R evap = evap_rate(o, t, rho, v, qs, rq) * dt;
          evap = rmin(evap, rq);
          const R lv = latent_v(t);
          const R cap = (qs - v) / ((R)1 + lv * lv * qs / ((R)kCp * (R)kRv * t * t));
          evap = rmin(evap, rmax(cap, (R)0));
          if (evap > (R)0) {
            qr = rq - evap;
            qv = v + evap;
            theta = theta - lv * evap / ((R)kCp * pk);
          }
        }
      }
    }
    // 5. positivity
    if (o.positive_definite) {
      qv = rmax(qv, (R)0);
      qc = rmax(qc, (R)0);
      qr = rmax(qr, (R)0);
    }
    // PhysicsTendency (accumulated onto the zeroed buffers)
    t_th[c] += (T)((theta - th0) / dt);
    t_qv[c] += (T)((qv - qv0) / dt);
    t_qc[c] += (T)((qc - qc0) / dt);
    t_qr[c] += (T)((qr - qr0) / dt);
  }
}

template <class R>
KesslerParams<R> params_of(const vibe_gb300_kessler& k) {
  KesslerParams<R> o;
  o.qc0 = (R)k.qc0;
  o.k1 = (R)k.k1;
  o.k2 = (R)k.k2;
  o.evap_coef = (R)k.evap_coef;
  o.rain_a = (R)k.rain_a;
  o.rain_b = (R)k.rain_b;
  o.rain_num = (R)(kPi / 6.0 * kRhoWater * kRainN0 * std::tgamma(1.0 + kRainB));
  o.cbrt_sc = (R)std::cbrt(kSchmidt);
  o.positive_definite = k.positive_definite;
  o.exner_offset = k.exner_offset;
  return o;
}

}  // namespace
}  // namespace vgb

using namespace vgb;

extern "C" {

void vibe_gb300_kessler_defaults(vibe_gb300_kessler* k) {  // PhysicsOptions, physics_types.hpp:420-429
  if (!k) return;
  k->qc0 = 1.0e-3;
  k->k1 = 1.0e-3;
  k->k2 = 2.2;
  k->evap_coef = 1.0;
  k->rain_a = 36.34;
  k->rain_b = 0.1364;
  k->positive_definite = 1;
  k->exner_offset = 1;
}

int vibe_gb300_physics_kessler(void* user, vibe_gb300_physics_args* a) {
  if (!user || !a || a->nx <= 0 || a->ny <= 0 || a->nz <= 0) return VIBE_GB300_EBADARG;
  if (!a->moist) return VIBE_GB300_EUNSUPPORTED;  // qc and qr must be prognostic
  for (int q : {THETA, PI, RHO, QV, QC, QR, QI, QS, QG})
    if (!a->state[q]) return VIBE_GB300_EUNSUPPORTED;  // needs the moisture species
  for (int q : {THETA, QV, QC, QR})
    if (!a->tend[q]) return VIBE_GB300_EBADARG;
  const vibe_gb300_kessler& k = *static_cast<const vibe_gb300_kessler*>(user);
  const dim3 b(32, 4), g((a->nx + 31) / 32, (a->ny + 3) / 4);
  cudaStream_t s = static_cast<cudaStream_t>(a->stream);
  a->written = (1u << THETA) | (1u << QV) | (1u << QC) | (1u << QR);
  if (a->precision == VIBE_GB300_MIXED) k_kessler<float, float><<<g, b, 0, s>>>(*a, params_of<float>(k));
  else k_kessler<double, double><<<g, b, 0, s>>>(*a, params_of<double>(k));
  return cudaGetLastError() == cudaSuccess ? 0 : VIBE_GB300_EDEVICE;
}

}  // extern "C"
