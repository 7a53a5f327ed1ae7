// vibe-model_gb300/csrc/diag.cu
//
// Time-step diagnostics of the device state, FP64, one pass:
//   Advection::cfl_number(s, dt)          (src/dyn/advection.cpp:325-340)
//   Equations::max_sound_speed(s)         (src/dyn/equations.cpp:238-249)
//   AcousticSubstepper::acoustic_cfl      (src/time/acoustic_substep.cpp:151-168)
//   max over cells of 1/dx + 1/dy + 1/dz  (the acoustic rate of
//                                          RungeKutta3Integrator::max_stable_dt,
//                                          src/time/runge_kutta.cpp:121-140,
//                                          is max sound speed times this)
// Every quantity is a maximum of non-negative doubles, reduced with an
// integer atomicMax on the IEEE bit pattern (monotonic for x >= 0), so the
// result does not depend on the reduction order and equals the serial loop's.
#include "step_kernels.cuh"

namespace vgb {
namespace {

__device__ __forceinline__ void amax(unsigned long long* slot, double v) {
  atomicMax(slot, (unsigned long long)__double_as_longlong(v));
}

__global__ void k_cfl(Dims d, Metric met, const double* __restrict__ u, const double* __restrict__ v,
                      const double* __restrict__ w, const double* __restrict__ th, const double* __restrict__ pi,
                      double dt, double dtau, unsigned long long* out) {
  const size_t n = (size_t)d.nx * d.ny * d.nz;
  double adv = 0.0, cs_max = 0.0, ac = 0.0, rate = 0.0;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(q % d.nx);
    const size_t qj = q / d.nx;
    const int j = (int)(qj % d.ny), k = (int)(qj / d.ny);
    const size_t c = d.idx(i, j, k);
    const double dx = met.dx, dy = met.dy;
    const double dz = dmax(met.dzeta[k] * met.scale[(size_t)j * d.nx + i], 1.0);
    const double uu = 0.5 * (u[c] + u[d.idx(i + 1, j, k)]);
    const double vv = 0.5 * (v[c] + v[d.idx(i, j + 1, k)]);
    const double ww = 0.5 * (w[c] + w[d.idx(i, j, k + 1)]);
    adv = dmax(adv, dt * (fabs(uu) / dx + fabs(vv) / dy + fabs(ww) / dz));
    const double t = th[c] * pi[c];
    const double cs = sqrt((kCp / kCv) * kRd * dmax(t, 1.0));
    cs_max = dmax(cs_max, cs);
    ac = dmax(ac, dtau * ((cs + fabs(uu)) / dx + (cs + fabs(vv)) / dy + (cs + fabs(ww)) / dz));
    rate = dmax(rate, 1.0 / dx + 1.0 / dy + 1.0 / dz);
  }
  amax(out + 0, adv);
  amax(out + 1, cs_max);
  amax(out + 2, ac);
  amax(out + 3, rate);
}

}  // namespace

void diag_cfl(const Dims& d, const Metric& met, double* const* st, double dt, double dtau, unsigned long long* out,
              cudaStream_t s) {
  const size_t n = (size_t)d.nx * d.ny * d.nz;
  const int blocks = (int)((n + 255) / 256 < 2048 ? (n + 255) / 256 : 2048);
  cudaMemsetAsync(out, 0, 4 * sizeof(unsigned long long), s);
  k_cfl<<<blocks > 0 ? blocks : 1, 256, 0, s>>>(d, met, st[U], st[V], st[W], st[THETA], st[PI], dt, dtau, out);
}

}  // namespace vgb
