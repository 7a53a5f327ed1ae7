/* oracle/vibe_oracle.c -- TEST INFRASTRUCTURE ONLY.
 *
 * Plain-C, serial, FP64 restatement of the VIBE-Model dynamics step as the
 * reference's source computes it. Every routine cites the reference
 * file:line it follows and keeps that code's floating-point operation order,
 * so that, built with -ffp-contract=off, it reproduces the reference compiled
 * unchanged (oracle/_ref) bit for bit in pgf_perturbation=0 mode.
 *
 * Used only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg, always as the checker -- never on the product path.
 */
#include "vibe_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* include/vibe/common/constants.hpp:16-60 */
#define K_GRAVITY 9.80665
#define K_RD 287.05
#define K_CP 1004.64
#define K_CV 717.63
#define K_EPS_VAP 0.62197
#define K_P0 100000.0
#define K_PI 3.14159265358979323846
#define K_OMEGA 7.2921159e-5
#define K_EARTH_RADIUS 6.371229e6
#define K_DEG2RAD (K_PI / 180.0)
#define K_BUOY_MOIST 0.608 /* equations.cpp:40 */

/* std::max / std::min / clamp semantics (include/vibe/common/types.hpp:83) */
static inline double dmax(double a, double b) { return (a < b) ? b : a; }
static inline double dmin(double a, double b) { return (b < a) ? b : a; }
static inline int imax(int a, int b) { return (a < b) ? b : a; }
static inline int imin(int a, int b) { return (b < a) ? b : a; }
static inline int iclamp(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }
static inline double sqr(double x) { return x * x; }
static inline double lerp(double a, double b, double w) { return a + w * (b - a); }

/* ------------------------------------------------------------------------ */
/* field storage: include/vibe/grid/field.hpp:40-96                          */
/* ------------------------------------------------------------------------ */
typedef struct {
  int nx, ny, nz;    /* grid interior sizes (same for every stagger) */
  int nsx, nsy, nsz; /* storage sizes incl. halo and the +1 face     */
  double *d;
} fld;

static void fld_alloc(fld *f, int nx, int ny, int nz, int stagger) {
  f->nx = nx; f->ny = ny; f->nz = nz;
  f->nsx = nx + 2 * VO_HALO + (stagger == 1);
  f->nsy = ny + 2 * VO_HALO + (stagger == 2);
  f->nsz = nz + 2 * VO_HALO + (stagger == 3);
  f->d = (double *)calloc((size_t)f->nsx * f->nsy * f->nsz, sizeof(double));
}
static size_t fld_size(const fld *f) { return (size_t)f->nsx * f->nsy * f->nsz; }
static void fld_zero(fld *f) { memset(f->d, 0, fld_size(f) * sizeof(double)); }
/* FieldT::offset (field.hpp:77-81) */
#define AT(f, i, j, k) \
  ((f).d[(size_t)((((k) + VO_HALO) * (f).nsy + ((j) + VO_HALO)) * (f).nsx + ((i) + VO_HALO))])
/* FieldT::clamp_at (field.hpp:91-96): clamps to the CELL interior for every stagger */
static inline double CL(const fld *f, int i, int j, int k) {
  return AT(*f, iclamp(i, 0, f->nx - 1), iclamp(j, 0, f->ny - 1), iclamp(k, 0, f->nz - 1));
}

static int stagger_of(int sp) { return sp == VO_U ? 1 : sp == VO_V ? 2 : sp == VO_W ? 3 : 0; }

struct vo_model {
  vo_setup s;
  int nx, ny, nz;
  double *zeta;   /* nz+1 */
  double *zs;     /* nx*ny terrain */
  double *sponge; /* nz */
  fld st[VO_NSPECIES];
  fld s0[VO_NSPECIES];
  fld slow[VO_NSPECIES];
  fld scr[VO_NSPECIES];
  fld ref[5];     /* theta0, pi0, rho0, p0, qv0 */
  double f0, beta;
  int physics;            /* 1: Kessler coupled into vo_rk3_step */
  vo_kessler kessler;
};

/* ------------------------------------------------------------------------ */
/* grid metrics: src/grid/geometry.cpp                                      */
/* ------------------------------------------------------------------------ */

/* make_stretched_zeta, geometry.cpp:39-60 */
static void make_stretched_zeta(int nz, double first, double stretch, double *zeta) {
  double *dz = (double *)malloc(sizeof(double) * (size_t)nz);
  double total = 0.0, h = first, acc = 0.0;
  for (int k = 0; k < nz; ++k) { dz[k] = h; total += h; h *= stretch; }
  zeta[0] = 0.0;
  for (int k = 0; k < nz; ++k) { acc += dz[k]; zeta[k + 1] = acc / total; }
  zeta[nz] = 1.0;
  free(dz);
}

/* Grid::dzeta, geometry.cpp:242-245 */
static inline double g_dzeta(const vo_model *m, int k) {
  const int kk = iclamp(k, 0, m->nz - 1);
  return m->zeta[kk + 1] - m->zeta[kk];
}
/* Grid::terrain, geometry.cpp:247-253 */
static inline double g_terrain(const vo_model *m, int i, int j) {
  return m->zs[(size_t)iclamp(j, 0, m->ny - 1) * m->nx + iclamp(i, 0, m->nx - 1)];
}
/* zeta_at, geometry.cpp:20-31 */
static double zeta_at(const vo_model *m, double kk) {
  const int nz = m->nz;
  if (kk <= 0.0) return m->zeta[0];
  if (kk >= (double)nz) return m->zeta[nz];
  const int k0 = (int)floor(kk);
  const double frac = kk - (double)k0;
  if (frac == 0.0) return m->zeta[k0];
  if (fabs(frac - 0.5) < 1e-12) return 0.5 * (m->zeta[k0] + m->zeta[k0 + 1]);
  return lerp(m->zeta[k0], m->zeta[k0 + 1], frac);
}
/* Grid::height, geometry.cpp:260-263; z_center/z_interface geometry.hpp:135-139 */
static double g_height(const vo_model *m, int i, int j, double kk) {
  const double zs = g_terrain(m, i, j);
  return zs + zeta_at(m, kk) * (m->s.z_top - zs);
}
static double g_zc(const vo_model *m, int i, int j, int k) { return g_height(m, i, j, (double)k + 0.5); }

/* ------------------------------------------------------------------------ */
/* reference state: src/dyn/reference_state.cpp                             */
/* ------------------------------------------------------------------------ */
static double density_from(double pi0, double theta0) { /* :26-28 */
  return K_P0 * pow(pi0, K_CV / K_RD) / (K_RD * theta0);
}
static double pressure_from(double pi0) { return K_P0 * pow(pi0, K_CP / K_RD); } /* :31 */

static void ref_isothermal(vo_model *m) { /* :35-59 */
  const double th = m->s.theta0;
  const double pi_surf = pow(m->s.p_surf / K_P0, K_RD / K_CP);
  for (int k = 0; k < m->nz; ++k)
    for (int j = 0; j < m->ny; ++j)
      for (int i = 0; i < m->nx; ++i) {
        const double z = g_zc(m, i, j, k);
        const double pi = pi_surf - K_GRAVITY * z / (K_CP * th);
        AT(m->ref[VO_THETA0], i, j, k) = th;
        AT(m->ref[VO_PI0], i, j, k) = pi;
        AT(m->ref[VO_P0], i, j, k) = pressure_from(pi);
        AT(m->ref[VO_RHO0], i, j, k) = density_from(pi, th);
        AT(m->ref[VO_QV0], i, j, k) = 0.0;
      }
}

static void ref_from_profile(vo_model *m) { /* :61-110 */
  const int np = (int)ceil(m->s.z_top / m->s.profile_dz) + 2;
  double *z = (double *)malloc(sizeof(double) * (size_t)np);
  double *th = (double *)malloc(sizeof(double) * (size_t)np);
  double *zi = (double *)malloc(sizeof(double) * (size_t)(m->nz + 1));
  for (int p = 0; p < np; ++p) {
    z[p] = (double)p * m->s.profile_dz;
    th[p] = m->s.theta0 * exp(m->s.bv_n * m->s.bv_n * z[p] / K_GRAVITY);
  }
  const double pi_surf = pow(m->s.p_surf / K_P0, K_RD / K_CP);
#define THETA_AT(zz, out)                                                   \
  do {                                                                      \
    const double zz_ = (zz);                                                \
    if (zz_ <= z[0]) { out = th[0]; }                                       \
    else if (zz_ >= z[np - 1]) { out = th[np - 1]; }                        \
    else {                                                                  \
      size_t kk_ = 0;                                                       \
      while (kk_ + 2 < (size_t)np && z[kk_ + 1] < zz_) ++kk_;               \
      const double w_ = (z[kk_ + 1] - z[kk_] > 0.0)                         \
                            ? (zz_ - z[kk_]) / (z[kk_ + 1] - z[kk_]) : 0.0; \
      out = lerp(th[kk_], th[kk_ + 1], w_);                                 \
    }                                                                       \
  } while (0)
  for (int j = 0; j < m->ny; ++j)
    for (int i = 0; i < m->nx; ++i) {
      for (int k = 0; k <= m->nz; ++k) zi[k] = g_height(m, i, j, (double)k);
      double pi = pi_surf, th_surf;
      THETA_AT(zi[0], th_surf);
      AT(m->ref[VO_THETA0], i, j, 0) = th_surf;
      for (int k = 0; k < m->nz; ++k) {
        double th_lo, th_hi;
        THETA_AT(zi[k], th_lo);
        THETA_AT(zi[k + 1], th_hi);
        const double th_mid = 0.5 * (th_lo + th_hi);
        const double dz = zi[k + 1] - zi[k];
        pi -= K_GRAVITY * dz / (K_CP * th_mid);
        const double th_c = 0.5 * (th_lo + th_hi);
        AT(m->ref[VO_THETA0], i, j, k) = th_c;
        AT(m->ref[VO_PI0], i, j, k) = pi;
        AT(m->ref[VO_P0], i, j, k) = pressure_from(pi);
        AT(m->ref[VO_RHO0], i, j, k) = density_from(pi, th_c);
        AT(m->ref[VO_QV0], i, j, k) = 0.0;
      }
    }
#undef THETA_AT
  free(z); free(th); free(zi);
}

/* ------------------------------------------------------------------------ */
/* initial conditions: src/driver/initial_conditions.cpp                     */
/* ------------------------------------------------------------------------ */
static void enforce_state_equation(vo_model *m) { /* :110-121 */
  for (int k = 0; k < m->nz; ++k)
    for (int j = 0; j < m->ny; ++j)
      for (int i = 0; i < m->nx; ++i) {
        const double qv = dmax(AT(m->st[VO_QV], i, j, k), 0.0);
        const double gamma_f = (1.0 + qv / K_EPS_VAP) / (1.0 + qv);
        const double val = AT(m->st[VO_RHO], i, j, k) * K_RD * AT(m->st[VO_THETA], i, j, k) * gamma_f / K_P0;
        if (val > 0.0) AT(m->st[VO_PI], i, j, k) = pow(val, K_RD / K_CV);
      }
}

static void init_warm_bubble(vo_model *m) { /* :136-159 with fill_base_state :66-91 */
  const vo_setup *s = &m->s;
  for (int k = 0; k < m->nz; ++k)
    for (int j = 0; j < m->ny; ++j)
      for (int i = 0; i < m->nx; ++i) {
        const double z = g_zc(m, i, j, k);
        AT(m->st[VO_THETA], i, j, k) = AT(m->ref[VO_THETA0], i, j, k);
        AT(m->st[VO_PI], i, j, k) = AT(m->ref[VO_PI0], i, j, k);
        AT(m->st[VO_RHO], i, j, k) = AT(m->ref[VO_RHO0], i, j, k);
        AT(m->st[VO_QV], i, j, k) = s->qv_surface * exp(-dmax(z, 0.0) / s->qv_decay_height);
        for (int sp = VO_QC; sp <= VO_QG; ++sp) AT(m->st[sp], i, j, k) = 0.0;
      }
  fld_zero(&m->st[VO_U]); fld_zero(&m->st[VO_V]); fld_zero(&m->st[VO_W]);
  const double xc = (s->bubble_xc != 0.0) ? s->bubble_xc : 0.5 * 0.0 + 0.5 * (double)m->nx * s->dx;
  const double yc = (s->bubble_yc != 0.0) ? s->bubble_yc : 0.5 * (double)m->ny * s->dy;
  for (int k = 0; k < m->nz; ++k)
    for (int j = 0; j < m->ny; ++j)
      for (int i = 0; i < m->nx; ++i) {
        const double x = (0 + (double)i + 0.5) * s->dx;
        const double y = (0 + (double)j + 0.5) * s->dy;
        const double z = g_zc(m, i, j, k);
        const double r2 = sqr((x - xc) / s->bubble_radius_x) + sqr((y - yc) / s->bubble_radius_x) +
                          sqr((z - s->bubble_zc) / s->bubble_radius_z);
        if (r2 < 1.0) {
          const double c = cos(0.5 * K_PI * sqrt(r2));
          AT(m->st[VO_THETA], i, j, k) += s->bubble_amplitude * c * c;
        }
      }
  /* apply_shear :94-102 */
  for (int k = 0; k < m->nz; ++k)
    for (int j = 0; j < m->ny; ++j)
      for (int i = 0; i <= m->nx; ++i) {
        const double z = g_zc(m, imin(i, m->nx - 1), j, k);
        AT(m->st[VO_U], i, j, k) = s->u_background + s->shear_u * z;
      }
  enforce_state_equation(m);
}

/* ------------------------------------------------------------------------ */
/* advection: src/dyn/advection.cpp                                          */
/* ------------------------------------------------------------------------ */

/* Advection::weno5_reconstruct, advection.cpp:62-98 */
static void weno5(double qm2, double qm1, double q0, double q1, double q2, double *ql, double *qr) {
  const double eps = 1e-6;
  const double d0 = 0.1, d1 = 0.6, d2 = 0.3;
  const double v0 = (2.0 * qm2 - 7.0 * qm1 + 11.0 * q0) / 6.0;
  const double v1 = (-qm1 + 5.0 * q0 + 2.0 * q1) / 6.0;
  const double v2 = (2.0 * q0 + 5.0 * q1 - q2) / 6.0;
  const double b0 = (13.0 / 12.0) * sqr(qm2 - 2.0 * qm1 + q0) + 0.25 * sqr(qm2 - 4.0 * qm1 + 3.0 * q0);
  const double b1 = (13.0 / 12.0) * sqr(qm1 - 2.0 * q0 + q1) + 0.25 * sqr(qm1 - q1);
  const double b2 = (13.0 / 12.0) * sqr(q0 - 2.0 * q1 + q2) + 0.25 * sqr(3.0 * q0 - 4.0 * q1 + q2);
  const double a0 = d0 / sqr(eps + b0);
  const double a1 = d1 / sqr(eps + b1);
  const double a2 = d2 / sqr(eps + b2);
  const double wsum = a0 + a1 + a2;
  *ql = (a0 * v0 + a1 * v1 + a2 * v2) / wsum;
  const double u0 = (2.0 * q2 - 7.0 * q1 + 11.0 * q0) / 6.0;
  const double u1 = (-q1 + 5.0 * q0 + 2.0 * qm1) / 6.0;
  const double u2 = (2.0 * q0 + 5.0 * qm1 - qm2) / 6.0;
  const double g0 = (13.0 / 12.0) * sqr(q2 - 2.0 * q1 + q0) + 0.25 * sqr(q2 - 4.0 * q1 + 3.0 * q0);
  const double g1 = (13.0 / 12.0) * sqr(q1 - 2.0 * q0 + qm1) + 0.25 * sqr(q1 - qm1);
  const double g2 = (13.0 / 12.0) * sqr(q0 - 2.0 * qm1 + qm2) + 0.25 * sqr(3.0 * q0 - 4.0 * qm1 + qm2);
  const double c0 = d0 / sqr(eps + g0);
  const double c1 = d1 / sqr(eps + g1);
  const double c2 = d2 / sqr(eps + g2);
  const double wsum2 = c0 + c1 + c2;
  *qr = (c0 * u0 + c1 * u1 + c2 * u2) / wsum2;
}

/* reconstruct_face lambda with local Lax-Friedrichs split, advection.cpp:151-156 */
static inline double weno_face(double qm2, double qm1, double q0, double q1, double q2, double vel) {
  double ql, qr;
  weno5(qm2, qm1, q0, q1, q2, &ql, &qr);
  const double alpha = dmax(fabs(vel), 1e-3);
  return 0.5 * (vel * (ql + qr) - alpha * (qr - ql));
}

/* Advection::scalar, WENO5 branch, advection.cpp:144-187 */
static void advect_weno5(const vo_model *m, const fld *q, const fld *u, const fld *v, const fld *w, fld *dq) {
  const int nx = m->nx, ny = m->ny, nz = m->nz;
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const double dx = m->s.dx, dy = m->s.dy;
        const double dz = g_dzeta(m, k) * (m->s.z_top - g_terrain(m, i, j));
        const double fe = weno_face(CL(q, i - 2, j, k), CL(q, i - 1, j, k), AT(*q, i, j, k),
                                    CL(q, i + 1, j, k), CL(q, i + 2, j, k), AT(*u, i + 1, j, k));
        const double fw = weno_face(CL(q, i - 3, j, k), CL(q, i - 2, j, k), CL(q, i - 1, j, k),
                                    AT(*q, i, j, k), CL(q, i + 1, j, k), AT(*u, i, j, k));
        const double fn = weno_face(CL(q, i, j - 2, k), CL(q, i, j - 1, k), AT(*q, i, j, k),
                                    CL(q, i, j + 1, k), CL(q, i, j + 2, k), AT(*v, i, j + 1, k));
        const double fs = weno_face(CL(q, i, j - 3, k), CL(q, i, j - 2, k), CL(q, i, j - 1, k),
                                    AT(*q, i, j, k), CL(q, i, j + 1, k), AT(*v, i, j, k));
        double ft = 0.0, fb = 0.0;
        if (k + 2 < nz || k >= 2) {
          ft = weno_face(CL(q, i, j, k - 2), CL(q, i, j, k - 1), AT(*q, i, j, k),
                         CL(q, i, j, k + 1), CL(q, i, j, k + 2), AT(*w, i, j, k + 1));
          fb = weno_face(CL(q, i, j, k - 3), CL(q, i, j, k - 2), CL(q, i, j, k - 1),
                         AT(*q, i, j, k), CL(q, i, j, k + 1), AT(*w, i, j, k));
        }
        AT(*dq, i, j, k) = -(fe - fw) / dx - (fn - fs) / dy - (ft - fb) / dz;
        if (m->s.weno_advective) {
          double div = (AT(*u, i + 1, j, k) - AT(*u, i, j, k)) / dx + (AT(*v, i, j + 1, k) - AT(*v, i, j, k)) / dy;
          if (k + 2 < nz || k >= 2) div += (AT(*w, i, j, k + 1) - AT(*w, i, j, k)) / dz;
          AT(*dq, i, j, k) += AT(*q, i, j, k) * div;
        }
      }
}

/* grad_x / grad_y, advection.cpp:106-136 */
static inline double grad_x(const fld *q, int i, int j, int k, double inv_dx, int order) {
  switch (order) {
    case 4:
      return (CL(q, i - 2, j, k) - 8.0 * CL(q, i - 1, j, k) + 8.0 * CL(q, i + 1, j, k) - CL(q, i + 2, j, k)) *
             (inv_dx / 12.0);
    case 6:
      return (-CL(q, i - 3, j, k) + 9.0 * CL(q, i - 2, j, k) - 45.0 * CL(q, i - 1, j, k) +
              45.0 * CL(q, i + 1, j, k) - 9.0 * CL(q, i + 2, j, k) + CL(q, i + 3, j, k)) *
             (inv_dx / 60.0);
    default:
      return (CL(q, i + 1, j, k) - CL(q, i - 1, j, k)) * (0.5 * inv_dx);
  }
}
static inline double grad_y(const fld *q, int i, int j, int k, double inv_dy, int order) {
  switch (order) {
    case 4:
      return (CL(q, i, j - 2, k) - 8.0 * CL(q, i, j - 1, k) + 8.0 * CL(q, i, j + 1, k) - CL(q, i, j + 2, k)) *
             (inv_dy / 12.0);
    case 6:
      return (-CL(q, i, j - 3, k) + 9.0 * CL(q, i, j - 2, k) - 45.0 * CL(q, i, j - 1, k) +
              45.0 * CL(q, i, j + 1, k) - 9.0 * CL(q, i, j + 2, k) + CL(q, i, j + 3, k)) *
             (inv_dy / 60.0);
    default:
      return (CL(q, i, j + 1, k) - CL(q, i, j - 1, k)) * (0.5 * inv_dy);
  }
}

/* Advection constructor order_ (advection.cpp:44-52): weno5 -> 5, which the
 * switches above treat as 2nd order. */
static int adv_order(const vo_model *m) { return m->s.advection; }

/* Advection::scalar_nonconservative, advection.cpp:224-244 */
static void advect_nonconservative(const vo_model *m, const fld *q, const fld *u, const fld *v, const fld *w, fld *dq) {
  const int order = adv_order(m);
  for (int k = 0; k < m->nz; ++k)
    for (int j = 0; j < m->ny; ++j)
      for (int i = 0; i < m->nx; ++i) {
        const double dx = m->s.dx, dy = m->s.dy;
        const double scale = m->s.z_top - g_terrain(m, i, j);
        const double dz = g_dzeta(m, k) * scale;
        const double ua = 0.5 * (AT(*u, i, j, k) + AT(*u, i + 1, j, k));
        const double va = 0.5 * (AT(*v, i, j, k) + AT(*v, i, j + 1, k));
        const double wa = 0.5 * (AT(*w, i, j, k) + AT(*w, i, j, k + 1));
        AT(*dq, i, j, k) = -(ua * grad_x(q, i, j, k, 1.0 / dx, order) + va * grad_y(q, i, j, k, 1.0 / dy, order) +
                             wa * (CL(q, i, j, k + 1) - CL(q, i, j, k - 1)) * (0.5 / dz));
      }
}

/* Advection::momentum, advection.cpp:250-319 */
static void advect_momentum(const vo_model *m, fld *st, fld *d) {
  const int nx = m->nx, ny = m->ny, nz = m->nz;
  const fld *u = &st[VO_U], *v = &st[VO_V], *w = &st[VO_W];
  fld *du = &d[VO_U], *dv = &d[VO_V], *dw = &d[VO_W];
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i <= nx; ++i) {
        const int ip = imin(i, nx - 1);
        const double dx = m->s.dx, dy = m->s.dy;
        const double scale = m->s.z_top - g_terrain(m, ip, j);
        const double dz = g_dzeta(m, imin(k, nz - 1)) * scale;
        const double uc = 0.5 * (AT(*u, imax(i - 1, 0), j, k) + AT(*u, ip, j, k));
        const double ux = (AT(*u, ip, j, k) - AT(*u, imax(i - 1, 0), j, k)) / dx;
        const double uy = (AT(*u, ip, imin(j + 1, ny - 1), k) - AT(*u, ip, imax(j - 1, 0), k)) / (2.0 * dy);
        const double uz = (AT(*u, ip, j, imin(k + 1, nz - 1)) - AT(*u, ip, j, imax(k - 1, 0))) / (2.0 * dz);
        const double vc = 0.25 * (AT(*v, imax(i - 1, 0), imax(j - 1, 0), k) + AT(*v, ip, imax(j - 1, 0), k) +
                                  AT(*v, imax(i - 1, 0), j, k) + AT(*v, ip, j, k));
        const double wc = 0.5 * (AT(*w, ip, j, k) + AT(*w, ip, j, imin(k + 1, nz - 1)));
        AT(*du, i, j, k) -= uc * ux + vc * uy + wc * uz;
      }
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j <= ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const int jp = imin(j, ny - 1);
        const double dx = m->s.dx, dy = m->s.dy;
        const double scale = m->s.z_top - g_terrain(m, i, jp);
        const double dz = g_dzeta(m, imin(k, nz - 1)) * scale;
        const double vc = 0.5 * (AT(*v, i, imax(j - 1, 0), k) + AT(*v, i, jp, k));
        const double vy = (AT(*v, i, jp, k) - AT(*v, i, imax(j - 1, 0), k)) / dy;
        const double vx = (AT(*v, imin(i + 1, nx - 1), jp, k) - AT(*v, imax(i - 1, 0), jp, k)) / (2.0 * dx);
        const double vz = (AT(*v, i, jp, imin(k + 1, nz - 1)) - AT(*v, i, jp, imax(k - 1, 0))) / (2.0 * dz);
        const double uc = 0.25 * (AT(*u, imax(i - 1, 0), imax(j - 1, 0), k) + AT(*u, i, imax(j - 1, 0), k) +
                                  AT(*u, imax(i - 1, 0), jp, k) + AT(*u, i, jp, k));
        const double wc = 0.5 * (AT(*w, i, jp, k) + AT(*w, i, jp, imin(k + 1, nz - 1)));
        AT(*dv, i, j, k) -= uc * vx + vc * vy + wc * vz;
      }
  for (int k = 0; k <= nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const int kc = imin(imax(k, 0), nz - 1);
        const double dx = m->s.dx, dy = m->s.dy;
        const double scale = m->s.z_top - g_terrain(m, i, j);
        const double dz = g_dzeta(m, kc) * scale;
        const double wc = 0.5 * (AT(*w, i, j, kc) + AT(*w, i, j, imin(k, nz)));
        const double wz = (AT(*w, i, j, imin(k, nz)) - AT(*w, i, j, imax(k - 1, 0))) / dz;
        const double wx = (AT(*w, imin(i + 1, nx - 1), j, imin(k, nz)) - AT(*w, imax(i - 1, 0), j, imin(k, nz))) / (2.0 * dx);
        const double wy = (AT(*w, i, imin(j + 1, ny - 1), imin(k, nz)) - AT(*w, i, imax(j - 1, 0), imin(k, nz))) / (2.0 * dy);
        const double uc = 0.5 * (AT(*u, i, j, kc) + AT(*u, i + 1, j, kc));
        const double vc = 0.5 * (AT(*v, i, j, kc) + AT(*v, i, j + 1, kc));
        AT(*dw, i, j, k) -= uc * wx + vc * wy + wc * wz;
      }
}

/* Coriolis::f_at / apply, coriolis.cpp:25-70 */
static double cor_f(const vo_model *m, int j) {
  if (m->s.coriolis != 2) return m->f0;
  const double y = (0.0 + (double)j + 0.5) * m->s.dy;
  const double y0 = 0.5 * (double)m->ny * m->s.dy;
  return m->f0 + m->beta * (y - y0);
}
static void coriolis_apply(const vo_model *m, fld *st, fld *d) {
  if (m->s.coriolis == 0) return;
  const int nx = m->nx, ny = m->ny, nz = m->nz;
  const fld *u = &st[VO_U], *v = &st[VO_V];
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i <= nx; ++i) {
        const double v_at_u = 0.25 * (AT(*v, imax(i - 1, 0), imax(j - 1, 0), k) + AT(*v, imin(i, nx - 1), imax(j - 1, 0), k) +
                                      AT(*v, imax(i - 1, 0), j, k) + AT(*v, imin(i, nx - 1), j, k));
        AT(d[VO_U], i, j, k) += cor_f(m, j) * v_at_u;
      }
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j <= ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const double u_at_v = 0.25 * (AT(*u, imax(i - 1, 0), imax(j - 1, 0), k) + AT(*u, i, imax(j - 1, 0), k) +
                                      AT(*u, imax(i - 1, 0), imin(j, ny - 1), k) + AT(*u, i, imin(j, ny - 1), k));
        AT(d[VO_V], i, j, k) -= cor_f(m, j) * u_at_v;
      }
}

/* Damping::tendencies (divergence damping), damping.cpp:43-74 */
static double lap2(const vo_model *m, const fld *f, int i, int j, int k) {
  const double dx = m->s.dx, dy = m->s.dy;
  return (CL(f, i + 1, j, k) - 2.0 * AT(*f, i, j, k) + CL(f, i - 1, j, k)) / (dx * dx) +
         (CL(f, i, j + 1, k) - 2.0 * AT(*f, i, j, k) + CL(f, i, j - 1, k)) / (dy * dy);
}
static void damping_tendencies(const vo_model *m, fld *st, fld *d) {
  if (m->s.divergence_damping <= 0.0) return;
  const double nu = m->s.divergence_damping;
  const fld *pi = &st[VO_PI];
  if (m->s.divergence_order <= 2) {
    for (int k = 0; k < m->nz; ++k)
      for (int j = 0; j < m->ny; ++j)
        for (int i = 0; i < m->nx; ++i) AT(d[VO_PI], i, j, k) -= nu * lap2(m, pi, i, j, k);
  } else {
    fld tmp;
    fld_alloc(&tmp, m->nx, m->ny, m->nz, 0);
    for (int k = 0; k < m->nz; ++k)
      for (int j = 0; j < m->ny; ++j)
        for (int i = 0; i < m->nx; ++i) AT(tmp, i, j, k) = lap2(m, pi, i, j, k);
    for (int k = 0; k < m->nz; ++k)
      for (int j = 0; j < m->ny; ++j)
        for (int i = 0; i < m->nx; ++i) AT(d[VO_PI], i, j, k) -= nu * lap2(m, &tmp, i, j, k);
    free(tmp.d);
  }
}

/* Exner difference used by every pressure-gradient term: total pi as the
 * reference code computes it, or pi' = pi - pi0 in the documented form. */
static inline double dpi(const vo_model *m, const fld *pi, int ia, int ja, int ka, int ib, int jb, int kb) {
  if (!m->s.pgf_perturbation) return AT(*pi, ia, ja, ka) - AT(*pi, ib, jb, kb);
  return (AT(*pi, ia, ja, ka) - AT(m->ref[VO_PI0], ia, ja, ka)) -
         (AT(*pi, ib, jb, kb) - AT(m->ref[VO_PI0], ib, jb, kb));
}

/* Equations::tendencies, equations.cpp:60-150 (+ the O-WENO override of the
 * scalar advection when weno_scalars is set). */
static void slow_tendency(vo_model *m, fld *st, fld *d) {
  const int nx = m->nx, ny = m->ny, nz = m->nz;
  for (int sp = 0; sp < VO_NSPECIES; ++sp) fld_zero(&d[sp]);
  advect_momentum(m, st, d);
  coriolis_apply(m, st, d);
  damping_tendencies(m, st, d);
  const fld *th = &st[VO_THETA], *pi = &st[VO_PI], *rho = &st[VO_RHO];
  for (int k = 0; k < nz; ++k) /* :72-80 */
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i <= nx; ++i) {
        const int ip = imin(i, nx - 1), im = imax(i - 1, 0);
        const double dx = m->s.dx;
        const double t = 0.5 * (AT(*th, im, j, k) + AT(*th, ip, j, k));
        AT(d[VO_U], i, j, k) -= K_CP * t * dpi(m, pi, ip, j, k, im, j, k) / dx;
      }
  for (int k = 0; k < nz; ++k) /* :81-89 */
    for (int j = 0; j <= ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const int jp = imin(j, ny - 1), jm = imax(j - 1, 0);
        const double dy = m->s.dy;
        const double t = 0.5 * (AT(*th, i, jm, k) + AT(*th, i, jp, k));
        AT(d[VO_V], i, j, k) -= K_CP * t * dpi(m, pi, i, jp, k, i, jm, k) / dy;
      }
  for (int k = 0; k <= nz; ++k) /* :91-110 */
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const int kc = imin(imax(k, 0), nz - 1), km = imax(k - 1, 0);
        const double scale = m->s.z_top - g_terrain(m, i, j);
        const double dz = dmax(g_dzeta(m, kc) * scale, 1.0);
        const double t = 0.5 * (AT(*th, i, j, km) + AT(*th, i, j, kc));
        AT(d[VO_W], i, j, k) -= K_CP * t * dpi(m, pi, i, j, kc, i, j, km) / dz;
        const double th0 = AT(m->ref[VO_THETA0], i, j, kc);
        const double thp = AT(*th, i, j, kc) - th0;
        const double qcond = AT(st[VO_QC], i, j, kc) + AT(st[VO_QR], i, j, kc) + AT(st[VO_QI], i, j, kc) +
                             AT(st[VO_QS], i, j, kc) + AT(st[VO_QG], i, j, kc);
        AT(d[VO_W], i, j, k) += K_GRAVITY * (thp / dmax(th0, 1.0) + K_BUOY_MOIST * AT(st[VO_QV], i, j, kc) - qcond);
      }
  for (int k = 0; k < nz; ++k) /* :112-127 */
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const double dx = m->s.dx, dy = m->s.dy;
        const double scale = m->s.z_top - g_terrain(m, i, j);
        const double dz = dmax(g_dzeta(m, k) * scale, 1.0);
        const double fx = AT(st[VO_U], i + 1, j, k) * 0.5 * (AT(*rho, i, j, k) + AT(*rho, i + 1, j, k)) -
                          AT(st[VO_U], i, j, k) * 0.5 * (AT(*rho, imax(i - 1, 0), j, k) + AT(*rho, i, j, k));
        const double fy = AT(st[VO_V], i, j + 1, k) * 0.5 * (AT(*rho, i, j, k) + AT(*rho, i, j + 1, k)) -
                          AT(st[VO_V], i, j, k) * 0.5 * (AT(*rho, i, imax(j - 1, 0), k) + AT(*rho, i, j, k));
        const double fz = AT(st[VO_W], i, j, k + 1) * 0.5 * (AT(*rho, i, j, k) + AT(*rho, i, j, imin(k + 1, nz - 1))) -
                          AT(st[VO_W], i, j, k) * 0.5 * (AT(*rho, i, j, imax(k - 1, 0)) + AT(*rho, i, j, k));
        AT(d[VO_RHO], i, j, k) = -(fx / dx + fy / dy + fz / dz);
      }
  const int last = m->s.moist ? VO_QG : VO_QV;
  for (int sp = VO_THETA; sp <= last; ++sp) { /* :129-137 */
    if (sp == VO_PI) continue;
    if (m->s.weno_scalars)
      advect_weno5(m, &st[sp], &st[VO_U], &st[VO_V], &st[VO_W], &d[sp]);
    else
      advect_nonconservative(m, &st[sp], &st[VO_U], &st[VO_V], &st[VO_W], &d[sp]);
  }
  for (int sp = VO_QV; sp <= VO_QG; ++sp) /* :139-149 */
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i)
          if (AT(st[sp], i, j, k) <= 0.0 && AT(d[sp], i, j, k) < 0.0) AT(d[sp], i, j, k) = 0.0;
}

static void acoustic_tendencies(vo_model *m, fld *st, fld *d);

/* split_fast composition: remove the terms the substeps integrate
 * (acoustic_tendencies of the same input state) from the slow tendency of
 * u, v, w and rho. */
static void slow_tendency_split(vo_model *m, fld *st, fld *d) {
  slow_tendency(m, st, d);
  if (!m->s.split_fast) return;
  acoustic_tendencies(m, st, m->scr);
  const int sps[4] = {VO_U, VO_V, VO_W, VO_RHO};
  for (int q = 0; q < 4; ++q) {
    const size_t n = fld_size(&d[sps[q]]);
    for (size_t e = 0; e < n; ++e) d[sps[q]].d[e] -= m->scr[sps[q]].d[e];
  }
}

/* linear mass divergence -div(rho0 u) with the reference's rho0 clamps,
 * equations.cpp:187-200 (identical in acoustic_substep.cpp:71-85) */
static double mass_div0(const vo_model *m, const fld *st, int i, int j, int k) {
  const int nx = m->nx, ny = m->ny, nz = m->nz;
  const fld *r0 = &m->ref[VO_RHO0];
  const double dx = m->s.dx, dy = m->s.dy;
  const double scale = m->s.z_top - g_terrain(m, i, j);
  const double dz = dmax(g_dzeta(m, k) * scale, 1.0);
  const double fx = AT(st[VO_U], i + 1, j, k) * 0.5 * (AT(*r0, i, j, k) + AT(*r0, imin(i + 1, nx - 1), j, k)) -
                    AT(st[VO_U], i, j, k) * 0.5 * (AT(*r0, imax(i - 1, 0), j, k) + AT(*r0, i, j, k));
  const double fy = AT(st[VO_V], i, j + 1, k) * 0.5 * (AT(*r0, i, j, k) + AT(*r0, i, imin(j + 1, ny - 1), k)) -
                    AT(st[VO_V], i, j, k) * 0.5 * (AT(*r0, i, imax(j - 1, 0), k) + AT(*r0, i, j, k));
  const double fz = AT(st[VO_W], i, j, k + 1) * 0.5 * (AT(*r0, i, j, k) + AT(*r0, i, j, imin(k + 1, nz - 1))) -
                    AT(st[VO_W], i, j, k) * 0.5 * (AT(*r0, i, j, imax(k - 1, 0)) + AT(*r0, i, j, k));
  return -(fx / dx + fy / dy + fz / dz);
}

/* Equations::acoustic_tendencies, equations.cpp:152-209 */
static void acoustic_tendencies(vo_model *m, fld *st, fld *d) {
  const int nx = m->nx, ny = m->ny, nz = m->nz;
  const fld *th0 = &m->ref[VO_THETA0], *pi = &st[VO_PI];
  for (int sp = 0; sp < VO_NSPECIES; ++sp) fld_zero(&d[sp]);
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i <= nx; ++i) {
        const int ip = imin(i, nx - 1), im = imax(i - 1, 0);
        const double t0 = 0.5 * (AT(*th0, im, j, k) + AT(*th0, ip, j, k));
        AT(d[VO_U], i, j, k) = -K_CP * t0 * dpi(m, pi, ip, j, k, im, j, k) / m->s.dx;
      }
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j <= ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const int jp = imin(j, ny - 1), jm = imax(j - 1, 0);
        const double t0 = 0.5 * (AT(*th0, i, jm, k) + AT(*th0, i, jp, k));
        AT(d[VO_V], i, j, k) = -K_CP * t0 * dpi(m, pi, i, jp, k, i, jm, k) / m->s.dy;
      }
  for (int k = 0; k <= nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const int kc = imin(imax(k, 0), nz - 1), km = imax(k - 1, 0);
        const double scale = m->s.z_top - g_terrain(m, i, j);
        const double dz = dmax(g_dzeta(m, kc) * scale, 1.0);
        const double t0 = 0.5 * (AT(*th0, i, j, km) + AT(*th0, i, j, kc));
        AT(d[VO_W], i, j, k) = -K_CP * t0 * dpi(m, pi, i, j, kc, i, j, km) / dz;
      }
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) AT(d[VO_RHO], i, j, k) = mass_div0(m, st, i, j, k);
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const double r0 = dmax(AT(m->ref[VO_RHO0], i, j, k), 1e-8);
        AT(d[VO_PI], i, j, k) = (K_RD / K_CV) * (AT(m->ref[VO_PI0], i, j, k) / r0) * AT(d[VO_RHO], i, j, k);
      }
}

static void add_scaled(fld *f, double a, const fld *x) { /* FieldT::add_scaled, field.hpp:108-111 */
  const size_t n = fld_size(f);
  for (size_t q = 0; q < n; ++q) f->d[q] += a * x->d[q];
}

/* RungeKutta3Integrator::acoustic_substep, runge_kutta.cpp:65-75 */
static void fb_substep(vo_model *m, double dtau) {
  acoustic_tendencies(m, m->st, m->scr);
  add_scaled(&m->st[VO_RHO], dtau, &m->scr[VO_RHO]);
  add_scaled(&m->st[VO_PI], dtau, &m->scr[VO_PI]);
  acoustic_tendencies(m, m->st, m->scr);
  add_scaled(&m->st[VO_U], dtau, &m->scr[VO_U]);
  add_scaled(&m->st[VO_V], dtau, &m->scr[VO_V]);
  add_scaled(&m->st[VO_W], dtau, &m->scr[VO_W]);
}

/* ------------------------------------------------------------------------ */
/* tridiagonal solves                                                        */
/* ------------------------------------------------------------------------ */

/* thomas_solve, helmholtz.cpp:57-86 (n>=2 branch; returns 1 on a pivot below
 * 1e-300, where the reference throws NumericalError) */
static int thomas(const double *a, const double *b, const double *c, const double *d, int n,
                  double *x, double *cp, double *dp) {
  if (n == 1) { x[0] = d[0] / b[0]; return 0; }
  double denom = b[0];
  if (!(fabs(denom) > 0.0)) return 1;
  cp[0] = c[0] / denom;
  dp[0] = d[0] / denom;
  for (int k = 1; k < n; ++k) {
    denom = b[k] - a[k - 1] * cp[k - 1];
    if (fabs(denom) < 1e-300) return 1;
    dp[k] = (d[k] - a[k - 1] * dp[k - 1]) / denom;
    if (k < n - 1) cp[k] = c[k] / denom;
  }
  x[n - 1] = dp[n - 1];
  for (int k = n - 1; k-- > 0;) x[k] = dp[k] - cp[k] * x[k + 1];
  return 0;
}

/* AcousticSubstepper: update_coefficients :38-65, update_mass_and_pressure
 * :67-94, update_momentum :96-124, solve_vertical_implicit :126-137, step
 * :139-149 (src/time/acoustic_substep.cpp) */
static void ref_hevi_substep(vo_model *m, double dtau) {
  const int nx = m->nx, ny = m->ny, nz = m->nz;
  fld *st = m->st;
  const fld *r0f = &m->ref[VO_RHO0], *th0f = &m->ref[VO_THETA0], *pi0f = &m->ref[VO_PI0];
  /* update_mass_and_pressure */
  fld drho;
  fld_alloc(&drho, nx, ny, nz, 0);
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const double dx = m->s.dx, dy = m->s.dy;
        const double scale = m->s.z_top - g_terrain(m, i, j);
        const double dz = dmax(g_dzeta(m, k) * scale, 1.0);
        const double r0 = AT(*r0f, i, j, k);
        const double fx = AT(st[VO_U], i + 1, j, k) * 0.5 * (r0 + AT(*r0f, imin(i + 1, nx - 1), j, k)) -
                          AT(st[VO_U], i, j, k) * 0.5 * (AT(*r0f, imax(i - 1, 0), j, k) + r0);
        const double fy = AT(st[VO_V], i, j + 1, k) * 0.5 * (r0 + AT(*r0f, i, imin(j + 1, ny - 1), k)) -
                          AT(st[VO_V], i, j, k) * 0.5 * (AT(*r0f, i, imax(j - 1, 0), k) + r0);
        const double fz = AT(st[VO_W], i, j, k + 1) * 0.5 * (r0 + AT(*r0f, i, j, imin(k + 1, nz - 1))) -
                          AT(st[VO_W], i, j, k) * 0.5 * (AT(*r0f, i, j, imax(k - 1, 0)) + r0);
        AT(drho, i, j, k) = -(fx / dx + fy / dy + fz / dz);
      }
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const double r0 = dmax(AT(*r0f, i, j, k), 1e-8);
        AT(st[VO_RHO], i, j, k) += dtau * AT(drho, i, j, k);
        AT(st[VO_PI], i, j, k) += dtau * (K_RD / K_CV) * (AT(*pi0f, i, j, k) / r0) * AT(drho, i, j, k);
      }
  free(drho.d);
  /* update_coefficients from column (0,0) */
  double *ta = (double *)calloc((size_t)(nz > 1 ? nz - 1 : 1), sizeof(double));
  double *tb = (double *)calloc((size_t)nz, sizeof(double));
  double *tc = (double *)calloc((size_t)(nz > 1 ? nz - 1 : 1), sizeof(double));
  double *rhs = (double *)calloc((size_t)nz, sizeof(double));
  double *sol = (double *)calloc((size_t)nz, sizeof(double));
  double *cp = (double *)calloc((size_t)nz, sizeof(double));
  double *dp = (double *)calloc((size_t)nz, sizeof(double));
  const double half = 0.5 * dtau;
  for (int k = 0; k < nz; ++k) {
    const double scale = m->s.z_top - g_terrain(m, 0, 0);
    const double dz = dmax(g_dzeta(m, k) * scale, 1.0);
    const double rho0 = AT(*r0f, 0, 0, k);
    const double th0 = AT(*th0f, 0, 0, k);
    const double cs2 = (K_CP / K_CV) * K_RD * AT(*th0f, 0, 0, k) * AT(*pi0f, 0, 0, k); /* sound_speed2 :149-153 */
    const double a_k = half * half * K_CP * th0 * rho0 / (dz * dz);
    const double a_kp1 = (k < nz - 1) ? half * half * K_CP * AT(*th0f, 0, 0, k + 1) * AT(*r0f, 0, 0, k + 1) / (dz * dz) : a_k;
    const double b0 = 1.0 / dmax(rho0 * cs2, 1e-12);
    tb[k] = b0 + a_k + a_kp1;
    if (k < nz - 1) tc[k] = -a_kp1;
    if (k > 0) ta[k - 1] = -a_k;
  }
  /* solve_vertical_implicit */
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
      for (int k = 0; k < nz; ++k) rhs[k] = AT(st[VO_PI], i, j, k);
      thomas(ta, tb, tc, rhs, nz, sol, cp, dp);
      for (int k = 0; k < nz; ++k) AT(st[VO_PI], i, j, k) = sol[k];
    }
  free(ta); free(tb); free(tc); free(rhs); free(sol); free(cp); free(dp);
  /* update_momentum */
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i <= nx; ++i) {
        const int ip = imin(i, nx - 1), im = imax(i - 1, 0);
        const double dx = m->s.dx;
        const double t0 = 0.5 * (AT(*th0f, im, j, k) + AT(*th0f, ip, j, k));
        AT(st[VO_U], i, j, k) -= dtau * K_CP * t0 * (AT(st[VO_PI], ip, j, k) - AT(st[VO_PI], im, j, k)) / dx;
      }
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j <= ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const int jp = imin(j, ny - 1), jm = imax(j - 1, 0);
        const double dy = m->s.dy;
        const double t0 = 0.5 * (AT(*th0f, i, jm, k) + AT(*th0f, i, jp, k));
        AT(st[VO_V], i, j, k) -= dtau * K_CP * t0 * (AT(st[VO_PI], i, jp, k) - AT(st[VO_PI], i, jm, k)) / dy;
      }
  for (int k = 0; k <= nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const int kc = imin(imax(k, 0), nz - 1), km = imax(k - 1, 0);
        const double scale = m->s.z_top - g_terrain(m, i, j);
        const double dz = dmax(g_dzeta(m, kc) * scale, 1.0);
        const double t0 = 0.5 * (AT(*th0f, i, j, km) + AT(*th0f, i, j, kc));
        AT(st[VO_W], i, j, k) -= dtau * K_CP * t0 * (AT(st[VO_PI], i, j, kc) - AT(st[VO_PI], i, j, km)) / dz;
      }
}

/* Vertically implicit acoustic substep written consistently with the
 * explicit operator above (no reference counterpart; its own restatement).
 * With weight b = hevi_beta, rho0 face values r_f = 0.5*(rho0(k-1)+rho0(k))
 * (clamped as in mass_div0), face thetas t_f and face spacings
 * dzf_k = max(dzeta(min(k,nz-1))*scale, 1) as in acoustic_tendencies:
 *   Dh   = horizontal part of mass_div0 with the old u, v
 *   G_k  = (pi'_k - pi'_{k-1}) / dzf_k on interior faces, 0 on k = 0, nz
 *   w~   = w - dtau*(1-b)*cp*t_f*G(pi'_old)
 *   pi*  = pi + dtau*kappa*(Dh + (1-b)*Dv(w_old) + b*Dv(w~))
 *   (1 + c_k(T_k + T_{k+1})) x_k - c_k T_k x_{k-1} - c_k T_{k+1} x_{k+1} = pi*_k - P0_k
 *   with c_k = (dtau*b)^2*kappa_k/dz_k, T_f = r_f*cp*t_f/dzf_f (T_0 = T_nz = 0),
 *   x = pi'_new, P0 = pi0 (perturbation form) or 0 (total form);
 *   w_new = w~ - dtau*b*cp*t_f*G(x);  rho_new = rho + dtau*(Dh + (1-b)Dv(w_old) + b Dv(w_new));
 *   u, v backward with the new pi as in the explicit substep. */
static void cons_hevi_substep(vo_model *m, double dtau) {
  const int nx = m->nx, ny = m->ny, nz = m->nz;
  fld *st = m->st;
  const fld *r0f = &m->ref[VO_RHO0], *th0f = &m->ref[VO_THETA0], *pi0f = &m->ref[VO_PI0];
  const double b = m->s.hevi_beta, ob = 1.0 - b;
  const int pert = m->s.pgf_perturbation;
  double *T = (double *)calloc((size_t)nz + 1, sizeof(double));
  double *rf = (double *)calloc((size_t)nz + 1, sizeof(double));
  double *tf = (double *)calloc((size_t)nz + 1, sizeof(double));
  double *dzf = (double *)calloc((size_t)nz + 1, sizeof(double));
  double *G = (double *)calloc((size_t)nz + 1, sizeof(double));
  double *wt = (double *)calloc((size_t)nz + 1, sizeof(double));
  double *wn = (double *)calloc((size_t)nz + 1, sizeof(double));
  double *Dh = (double *)calloc((size_t)nz, sizeof(double));
  double *dzc = (double *)calloc((size_t)nz, sizeof(double));
  double *kap = (double *)calloc((size_t)nz, sizeof(double));
  double *ta = (double *)calloc((size_t)nz, sizeof(double));
  double *tb = (double *)calloc((size_t)nz, sizeof(double));
  double *tc = (double *)calloc((size_t)nz, sizeof(double));
  double *rhs = (double *)calloc((size_t)nz, sizeof(double));
  double *x = (double *)calloc((size_t)nz, sizeof(double));
  double *cp = (double *)calloc((size_t)nz, sizeof(double));
  double *dp = (double *)calloc((size_t)nz, sizeof(double));
  fld pin; /* new pi for the horizontal momentum update */
  fld_alloc(&pin, nx, ny, nz, 0);
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
      const double scale = m->s.z_top - g_terrain(m, i, j);
      for (int k = 0; k < nz; ++k) {
        dzc[k] = dmax(g_dzeta(m, k) * scale, 1.0);
        kap[k] = (K_RD / K_CV) * (AT(*pi0f, i, j, k) / dmax(AT(*r0f, i, j, k), 1e-8));
        const double r0 = AT(*r0f, i, j, k);
        const double fx = AT(st[VO_U], i + 1, j, k) * 0.5 * (r0 + AT(*r0f, imin(i + 1, nx - 1), j, k)) -
                          AT(st[VO_U], i, j, k) * 0.5 * (AT(*r0f, imax(i - 1, 0), j, k) + r0);
        const double fy = AT(st[VO_V], i, j + 1, k) * 0.5 * (r0 + AT(*r0f, i, imin(j + 1, ny - 1), k)) -
                          AT(st[VO_V], i, j, k) * 0.5 * (AT(*r0f, i, imax(j - 1, 0), k) + r0);
        Dh[k] = -(fx / m->s.dx + fy / m->s.dy);
      }
      for (int k = 0; k <= nz; ++k) {
        const int kc = imin(k, nz - 1), km = imax(k - 1, 0);
        rf[k] = 0.5 * (AT(*r0f, i, j, km) + AT(*r0f, i, j, kc));
        tf[k] = 0.5 * (AT(*th0f, i, j, km) + AT(*th0f, i, j, kc));
        dzf[k] = dmax(g_dzeta(m, kc) * scale, 1.0);
        if (k == 0 || k == nz) {
          G[k] = 0.0; T[k] = 0.0;
        } else {
          const double pa = AT(st[VO_PI], i, j, kc) - (pert ? AT(*pi0f, i, j, kc) : 0.0);
          const double pb = AT(st[VO_PI], i, j, km) - (pert ? AT(*pi0f, i, j, km) : 0.0);
          G[k] = (pa - pb) / dzf[k];
          T[k] = rf[k] * K_CP * tf[k] / dzf[k];
        }
        wt[k] = AT(st[VO_W], i, j, k) - dtau * ob * K_CP * tf[k] * G[k];
      }
      for (int k = 0; k < nz; ++k) {
        const double dv_old = -(rf[k + 1] * AT(st[VO_W], i, j, k + 1) - rf[k] * AT(st[VO_W], i, j, k)) / dzc[k];
        const double dv_t = -(rf[k + 1] * wt[k + 1] - rf[k] * wt[k]) / dzc[k];
        const double pstar = AT(st[VO_PI], i, j, k) + dtau * kap[k] * (Dh[k] + ob * dv_old + b * dv_t);
        const double ck = (dtau * b) * (dtau * b) * kap[k] / dzc[k];
        ta[k] = -ck * T[k];
        tc[k] = -ck * T[k + 1];
        tb[k] = 1.0 + ck * (T[k] + T[k + 1]);
        rhs[k] = pstar - (pert ? AT(*pi0f, i, j, k) : 0.0);
      }
      thomas(ta + 1, tb, tc, rhs, nz, x, cp, dp);
      for (int k = 0; k <= nz; ++k) {
        double g = 0.0;
        if (k > 0 && k < nz) g = (x[k] - x[k - 1]) / dzf[k];
        wn[k] = wt[k] - dtau * b * K_CP * tf[k] * g;
      }
      for (int k = 0; k < nz; ++k) {
        const double dv_old = -(rf[k + 1] * AT(st[VO_W], i, j, k + 1) - rf[k] * AT(st[VO_W], i, j, k)) / dzc[k];
        const double dv_new = -(rf[k + 1] * wn[k + 1] - rf[k] * wn[k]) / dzc[k];
        AT(st[VO_RHO], i, j, k) += dtau * (Dh[k] + ob * dv_old + b * dv_new);
        AT(pin, i, j, k) = x[k] + (pert ? AT(*pi0f, i, j, k) : 0.0);
      }
      for (int k = 0; k <= nz; ++k) AT(st[VO_W], i, j, k) = wn[k];
    }
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) AT(st[VO_PI], i, j, k) = AT(pin, i, j, k);
  free(pin.d);
  for (int k = 0; k < nz; ++k) /* backward horizontal momentum, as equations.cpp:157-174 */
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i <= nx; ++i) {
        const int ip = imin(i, nx - 1), im = imax(i - 1, 0);
        const double t0 = 0.5 * (AT(*th0f, im, j, k) + AT(*th0f, ip, j, k));
        AT(st[VO_U], i, j, k) += dtau * (-K_CP * t0 * dpi(m, &st[VO_PI], ip, j, k, im, j, k) / m->s.dx);
      }
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j <= ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const int jp = imin(j, ny - 1), jm = imax(j - 1, 0);
        const double t0 = 0.5 * (AT(*th0f, i, jm, k) + AT(*th0f, i, jp, k));
        AT(st[VO_V], i, j, k) += dtau * (-K_CP * t0 * dpi(m, &st[VO_PI], i, jp, k, i, jm, k) / m->s.dy);
      }
  free(T); free(rf); free(tf); free(dzf); free(G); free(wt); free(wn); free(Dh); free(dzc);
  free(kap); free(ta); free(tb); free(tc); free(rhs); free(x); free(cp); free(dp);
}

/* Damping::apply_sponge, damping.cpp:76-140 */
static void sponge_apply(vo_model *m, double dt) {
  const int nx = m->nx, ny = m->ny, nz = m->nz;
  int kmin = nz;
  for (int k = 0; k < nz; ++k)
    if (m->sponge[k] > 0.0) { kmin = k; break; }
  if (kmin >= nz) return;
#define ALPHA_AT(k) (m->sponge[imin((k), nz - 1)])
  for (int k = kmin; k < nz; ++k) { /* u */
    const double a = ALPHA_AT(k);
    if (a <= 0.0) continue;
    const double w = 1.0 / (1.0 + dt * a);
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i <= nx; ++i) AT(m->st[VO_U], i, j, k) = w * AT(m->st[VO_U], i, j, k);
  }
  for (int k = kmin; k < nz; ++k) { /* v */
    const double a = ALPHA_AT(k);
    if (a <= 0.0) continue;
    const double w = 1.0 / (1.0 + dt * a);
    for (int j = 0; j <= ny; ++j)
      for (int i = 0; i < nx; ++i) AT(m->st[VO_V], i, j, k) = w * AT(m->st[VO_V], i, j, k);
  }
  for (int k = kmin; k <= nz; ++k) { /* w */
    const double a = ALPHA_AT(k);
    if (a <= 0.0) continue;
    const double w = 1.0 / (1.0 + dt * a);
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) AT(m->st[VO_W], i, j, k) = w * AT(m->st[VO_W], i, j, k);
  }
  const int cells[3] = {VO_RHO, VO_THETA, VO_PI};
  const int tgts[3] = {VO_RHO0, VO_THETA0, VO_PI0};
  for (int c = 0; c < 3; ++c)
    for (int k = kmin; k < nz; ++k) {
      const double a = ALPHA_AT(k);
      if (a <= 0.0) continue;
      const double w = 1.0 / (1.0 + dt * a);
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
          const double tgt = AT(m->ref[tgts[c]], i, j, k);
          AT(m->st[cells[c]], i, j, k) = w * (AT(m->st[cells[c]], i, j, k) + dt * a * tgt);
        }
    }
#undef ALPHA_AT
}

static int has_nonfinite(const vo_model *m) { /* State::has_nonfinite, state.cpp:96-101 */
  for (int sp = 0; sp < VO_NSPECIES; ++sp) {
    const size_t n = fld_size(&m->st[sp]);
    for (size_t q = 0; q < n; ++q)
      if (!isfinite(m->st[sp].d[q])) return 1;
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* public entry points                                                      */
/* ------------------------------------------------------------------------ */
void vo_setup_defaults(vo_setup *s) {
  memset(s, 0, sizeof(*s));
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

vo_model *vo_create(const vo_setup *su) {
  vo_model *m = (vo_model *)calloc(1, sizeof(vo_model));
  m->s = *su;
  m->nx = su->nx; m->ny = su->ny; m->nz = su->nz;
  const int nx = m->nx, ny = m->ny, nz = m->nz;
  m->zeta = (double *)calloc((size_t)nz + 1, sizeof(double));
  make_stretched_zeta(nz, su->zeta_first, su->zeta_stretch, m->zeta);
  m->zs = (double *)calloc((size_t)nx * ny, sizeof(double));
  if (su->terrain_kind == 1) /* Gaussian hill at cell centres (build-defined case) */
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const double x = ((double)i + 0.5) * su->dx - su->hill_xc;
        const double y = ((double)j + 0.5) * su->dy - su->hill_yc;
        m->zs[(size_t)j * nx + i] = su->hill_h * exp(-(x * x + y * y) / (su->hill_a * su->hill_a));
      }
  for (int sp = 0; sp < VO_NSPECIES; ++sp) {
    fld_alloc(&m->st[sp], nx, ny, nz, stagger_of(sp));
    fld_alloc(&m->s0[sp], nx, ny, nz, stagger_of(sp));
    fld_alloc(&m->slow[sp], nx, ny, nz, stagger_of(sp));
    fld_alloc(&m->scr[sp], nx, ny, nz, stagger_of(sp));
  }
  for (int r = 0; r < 5; ++r) fld_alloc(&m->ref[r], nx, ny, nz, 0);
  if (su->ref_kind == 1) ref_from_profile(m); else ref_isothermal(m);
  /* Damping constructor sponge profile, damping.cpp:24-41 */
  m->sponge = (double *)calloc((size_t)nz, sizeof(double));
  {
    const double zs0 = su->sponge_start_fraction * su->z_top;
    for (int k = 0; k < nz; ++k) {
      const double z = g_zc(m, 0, 0, k);
      if (z <= zs0) { m->sponge[k] = 0.0; continue; }
      const double t = (z - zs0) / dmax(su->z_top - zs0, 1.0);
      const double sn = sin(0.5 * K_PI * (t < 0.0 ? 0.0 : (t > 1.0 ? 1.0 : t)));
      m->sponge[k] = su->sponge_alpha * sn * sn;
    }
  }
  /* Coriolis constructor, coriolis.cpp:25-32 */
  m->f0 = 2.0 * K_OMEGA * sin(su->latitude * K_DEG2RAD);
  m->beta = 2.0 * K_OMEGA * cos(su->latitude * K_DEG2RAD) / K_EARTH_RADIUS;
  init_warm_bubble(m);
  return m;
}

void vo_destroy(vo_model *m) {
  if (!m) return;
  for (int sp = 0; sp < VO_NSPECIES; ++sp) {
    free(m->st[sp].d); free(m->s0[sp].d); free(m->slow[sp].d); free(m->scr[sp].d);
  }
  for (int r = 0; r < 5; ++r) free(m->ref[r].d);
  free(m->zeta); free(m->zs); free(m->sponge);
  free(m);
}

size_t vo_storage_size(const vo_model *m, int species) { return fld_size(&m->st[species]); }
void vo_get_field(const vo_model *m, int sp, double *out) {
  memcpy(out, m->st[sp].d, fld_size(&m->st[sp]) * sizeof(double));
}
void vo_set_field(vo_model *m, int sp, const double *in) {
  memcpy(m->st[sp].d, in, fld_size(&m->st[sp]) * sizeof(double));
}
void vo_get_reffield(const vo_model *m, int which, double *out) {
  memcpy(out, m->ref[which].d, fld_size(&m->ref[which]) * sizeof(double));
}
void vo_get_zeta(const vo_model *m, double *out) { memcpy(out, m->zeta, sizeof(double) * (size_t)(m->nz + 1)); }
void vo_get_terrain(const vo_model *m, double *out) { memcpy(out, m->zs, sizeof(double) * (size_t)m->nx * m->ny); }
void vo_get_sponge(const vo_model *m, double *out) { memcpy(out, m->sponge, sizeof(double) * (size_t)m->nz); }

void vo_acoustic_substep(vo_model *m, double dtau) { fb_substep(m, dtau); }
void vo_hevi_substep(vo_model *m, double dtau) {
  if (m->s.acoustic_mode == 1) ref_hevi_substep(m, dtau); else cons_hevi_substep(m, dtau);
}
void vo_sponge(vo_model *m, double dt) { sponge_apply(m, dt); }

void vo_slow_tendency(vo_model *m, double *const *out) {
  slow_tendency_split(m, m->st, m->slow);
  for (int sp = 0; sp < VO_NSPECIES; ++sp)
    memcpy(out[sp], m->slow[sp].d, fld_size(&m->slow[sp]) * sizeof(double));
}

/* ------------------------------------------------------------------------ */
/* Kessler warm rain: src/physics/microphysics_kessler.cpp, helpers from      */
/* src/physics/physics_types.cpp and include/vibe/physics/physics_types.hpp  */
/* ------------------------------------------------------------------------ */
static fld fld_view(const vo_model *m, const double *p);
#define KP_RV 461.51
#define KP_KAPPA 0.28571
#define KP_T0 273.15
#define KP_RHO_WATER 1000.0
#define KP_DV_WATER 2.21e-5
#define KP_THERM_COND_AIR 2.40e-2
#define KP_DYN_VISC_AIR 1.8e-5 /* microphysics_kessler.cpp:23 */
#define KP_SCHMIDT 0.6         /* :24 */
#define KP_RAIN_N0 8.0e6       /* microphysics.hpp:192 */
#define KP_RAIN_B 3.0          /* microphysics.hpp:195 */

static double kp_max(double a, double b) { return a > b ? a : b; } /* std::max: a < b ? b : a */
static double kp_min(double a, double b) { return b < a ? b : a; } /* std::min */
static double kp_clamp(double v, double lo, double hi) { return v < lo ? lo : (hi < v ? hi : v); }

void vo_kessler_defaults(vo_kessler *k) { /* PhysicsOptions, physics_types.hpp:420-429 */
  k->qc0 = 1.0e-3;
  k->k1 = 1.0e-3;
  k->k2 = 2.2;
  k->evap_coef = 1.0;
  k->rain_a = 36.34;
  k->rain_b = 0.1364;
  k->positive_definite = 1;
  k->exner_offset = 1;
}

static double kp_exner(double p) { return pow(p / K_P0, KP_KAPPA); }            /* physics_types.hpp:136-138 */
static double kp_lv(double t) { return (2.501 - 0.00237 * (t - KP_T0)) * 1.0e6; } /* :159-161 */
static double kp_es(double t) {                                                 /* physics_types.cpp:143-146 */
  const double tc = kp_max(t - KP_T0, -80.0);
  return 611.2 * exp(17.67 * tc / (tc + 243.5));
}
static double kp_qs(double p, double t) { /* saturation_mixing_ratio, physics_types.cpp:163-167 (liquid) */
  const double es = kp_es(t);
  const double den = kp_max(p - es, 1.0);
  return K_EPS_VAP * es / den;
}
static double kp_fall_speed(const vo_kessler *o, double rho, double qr) { /* microphysics_kessler.cpp:188-191 */
  const double load = kp_max(rho * kp_max(qr, 0.0), 0.0);
  return o->rain_a * pow(load, o->rain_b);
}

/* saturation_adjust_point (liquid), microphysics_kessler.cpp:100-144 */
static void kp_adjust(double *qv_io, double *qc_io, double *theta_io, double p) {
  double qv = kp_max(*qv_io, 0.0), qc = kp_max(*qc_io, 0.0), theta = *theta_io;
  const double pi = kp_exner(p);
  double t = kp_max(theta * pi, 150.0);
  double qs = kp_qs(p, t);
  double l = kp_lv(t);
  const double denom0 = 1.0 + l * l * qs / (K_CP * KP_RV * t * t);
  double delta = kp_clamp((qv - qs) / denom0, -qc, qv);
  if (fabs(delta) < 1.0e-16) {
    *qv_io = qv;
    *qc_io = qc;
    return;
  }
  for (int it = 1; it <= 10; ++it) {
    t = theta * pi + (l / K_CP) * delta;
    t = kp_max(t, 150.0);
    qs = kp_qs(p, t);
    l = kp_lv(t);
    const double f = qv - delta - qs;
    const double dqsdT = l * qs / (KP_RV * t * t);
    const double df = -1.0 - (l / K_CP) * dqsdT;
    const double residual = fabs(f) / kp_max(qs, 1.0e-12);
    if (residual <= 1.0e-10) break;
    const double step = -f / df;
    const double trial = kp_clamp(delta + kp_clamp(step, -1.0, 1.0), -qc, qv);
    if (trial == delta) break;
    delta = trial;
  }
  qv -= delta;
  qc += delta;
  theta += l * delta / (K_CP * pi);
  *qv_io = kp_max(qv, 0.0);
  *qc_io = kp_max(qc, 0.0);
  *theta_io = theta;
}

/* rain_evaporation_rate, microphysics_kessler.cpp:213-227, with
 * slope_parameter, number_concentration, ventilation_factor and
 * particle_mass_rate (:38-76) */
static double kp_evap_rate(const vo_kessler *o, double p, double t, double rho, double qv, double qs, double qr) {
  (void)p;
  if (!(qr > 0.0) || !(rho > 0.0)) return 0.0;
  const double a = K_PI / 6.0 * KP_RHO_WATER;
  const double qq = kp_max(qr, 1.0e-14);
  const double num = a * KP_RAIN_N0 * tgamma(1.0 + KP_RAIN_B);
  const double den = kp_max(rho * qq, 1.0e-20);
  const double lambda = pow(num / den, 1.0 / KP_RAIN_B);
  const double nr = KP_RAIN_N0 / kp_max(lambda, 1.0e-8);
  const double r_mean = 0.5 / kp_max(lambda, 1.0e-8);
  const double vt = kp_fall_speed(o, rho, qr);
  double fv = 1.0;
  if (r_mean > 0.0) {
    const double re = 2.0 * r_mean * kp_max(vt, 0.0) * rho / KP_DYN_VISC_AIR;
    fv = kp_max(0.78 + 0.308 * cbrt(KP_SCHMIDT) * sqrt(kp_max(re, 0.0)), 1.0);
  }
  double dm = 0.0;
  if (r_mean > 0.0 && rho > 0.0 && t > 0.0) {
    const double rho_v = qv * rho, rho_vs = qs * rho;
    const double l = kp_lv(t);
    const double dnm = 1.0 + l * l * KP_DV_WATER * rho_vs / (KP_THERM_COND_AIR * KP_RV * t * t);
    dm = 4.0 * K_PI * r_mean * fv * (rho_v - rho_vs) / dnm;
  }
  const double rate = (-dm) * nr / rho;
  return kp_max(o->evap_coef * rate, 0.0);
}

/* KesslerMicrophysics::step_column, microphysics_kessler.cpp:269-331, with
 * PhysicsColumn::diagnose_layer_depth (physics_types.cpp:257-284) for dz */
double vo_kessler_column(const vo_kessler *o, int n, double dt, const double *z, const double *p,
                         const double *rho, double *theta, double *qv, double *qc, double *qr) {
  if (!(dt > 0.0) || n <= 0) return 0.0;
  double *dz = (double *)malloc(sizeof(double) * (size_t)n);
  double *zf = (double *)malloc(sizeof(double) * (size_t)(n + 1));
  if (n == 1) {
    zf[0] = z[0] - 0.5 * 100.0;
    zf[1] = z[0] + 0.5 * 100.0;
  } else {
    zf[0] = z[0] - 0.5 * (z[1] - z[0]);
    for (int k = 1; k < n; ++k) zf[k] = 0.5 * (z[k - 1] + z[k]);
    zf[n] = z[n - 1] + 0.5 * (z[n - 1] - z[n - 2]);
  }
  for (int k = 0; k < n; ++k) dz[k] = kp_max(zf[k + 1] - zf[k], 1.0e-6);
  /* 1. saturation adjustment */
  for (int k = 0; k < n; ++k) kp_adjust(&qv[k], &qc[k], &theta[k], p[k]);
  /* 2. autoconversion + accretion */
  for (int k = 0; k < n; ++k) {
    const double c = kp_max(qc[k], 0.0), r = kp_max(qr[k], 0.0);
    const double rate = o->k1 * kp_max(c - o->qc0, 0.0) + o->k2 * kp_max(c, 0.0) * kp_max(r, 0.0);
    const double dq = kp_min(rate * dt, c);
    qc[k] = c - dq;
    qr[k] = r + dq;
  }
  /* 3. sedimentation (sediment_rain, :240-262) */
  double flux_in = 0.0;
  for (int k = n - 1; k >= 0; --k) {
    const double rh = kp_max(rho[k], 1.0e-6), d = kp_max(dz[k], 1.0e-6), r = kp_max(qr[k], 0.0);
    const double mass = rh * r * d;
    const double vt = kp_fall_speed(o, rh, r);
    const double available = mass + flux_in * dt;
    const double out = kp_min(rh * r * vt * dt, kp_max(available, 0.0));
    qr[k] = kp_max(available - out, 0.0) / (rh * d);
    flux_in = out / dt;
  }
  const double precip = flux_in * dt;
  /* 4. rain evaporation */
  for (int k = 0; k < n; ++k) {
    const double r = kp_max(qr[k], 0.0);
    if (r <= 0.0) continue;
    const double pk = kp_exner(p[k]);
    const double t = theta[k] * pk;
    const double qs = kp_qs(p[k], t);
    const double v = kp_max(qv[k], 0.0);
    if (v >= qs) continue;
    double evap = kp_evap_rate(o, p[k], t, rho[k], v, qs, r) * dt;
    evap = kp_min(evap, r);
    const double lv = kp_lv(t);
    const double cap = (qs - v) / (1.0 + lv * lv * qs / (K_CP * KP_RV * t * t));
    evap = kp_min(evap, kp_max(cap, 0.0));
    if (!(evap > 0.0)) continue;
    qr[k] = r - evap;
    qv[k] = v + evap;
    theta[k] = theta[k] - lv * evap / (K_CP * pk);
  }
  /* 5. positive definite */
  if (o->positive_definite)
    for (int k = 0; k < n; ++k) {
      qv[k] = kp_max(qv[k], 0.0);
      qc[k] = kp_max(qc[k], 0.0);
      qr[k] = kp_max(qr[k], 0.0);
    }
  free(dz);
  free(zf);
  return precip / dt;
}

/* PhysicsDriver microphysics step for the current state: state_to_column
 * (physics_driver.cpp:95-128; qi, qs, qg enter only the virtual temperature
 * used where rho <= 0), step_column, td = (after - before) / dt (:271-288),
 * scattered into cell fields (:369-383). pt[0..3]: theta, qv, qc, qr. */
static void kessler_tendency(const vo_model *m, const vo_kessler *o, double dt, fld *pt) {
  const int nz = m->nz;
  double *z = (double *)malloc(sizeof(double) * (size_t)nz * 10);
  double *p = z + nz, *rho = p + nz, *th = rho + nz, *qv = th + nz, *qc = qv + nz, *qr = qc + nz;
  double *th0 = qr + nz, *qv0 = th0 + nz, *qc0 = qv0 + nz;
  double *qr0 = (double *)malloc(sizeof(double) * (size_t)nz);
  for (int j = 0; j < m->ny; ++j)
    for (int i = 0; i < m->nx; ++i) {
      for (int k = 0; k < nz; ++k) {
        z[k] = g_zc(m, i, j, k);
        const double pi0 = AT(m->ref[1], i, j, k);
        const double pis = AT(m->st[VO_PI], i, j, k);
        const double pi = o->exner_offset ? pi0 + pis : pis;
        p[k] = K_P0 * pow(kp_max(pi, 1.0e-3), 1.0 / KP_KAPPA);
        th[k] = AT(m->st[VO_THETA], i, j, k);
        qv[k] = kp_max(AT(m->st[VO_QV], i, j, k), 0.0);
        qc[k] = kp_max(AT(m->st[VO_QC], i, j, k), 0.0);
        qr[k] = kp_max(AT(m->st[VO_QR], i, j, k), 0.0);
        const double rs = AT(m->st[VO_RHO], i, j, k);
        if (rs > 0.0) {
          rho[k] = rs;
        } else {
          const double qi = kp_max(AT(m->st[VO_QI], i, j, k), 0.0), qsn = kp_max(AT(m->st[VO_QS], i, j, k), 0.0),
                       qg = kp_max(AT(m->st[VO_QG], i, j, k), 0.0);
          const double tv = th[k] * kp_exner(p[k]) * (1.0 + 0.608 * qv[k] - qc[k] - qi - qsn - qg);
          rho[k] = p[k] / (K_RD * tv);
        }
        th0[k] = th[k]; qv0[k] = qv[k]; qc0[k] = qc[k]; qr0[k] = qr[k];
      }
      vo_kessler_column(o, nz, dt, z, p, rho, th, qv, qc, qr);
      for (int k = 0; k < nz; ++k) {
        AT(pt[0], i, j, k) = 0.0 + (th[k] - th0[k]) / dt;
        AT(pt[1], i, j, k) = 0.0 + (qv[k] - qv0[k]) / dt;
        AT(pt[2], i, j, k) = 0.0 + (qc[k] - qc0[k]) / dt;
        AT(pt[3], i, j, k) = 0.0 + (qr[k] - qr0[k]) / dt;
      }
    }
  free(z);
  free(qr0);
}

void vo_kessler_tendency(const vo_model *m, const vo_kessler *k, double dt, double *const *out) {
  fld pt[4];
  for (int q = 0; q < 4; ++q) {
    pt[q] = fld_view(m, out[q]);
    memset(out[q], 0, fld_size(&pt[q]) * sizeof(double));
  }
  kessler_tendency(m, k, dt, pt);
}

void vo_set_physics_kessler(vo_model *m, const vo_kessler *k) {
  m->physics = k != NULL;
  if (k) m->kessler = *k;
}

/* RungeKutta3Integrator::slow_tendency with physics (runge_kutta.cpp:46-63):
 * d += pt for theta, qv, qc, qr (the other PhysicsTendency fields stay zero
 * under this scheme) */
static void physics_into(vo_model *m, double dt) {
  fld pt[4];
  for (int q = 0; q < 4; ++q) {
    fld_alloc(&pt[q], m->nx, m->ny, m->nz, 0);
    fld_zero(&pt[q]);
  }
  kessler_tendency(m, &m->kessler, dt, pt);
  const int sp[4] = {VO_THETA, VO_QV, VO_QC, VO_QR};
  for (int q = 0; q < 4; ++q) {
    add_scaled(&m->slow[sp[q]], 1.0, &pt[q]);
    free(pt[q].d);
  }
}

/* RungeKutta3Integrator::step, runge_kutta.cpp:77-119, with
 * State::add_scaled(Real, Tendency) expanded field by field */
int vo_rk3_step(vo_model *m, double dt, int n_sub_in) {
  const int n_sub = n_sub_in > 1 ? n_sub_in : 1;
  for (int sp = 0; sp < VO_NSPECIES; ++sp)
    memcpy(m->s0[sp].d, m->st[sp].d, fld_size(&m->st[sp]) * sizeof(double));
  const double dt_stage[3] = {dt / 3.0, dt / 2.0, dt};
  for (int stage = 0; stage < 3; ++stage) {
    slow_tendency_split(m, m->st, m->slow);
    if (m->physics) physics_into(m, dt);
    for (int sp = 0; sp < VO_NSPECIES; ++sp) {
      memcpy(m->st[sp].d, m->s0[sp].d, fld_size(&m->st[sp]) * sizeof(double));
      add_scaled(&m->st[sp], dt_stage[stage], &m->slow[sp]);
    }
    const double dtau = dt_stage[stage] / (double)n_sub;
    for (int n = 0; n < n_sub; ++n) {
      if (m->s.acoustic_mode == 0) fb_substep(m, dtau);
      else vo_hevi_substep(m, dtau);
    }
    if (has_nonfinite(m)) return 1;
  }
  sponge_apply(m, dt);
  if (m->s.w_rigid)
    for (int j = 0; j < m->ny; ++j)
      for (int i = 0; i < m->nx; ++i) {
        AT(m->st[VO_W], i, j, 0) = 0.0;
        AT(m->st[VO_W], i, j, m->nz) = 0.0;
      }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Helmholtz family: src/time/helmholtz.cpp:126-495                          */
/* ------------------------------------------------------------------------ */

/* a cell field over caller storage (FieldT layout, halo 4) */
static fld fld_view(const vo_model *m, const double *p) {
  fld f;
  f.nx = m->nx; f.ny = m->ny; f.nz = m->nz;
  f.nsx = m->nx + 2 * VO_HALO; f.nsy = m->ny + 2 * VO_HALO; f.nsz = m->nz + 2 * VO_HALO;
  f.d = (double *)p;
  return f;
}
static fld fld_cell(const vo_model *m) {
  fld f;
  fld_alloc(&f, m->nx, m->ny, m->nz, 0);
  return f;
}
static void fld_copy(fld *dst, const fld *src) { memcpy(dst->d, src->d, fld_size(src) * sizeof(double)); }

/* apply_operator, helmholtz.cpp:173-201: y = -div(a grad x) + b x with
 * arithmetic face means of a and clamped neighbours */
static void h_apply(const vo_model *m, const fld *a, const fld *b, const fld *x, fld *y) {
  const int nx = m->nx, ny = m->ny, nz = m->nz;
  const double dx = m->s.dx, dy = m->s.dy;
  fld_zero(y);
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const double scale = m->s.z_top - g_terrain(m, i, j);
        const double dz = dmax(g_dzeta(m, k) * scale, 1.0);
        const double ac = AT(*a, i, j, k);
        const double ae = 0.5 * (ac + CL(a, i + 1, j, k));
        const double aw = 0.5 * (ac + CL(a, i - 1, j, k));
        const double an = 0.5 * (ac + CL(a, i, j + 1, k));
        const double as = 0.5 * (ac + CL(a, i, j - 1, k));
        const double at = 0.5 * (ac + CL(a, i, j, k + 1));
        const double ab = 0.5 * (ac + CL(a, i, j, k - 1));
        const double xc = AT(*x, i, j, k);
        const double fx = (ae * (CL(x, i + 1, j, k) - xc) - aw * (xc - CL(x, i - 1, j, k))) / (dx * dx);
        const double fy = (an * (CL(x, i, j + 1, k) - xc) - as * (xc - CL(x, i, j - 1, k))) / (dy * dy);
        const double fz = (at * (CL(x, i, j, k + 1) - xc) - ab * (xc - CL(x, i, j, k - 1))) / (dz * dz);
        AT(*y, i, j, k) = -fx - fy - fz + AT(*b, i, j, k) * xc;
      }
}

/* dot_field, helmholtz.cpp:203-207: serial sum over the whole storage */
static double h_dot(const fld *a, const fld *b) {
  double s = 0.0;
  const size_t n = fld_size(a);
  for (size_t q = 0; q < n; ++q) s += a->d[q] * b->d[q];
  return s;
}

/* helmholtz_residual_l2, helmholtz.cpp:211-227 */
static double h_residual_l2(const vo_model *m, const fld *a, const fld *b, const fld *f, const fld *x) {
  fld lx = fld_cell(m);
  h_apply(m, a, b, x, &lx);
  double s = 0.0;
  for (int k = 0; k < m->nz; ++k)
    for (int j = 0; j < m->ny; ++j)
      for (int i = 0; i < m->nx; ++i) {
        const double r = AT(lx, i, j, k) - AT(*f, i, j, k);
        s += r * r;
      }
  free(lx.d);
  return sqrt(s);
}

/* VerticalTridiagonalSolver::solve, helmholtz.cpp:241-274, with the Thomas
 * solve of the documented C contract (the reference calls its own C Thomas,
 * which does not solve the system, c_kernels.c:18-60) */
static int h_solve_vertical(const vo_model *m, const fld *a, const fld *b, const fld *f, fld *x, int *iters,
                            double *res) {
  const int nx = m->nx, ny = m->ny, nz = m->nz;
  double *sa = (double *)calloc((size_t)nz + 1, sizeof(double)), *sb = (double *)calloc((size_t)nz, sizeof(double));
  double *sc = (double *)calloc((size_t)nz + 1, sizeof(double)), *sd = (double *)calloc((size_t)nz, sizeof(double));
  double *sx = (double *)calloc((size_t)nz, sizeof(double)), *ws = (double *)calloc((size_t)nz, sizeof(double));
  int rc = 0;
  fld_zero(x);
  for (int j = 0; j < ny && !rc; ++j)
    for (int i = 0; i < nx && !rc; ++i) {
      for (int k = 0; k < nz; ++k) {
        const double scale = m->s.z_top - g_terrain(m, i, j);
        const double dz = dmax(g_dzeta(m, k) * scale, 1.0);
        const double az = 0.5 * (AT(*a, i, j, k) + CL(a, i, j, k + 1));
        const double azm = 0.5 * (AT(*a, i, j, k) + CL(a, i, j, k - 1));
        sb[k] = (az + azm) / (dz * dz) + AT(*b, i, j, k);
        if (k > 0) sa[k - 1] = -azm / (dz * dz);
        if (k < nz - 1) sc[k] = -az / (dz * dz);
        sd[k] = AT(*f, i, j, k);
      }
      if (vo_tridiagonal_solve(sa, sb, sc, sd, nz, sx, ws) != 0) { rc = 1; break; }
      for (int k = 0; k < nz; ++k) AT(*x, i, j, k) = sx[k];
    }
  free(sa); free(sb); free(sc); free(sd); free(sx); free(ws);
  *iters = 1;
  *res = 0.0;
  return rc;
}

/* KrylovJacobiSolver::solve, helmholtz.cpp:296-366, operation for operation
 * (including its residual recomputed from x at the top of each iteration and
 * the update x += alpha p + omega s) */
static void h_solve_krylov_jacobi(const vo_model *m, int max_iter, double tol, const fld *a, const fld *b,
                                  const fld *f, fld *x, int *iters, double *res_out) {
  const int nx = m->nx, ny = m->ny, nz = m->nz;
  fld r = fld_cell(m), r0 = fld_cell(m), p = fld_cell(m), v = fld_cell(m), s = fld_cell(m), t = fld_cell(m);
  fld prec = fld_cell(m), rhat = fld_cell(m), shat = fld_cell(m);
  const size_t n = fld_size(&r);
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const double dx = m->s.dx, dy = m->s.dy;
        const double scale = m->s.z_top - g_terrain(m, i, j);
        const double dz = dmax(g_dzeta(m, k) * scale, 1.0);
        const double ac = AT(*a, i, j, k);
        const double diag = 2.0 * ac / (dx * dx) + 2.0 * ac / (dy * dy) + 2.0 * ac / (dz * dz) + AT(*b, i, j, k);
        AT(prec, i, j, k) = 1.0 / dmax(diag, 1e-30);
      }
  fld_zero(x);
  fld_copy(&r, f);
  fld_copy(&r0, &r);
  double rho = 1.0, alpha = 1.0, omega = 1.0, rho_prev = 1.0;
  const double f_norm = sqrt(dmax(h_dot(f, f), 1e-300));
  double res = 1.0;
  int it = 0;
  for (; it < max_iter; ++it) {
    h_apply(m, a, b, x, &v);
    for (size_t q = 0; q < n; ++q) r.d[q] = f->d[q] - v.d[q];
    res = sqrt(h_dot(&r, &r)) / f_norm;
    if (res < tol) break;
    for (size_t q = 0; q < n; ++q) rhat.d[q] = prec.d[q] * r.d[q];
    rho = h_dot(&rhat, &r0);
    if (fabs(rho) < 1e-300) break;
    const double beta = (rho / rho_prev) * (alpha / omega);
    for (size_t q = 0; q < n; ++q) p.d[q] = rhat.d[q] + beta * (p.d[q] - omega * v.d[q]);
    h_apply(m, a, b, &p, &v);
    const double denom = h_dot(&r0, &v);
    alpha = (fabs(denom) > 1e-300) ? rho / denom : 0.0;
    for (size_t q = 0; q < n; ++q) s.d[q] = r.d[q] - alpha * v.d[q];
    if (sqrt(h_dot(&s, &s)) / f_norm < tol) {
      for (size_t q = 0; q < n; ++q) x->d[q] += alpha * p.d[q];
      break;
    }
    for (size_t q = 0; q < n; ++q) shat.d[q] = prec.d[q] * s.d[q];
    h_apply(m, a, b, &shat, &t);
    const double tt = h_dot(&t, &t);
    omega = (tt > 1e-300) ? h_dot(&t, &s) / tt : 0.0;
    for (size_t q = 0; q < n; ++q) x->d[q] += alpha * p.d[q] + omega * s.d[q];
    for (size_t q = 0; q < n; ++q) r.d[q] = s.d[q] - omega * t.d[q];
    rho_prev = rho;
    if (fabs(omega) < 1e-300) break;
  }
  *iters = it;
  *res_out = res;
  free(r.d); free(r0.d); free(p.d); free(v.d); free(s.d); free(t.d); free(prec.d); free(rhat.d); free(shat.d);
}

/* multigrid_restrict, helmholtz.cpp:130-145 (coarse has the fine field's
 * shape; fine indices clamp at the edge) */
static void h_restrict(const vo_model *m, const fld *fine, fld *coarse) {
  for (int k = 0; k < m->nz; ++k)
    for (int j = 0; j < m->ny; ++j)
      for (int i = 0; i < m->nx; ++i) {
        const int fi = 2 * i, fj = 2 * j;
        double acc = 0.25 * CL(fine, fi, fj, k);
        acc += 0.125 * (CL(fine, fi - 1, fj, k) + CL(fine, fi + 1, fj, k) + CL(fine, fi, fj - 1, k) +
                        CL(fine, fi, fj + 1, k));
        acc += 0.0625 * (CL(fine, fi - 1, fj - 1, k) + CL(fine, fi + 1, fj - 1, k) + CL(fine, fi - 1, fj + 1, k) +
                         CL(fine, fi + 1, fj + 1, k));
        AT(*coarse, i, j, k) = acc;
      }
}

/* multigrid_prolong, helmholtz.cpp:147-164 */
static void h_prolong(const vo_model *m, const fld *coarse, fld *fine) {
  for (int k = 0; k < m->nz; ++k)
    for (int j = 0; j < m->ny; ++j)
      for (int i = 0; i < m->nx; ++i) {
        const double xs = 0.5 * (double)i, ys = 0.5 * (double)j;
        const int i0 = (int)floor(xs), j0 = (int)floor(ys);
        const double wx = xs - (double)i0, wy = ys - (double)j0;
        AT(*fine, i, j, k) = lerp(lerp(CL(coarse, i0, j0, k), CL(coarse, i0 + 1, j0, k), wx),
                                  lerp(CL(coarse, i0, j0 + 1, k), CL(coarse, i0 + 1, j0 + 1, k), wx), wy);
      }
}

/* KrylovMultigridSolver::solve, helmholtz.cpp:393-405. Its coarse solve
 * (restrict f, solve, prolong into x) is discarded: the inner solver starts
 * by zeroing x (:316). The result is the inner solve of f, restated so. */
static void h_solve_krylov_mg(const vo_model *m, int max_iter, double tol, const fld *a, const fld *b,
                              const fld *f, fld *x, int *iters, double *res) {
  h_solve_krylov_jacobi(m, max_iter, tol, a, b, f, x, iters, res);
}

/* RefinementSolver::solve, helmholtz.cpp:433-462 (max_refine 3) */
static void h_solve_refined(const vo_model *m, int max_iter, double tol, int refine, const fld *a, const fld *b,
                            const fld *f, fld *x, int *iters, double *res) {
  int it_in = 0;
  double res_in = 1.0;
  h_solve_krylov_mg(m, max_iter, tol, a, b, f, x, &it_in, &res_in);
  if (!refine) { *iters = it_in; *res = res_in; return; }
  fld r = fld_cell(m), lx = fld_cell(m), dxf = fld_cell(m);
  const size_t n = fld_size(&r);
  int total = it_in;
  double residual = res_in;
  for (int it = 0; it < 3; ++it) {
    h_apply(m, a, b, x, &lx);
    double rn = 0.0, fn = 0.0;
    for (size_t q = 0; q < n; ++q) {
      r.d[q] = f->d[q] - lx.d[q];
      rn += r.d[q] * r.d[q];
      fn += f->d[q] * f->d[q];
    }
    const double rel = sqrt(rn / dmax(fn, 1e-300));
    residual = rel;
    if (rel < tol) break;
    fld_zero(&dxf);
    h_solve_krylov_mg(m, max_iter, tol, a, b, &r, &dxf, &it_in, &res_in);
    for (size_t q = 0; q < n; ++q) x->d[q] += dxf.d[q];
    total += it_in;
  }
  *iters = total;
  *res = residual;
  free(r.d); free(lx.d); free(dxf.d);
}

static int h_solve(const vo_model *m, int kind, int max_iter, double tol, int refine, const fld *a, const fld *b,
                   const fld *f, fld *x, int *iters, double *res) {
  if (kind == VO_HZ_VERTICAL) return h_solve_vertical(m, a, b, f, x, iters, res);
  if (kind == VO_HZ_KRYLOV_JACOBI) {
    h_solve_krylov_jacobi(m, max_iter, tol, a, b, f, x, iters, res);
    return 0;
  }
  h_solve_refined(m, max_iter, tol, refine, a, b, f, x, iters, res);
  return 0;
}

void vo_helmholtz_apply(const vo_model *m, const double *a, const double *b, const double *x, double *y) {
  const fld fa = fld_view(m, a), fb = fld_view(m, b), fx = fld_view(m, x);
  fld fy = fld_view(m, y);
  h_apply(m, &fa, &fb, &fx, &fy);
}

double vo_helmholtz_residual_l2(const vo_model *m, const double *a, const double *b, const double *f,
                                const double *x) {
  const fld fa = fld_view(m, a), fb = fld_view(m, b), ff = fld_view(m, f), fx = fld_view(m, x);
  return h_residual_l2(m, &fa, &fb, &ff, &fx);
}

int vo_helmholtz_solve(const vo_model *m, int kind, int max_iter, double tol, int refine, const double *a,
                       const double *b, const double *f, double *x, int *iterations, double *residual) {
  const fld fa = fld_view(m, a), fb = fld_view(m, b), ff = fld_view(m, f);
  fld fx = fld_view(m, x);
  return h_solve(m, kind, max_iter, tol, refine, &fa, &fb, &ff, &fx, iterations, residual);
}

void vo_multigrid_restrict(const vo_model *m, const double *fine, double *coarse) {
  const fld ff = fld_view(m, fine);
  fld fc = fld_view(m, coarse);
  h_restrict(m, &ff, &fc);
}
void vo_multigrid_prolong(const vo_model *m, const double *coarse, double *fine) {
  const fld fc = fld_view(m, coarse);
  fld ff = fld_view(m, fine);
  h_prolong(m, &fc, &ff);
}

/* SemiImplicitIntegrator::assemble_rhs, semi_implicit.cpp:56-106: a =
 * (dt/2)^2 (Rd/cv) pi0 cp theta0, b = 1, rhs = pi - dt c G + (horizontal)
 * div(a0 grad pi), G = div(rho0 u^n) + dt/2 div(rho0 N_u) */
static void si_assemble(const vo_model *m, const fld *st, const fld *n, double dt, fld *acoef, fld *bcoef,
                        fld *rhs) {
  const int nx = m->nx, ny = m->ny, nz = m->nz;
  const double half_dt = 0.5 * dt;
  const fld *pi0 = &m->ref[VO_PI0], *th0 = &m->ref[VO_THETA0], *r0 = &m->ref[VO_RHO0];
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        AT(*acoef, i, j, k) = half_dt * half_dt * (K_RD / K_CV) * AT(*pi0, i, j, k) * K_CP * AT(*th0, i, j, k);
        AT(*bcoef, i, j, k) = 1.0;
      }
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const double dx = m->s.dx, dy = m->s.dy;
        const double scale = m->s.z_top - g_terrain(m, i, j);
        const double dz = dmax(g_dzeta(m, k) * scale, 1.0);
        const fld *U[2] = {&st[VO_U], &n[VO_U]}, *V[2] = {&st[VO_V], &n[VO_V]}, *W[2] = {&st[VO_W], &n[VO_W]};
        double dv[2];
        for (int c = 0; c < 2; ++c) { /* flux_div lambda, :82-91 (unclamped i+1, j+1, k+1 face reads) */
          const double fx = AT(*U[c], i + 1, j, k) * 0.5 * (AT(*r0, i, j, k) + AT(*r0, imin(i + 1, nx - 1), j, k)) -
                            AT(*U[c], i, j, k) * 0.5 * (AT(*r0, imax(i - 1, 0), j, k) + AT(*r0, i, j, k));
          const double fy = AT(*V[c], i, j + 1, k) * 0.5 * (AT(*r0, i, j, k) + AT(*r0, i, imin(j + 1, ny - 1), k)) -
                            AT(*V[c], i, j, k) * 0.5 * (AT(*r0, i, imax(j - 1, 0), k) + AT(*r0, i, j, k));
          const double fz = AT(*W[c], i, j, k + 1) * 0.5 * (AT(*r0, i, j, k) + AT(*r0, i, j, imin(k + 1, nz - 1))) -
                            AT(*W[c], i, j, k) * 0.5 * (AT(*r0, i, j, imax(k - 1, 0)) + AT(*r0, i, j, k));
          dv[c] = fx / dx + fy / dy + fz / dz;
        }
        const double G = dv[0] + half_dt * dv[1];
        const double c = (K_RD / K_CV) * (AT(*pi0, i, j, k) / dmax(AT(*r0, i, j, k), 1e-8));
        const double a0 = AT(*acoef, i, j, k);
        const fld *pi = &st[VO_PI];
        const double pc = AT(*pi, i, j, k);
        const double div_a_grad =
            (a0 * (AT(*pi, imin(i + 1, nx - 1), j, k) - pc) - a0 * (pc - AT(*pi, imax(i - 1, 0), j, k))) / (dx * dx) +
            (a0 * (AT(*pi, i, imin(j + 1, ny - 1), k) - pc) - a0 * (pc - AT(*pi, i, imax(j - 1, 0), k))) / (dy * dy);
        AT(*rhs, i, j, k) = pc - dt * c * G + div_a_grad;
      }
}

/* SemiImplicitIntegrator::step, semi_implicit.cpp:167-226 (O-SI). The
 * shipped step does not compile (State::add_scaled(Real, Tendency),
 * :182); restated with that update expanded field by field. Observable
 * effects kept: the Helmholtz solve (its solution and statistics), the
 * explicit theta/qv/rho/moisture update, the sponge and the non-finite check.
 * The shipped step writes the solved pressure only into its local copy
 * s_explicit (update_from_pressure, :188), which it then drops, so u, v, w
 * and pi of the state change only through the sponge; that copy is not
 * formed here. No physics driver, RA filter off (its default). */
int vo_si_step(vo_model *m, double dt, int kind, int max_iter, double tol, int *iterations, double *residual,
               double *pi_new, double *rhs_out, double *a_out) {
  fld acoef = fld_cell(m), bcoef = fld_cell(m), rhs = fld_cell(m), x = fld_cell(m);
  slow_tendency_split(m, m->st, m->slow);
  si_assemble(m, m->st, m->slow, dt, &acoef, &bcoef, &rhs);
  int it = 0;
  double res = 0.0;
  int rc = h_solve(m, kind, max_iter, tol, 1, &acoef, &bcoef, &rhs, &x, &it, &res);
  if (iterations) *iterations = it;
  if (residual) *residual = res;
  if (pi_new) memcpy(pi_new, x.d, fld_size(&x) * sizeof(double));
  if (rhs_out) memcpy(rhs_out, rhs.d, fld_size(&rhs) * sizeof(double));
  if (a_out) memcpy(a_out, acoef.d, fld_size(&acoef) * sizeof(double));
  free(acoef.d); free(bcoef.d); free(rhs.d); free(x.d);
  if (rc) return 2;
  add_scaled(&m->st[VO_THETA], dt, &m->slow[VO_THETA]);
  add_scaled(&m->st[VO_QV], dt, &m->slow[VO_QV]);
  add_scaled(&m->st[VO_RHO], dt, &m->slow[VO_RHO]);
  for (int sp = VO_QC; sp <= VO_QG; ++sp) add_scaled(&m->st[sp], dt, &m->slow[sp]);
  sponge_apply(m, dt);
  return has_nonfinite(m) ? 1 : 0;
}

/* ------------------------------------------------------------------------ */
/* TL/AD of the simplified collocated RK3: src/da/tangent_linear.cpp        */
/* ------------------------------------------------------------------------ */
/* Grid::inv_dz, geometry.cpp:265-270 (no 1 m floor here) */
static double g_inv_dz(const vo_model *m, int i, int j, int k) {
  const double dz = g_dzeta(m, k) * (m->s.z_top - g_terrain(m, i, j));
  return dz > 0.0 ? 1.0 / dz : 0.0;
}
static fld sp_view(const vo_model *m, int sp, const double *p) { fld f = m->st[sp]; f.d = (double *)p; return f; }

/* dop_x/y/z, tangent_linear.cpp:82-122: out += scale * c * (f(+1) - f(-1)) * inv, interior */
static void dop(const vo_model *m, int dir, const fld *f, const fld *c, fld *out, double scale) {
  const int nx = m->nx, ny = m->ny, nz = m->nz;
  if (dir == 0) {
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 1; i + 1 < nx; ++i) {
          const double inv = 0.5 / dmax(m->s.dx, 1e-6);
          AT(*out, i, j, k) += scale * AT(*c, i, j, k) * (AT(*f, i + 1, j, k) - AT(*f, i - 1, j, k)) * inv;
        }
  } else if (dir == 1) {
    for (int k = 0; k < nz; ++k)
      for (int j = 1; j + 1 < ny; ++j) {
        const double inv = 0.5 / dmax(m->s.dy, 1e-6);
        for (int i = 0; i < nx; ++i)
          AT(*out, i, j, k) += scale * AT(*c, i, j, k) * (AT(*f, i, j + 1, k) - AT(*f, i, j - 1, k)) * inv;
      }
  } else {
    for (int k = 1; k + 1 < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
          const double inv = 0.5 * g_inv_dz(m, i, j, k);
          AT(*out, i, j, k) += scale * AT(*c, i, j, k) * (AT(*f, i, j, k + 1) - AT(*f, i, j, k - 1)) * inv;
        }
  }
}
/* dop_*_ad_f, tangent_linear.cpp:124-205: transpose in the differentiated field */
static void dop_ad_f(const vo_model *m, int dir, const fld *c, fld *bar_f, const fld *bar_out, double scale) {
  const int nx = m->nx, ny = m->ny, nz = m->nz;
  if (dir == 0) {
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 1; i + 1 < nx; ++i) {
          const double inv = 0.5 / dmax(m->s.dx, 1e-6);
          const double w = scale * AT(*c, i, j, k) * inv * AT(*bar_out, i, j, k);
          AT(*bar_f, i + 1, j, k) += w;
          AT(*bar_f, i - 1, j, k) -= w;
        }
  } else if (dir == 1) {
    for (int k = 0; k < nz; ++k)
      for (int j = 1; j + 1 < ny; ++j) {
        const double inv = 0.5 / dmax(m->s.dy, 1e-6);
        for (int i = 0; i < nx; ++i) {
          const double w = scale * AT(*c, i, j, k) * inv * AT(*bar_out, i, j, k);
          AT(*bar_f, i, j + 1, k) += w;
          AT(*bar_f, i, j - 1, k) -= w;
        }
      }
  } else {
    for (int k = 1; k + 1 < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
          const double inv = 0.5 * g_inv_dz(m, i, j, k);
          const double w = scale * AT(*c, i, j, k) * inv * AT(*bar_out, i, j, k);
          AT(*bar_f, i, j, k + 1) += w;
          AT(*bar_f, i, j, k - 1) -= w;
        }
  }
}
/* dop_*_ad_c: transpose in the (perturbed) coefficient */
static void dop_ad_c(const vo_model *m, int dir, const fld *f, fld *bar_c, const fld *bar_out, double scale) {
  const int nx = m->nx, ny = m->ny, nz = m->nz;
  if (dir == 0) {
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 1; i + 1 < nx; ++i) {
          const double inv = 0.5 / dmax(m->s.dx, 1e-6);
          AT(*bar_c, i, j, k) += scale * AT(*bar_out, i, j, k) * (AT(*f, i + 1, j, k) - AT(*f, i - 1, j, k)) * inv;
        }
  } else if (dir == 1) {
    for (int k = 0; k < nz; ++k)
      for (int j = 1; j + 1 < ny; ++j) {
        const double inv = 0.5 / dmax(m->s.dy, 1e-6);
        for (int i = 0; i < nx; ++i)
          AT(*bar_c, i, j, k) += scale * AT(*bar_out, i, j, k) * (AT(*f, i, j + 1, k) - AT(*f, i, j - 1, k)) * inv;
      }
  } else {
    for (int k = 1; k + 1 < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
          const double inv = 0.5 * g_inv_dz(m, i, j, k);
          AT(*bar_c, i, j, k) += scale * AT(*bar_out, i, j, k) * (AT(*f, i, j, k + 1) - AT(*f, i, j, k - 1)) * inv;
        }
  }
}
/* base_divergence (:207-235) and base_gradient (:237-266) */
static void base_div(const vo_model *m, const fld *ub, const fld *vb, const fld *wb, fld *div) {
  const int nx = m->nx, ny = m->ny, nz = m->nz;
  fld_zero(div);
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        double d = 0.0;
        if (i >= 1 && i + 1 < nx) d += (AT(*ub, i + 1, j, k) - AT(*ub, i - 1, j, k)) * (0.5 / dmax(m->s.dx, 1e-6));
        if (j >= 1 && j + 1 < ny) d += (AT(*vb, i, j + 1, k) - AT(*vb, i, j - 1, k)) * (0.5 / dmax(m->s.dy, 1e-6));
        if (k >= 1 && k + 1 < nz) d += (AT(*wb, i, j, k + 1) - AT(*wb, i, j, k - 1)) * (0.5 * g_inv_dz(m, i, j, k));
        AT(*div, i, j, k) = d;
      }
}
static void base_grad(const vo_model *m, const fld *f, fld *gx, fld *gy, fld *gz) {
  const int nx = m->nx, ny = m->ny, nz = m->nz;
  fld_zero(gx); fld_zero(gy); fld_zero(gz);
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        if (i >= 1 && i + 1 < nx) AT(*gx, i, j, k) = (AT(*f, i + 1, j, k) - AT(*f, i - 1, j, k)) * (0.5 / dmax(m->s.dx, 1e-6));
        if (j >= 1 && j + 1 < ny) AT(*gy, i, j, k) = (AT(*f, i, j + 1, k) - AT(*f, i, j - 1, k)) * (0.5 / dmax(m->s.dy, 1e-6));
        if (k >= 1 && k + 1 < nz) AT(*gz, i, j, k) = (AT(*f, i, j, k + 1) - AT(*f, i, j, k - 1)) * (0.5 * g_inv_dz(m, i, j, k));
      }
}
static double tl_coriolis(void) { return 2.0 * K_OMEGA * sin(45.0 * (K_PI / 180.0)); } /* kCoriolis, :79 */
static const int kTlScalars[7] = {VO_THETA, VO_QV, VO_QC, VO_QR, VO_QI, VO_QS, VO_QG};

/* tendency_tl, tangent_linear.cpp:295-412 */
static void tl_tendency(const vo_model *m, fld *xb, fld *dx, fld *d) {
  const int nx = m->nx, ny = m->ny, nz = m->nz;
  const double rdcv = K_RD / K_CV, fc = tl_coriolis();
  for (int sp = 0; sp < VO_NSPECIES; ++sp) fld_zero(&d[sp]);
  fld *ub = &xb[VO_U], *vb = &xb[VO_V], *wb = &xb[VO_W];
  fld *rhob = &xb[VO_RHO], *thb = &xb[VO_THETA], *pib = &xb[VO_PI];
  fld *du = &dx[VO_U], *dv = &dx[VO_V], *dw = &dx[VO_W], *drho = &dx[VO_RHO], *dth = &dx[VO_THETA], *dpi = &dx[VO_PI];
  fld div = fld_cell(m);
  base_div(m, ub, vb, wb, &div);
  for (int si = 0; si < 7; ++si) {
    const int sp = kTlScalars[si];
    fld *sb = &xb[sp], *ds = &dx[sp], *out = &d[sp];
    dop(m, 0, ds, ub, out, -1.0); dop(m, 1, ds, vb, out, -1.0); dop(m, 2, ds, wb, out, -1.0);
    dop(m, 0, sb, du, out, -1.0); dop(m, 1, sb, dv, out, -1.0); dop(m, 2, sb, dw, out, -1.0);
  }
  {
    fld *out = &d[VO_RHO];
    dop(m, 0, du, rhob, out, -1.0); dop(m, 1, dv, rhob, out, -1.0); dop(m, 2, dw, rhob, out, -1.0);
    dop(m, 0, drho, ub, out, -1.0); dop(m, 1, drho, vb, out, -1.0); dop(m, 2, drho, wb, out, -1.0);
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) AT(*out, i, j, k) -= AT(div, i, j, k) * AT(*drho, i, j, k);
    fld gx = fld_cell(m), gy = fld_cell(m), gz = fld_cell(m);
    base_grad(m, rhob, &gx, &gy, &gz);
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i)
          AT(*out, i, j, k) -= AT(*du, i, j, k) * AT(gx, i, j, k) + AT(*dv, i, j, k) * AT(gy, i, j, k) +
                               AT(*dw, i, j, k) * AT(gz, i, j, k);
    free(gx.d); free(gy.d); free(gz.d);
  }
  {
    fld *out = &d[VO_PI];
    dop(m, 0, dpi, ub, out, -1.0); dop(m, 1, dpi, vb, out, -1.0); dop(m, 2, dpi, wb, out, -1.0);
    dop(m, 0, pib, du, out, -1.0); dop(m, 1, pib, dv, out, -1.0); dop(m, 2, pib, dw, out, -1.0);
    dop(m, 0, du, pib, out, -rdcv); dop(m, 1, dv, pib, out, -rdcv); dop(m, 2, dw, pib, out, -rdcv);
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) AT(*out, i, j, k) -= rdcv * AT(div, i, j, k) * AT(*dpi, i, j, k);
  }
  {
    fld *out = &d[VO_U];
    dop(m, 0, du, ub, out, -1.0); dop(m, 1, du, vb, out, -1.0); dop(m, 2, du, wb, out, -1.0);
    dop(m, 0, ub, du, out, -1.0); dop(m, 1, ub, dv, out, -1.0); dop(m, 2, ub, dw, out, -1.0);
    dop(m, 0, dpi, thb, out, -K_CP); dop(m, 0, pib, dth, out, -K_CP);
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) AT(*out, i, j, k) += fc * AT(*dv, i, j, k);
  }
  {
    fld *out = &d[VO_V];
    dop(m, 0, dv, ub, out, -1.0); dop(m, 1, dv, vb, out, -1.0); dop(m, 2, dv, wb, out, -1.0);
    dop(m, 0, vb, du, out, -1.0); dop(m, 1, vb, dv, out, -1.0); dop(m, 2, vb, dw, out, -1.0);
    dop(m, 1, dpi, thb, out, -K_CP); dop(m, 1, pib, dth, out, -K_CP);
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) AT(*out, i, j, k) -= fc * AT(*du, i, j, k);
  }
  {
    fld *out = &d[VO_W];
    dop(m, 0, dw, ub, out, -1.0); dop(m, 1, dw, vb, out, -1.0); dop(m, 2, dw, wb, out, -1.0);
    dop(m, 0, wb, du, out, -1.0); dop(m, 1, wb, dv, out, -1.0); dop(m, 2, wb, dw, out, -1.0);
    dop(m, 2, dpi, thb, out, -K_CP); dop(m, 2, pib, dth, out, -K_CP);
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
          const double th = dmax(AT(*thb, i, j, k), 1.0);
          AT(*out, i, j, k) += K_GRAVITY * AT(*dth, i, j, k) / th;
        }
  }
  free(div.d);
}

/* tendency_ad, tangent_linear.cpp:414-549: the statements of tendency_tl in
 * reverse order, each replaced by its transpose; accumulates into bar_dx */
static void ad_tendency(const vo_model *m, fld *xb, fld *bd, fld *bx) {
  const int nx = m->nx, ny = m->ny, nz = m->nz;
  const double rdcv = K_RD / K_CV, fc = tl_coriolis();
  fld *ub = &xb[VO_U], *vb = &xb[VO_V], *wb = &xb[VO_W];
  fld *rhob = &xb[VO_RHO], *thb = &xb[VO_THETA], *pib = &xb[VO_PI];
  fld div = fld_cell(m);
  base_div(m, ub, vb, wb, &div);
  {
    fld *bo = &bd[VO_W];
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
          const double th = dmax(AT(*thb, i, j, k), 1.0);
          AT(bx[VO_THETA], i, j, k) += K_GRAVITY * AT(*bo, i, j, k) / th;
        }
    dop_ad_c(m, 2, pib, &bx[VO_THETA], bo, -K_CP);
    dop_ad_f(m, 2, thb, &bx[VO_PI], bo, -K_CP);
    dop_ad_c(m, 2, wb, &bx[VO_W], bo, -1.0);
    dop_ad_c(m, 1, wb, &bx[VO_V], bo, -1.0);
    dop_ad_c(m, 0, wb, &bx[VO_U], bo, -1.0);
    dop_ad_f(m, 2, wb, &bx[VO_W], bo, -1.0);
    dop_ad_f(m, 1, vb, &bx[VO_W], bo, -1.0);
    dop_ad_f(m, 0, ub, &bx[VO_W], bo, -1.0);
  }
  {
    fld *bo = &bd[VO_V];
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) AT(bx[VO_U], i, j, k) -= fc * AT(*bo, i, j, k);
    dop_ad_c(m, 1, pib, &bx[VO_THETA], bo, -K_CP);
    dop_ad_f(m, 1, thb, &bx[VO_PI], bo, -K_CP);
    dop_ad_c(m, 2, vb, &bx[VO_W], bo, -1.0);
    dop_ad_c(m, 1, vb, &bx[VO_V], bo, -1.0);
    dop_ad_c(m, 0, vb, &bx[VO_U], bo, -1.0);
    dop_ad_f(m, 2, wb, &bx[VO_V], bo, -1.0);
    dop_ad_f(m, 1, vb, &bx[VO_V], bo, -1.0);
    dop_ad_f(m, 0, ub, &bx[VO_V], bo, -1.0);
  }
  {
    fld *bo = &bd[VO_U];
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) AT(bx[VO_V], i, j, k) += fc * AT(*bo, i, j, k);
    dop_ad_c(m, 0, pib, &bx[VO_THETA], bo, -K_CP);
    dop_ad_f(m, 0, thb, &bx[VO_PI], bo, -K_CP);
    dop_ad_c(m, 2, ub, &bx[VO_W], bo, -1.0);
    dop_ad_c(m, 1, ub, &bx[VO_V], bo, -1.0);
    dop_ad_c(m, 0, ub, &bx[VO_U], bo, -1.0);
    dop_ad_f(m, 2, wb, &bx[VO_U], bo, -1.0);
    dop_ad_f(m, 1, vb, &bx[VO_U], bo, -1.0);
    dop_ad_f(m, 0, ub, &bx[VO_U], bo, -1.0);
  }
  {
    fld *bo = &bd[VO_PI];
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) AT(bx[VO_PI], i, j, k) -= rdcv * AT(div, i, j, k) * AT(*bo, i, j, k);
    dop_ad_f(m, 2, pib, &bx[VO_W], bo, -rdcv);
    dop_ad_f(m, 1, pib, &bx[VO_V], bo, -rdcv);
    dop_ad_f(m, 0, pib, &bx[VO_U], bo, -rdcv);
    dop_ad_c(m, 2, pib, &bx[VO_W], bo, -1.0);
    dop_ad_c(m, 1, pib, &bx[VO_V], bo, -1.0);
    dop_ad_c(m, 0, pib, &bx[VO_U], bo, -1.0);
    dop_ad_f(m, 2, wb, &bx[VO_PI], bo, -1.0);
    dop_ad_f(m, 1, vb, &bx[VO_PI], bo, -1.0);
    dop_ad_f(m, 0, ub, &bx[VO_PI], bo, -1.0);
  }
  {
    fld *bo = &bd[VO_RHO];
    fld gx = fld_cell(m), gy = fld_cell(m), gz = fld_cell(m);
    base_grad(m, rhob, &gx, &gy, &gz);
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
          const double b = AT(*bo, i, j, k);
          AT(bx[VO_U], i, j, k) -= AT(gx, i, j, k) * b;
          AT(bx[VO_V], i, j, k) -= AT(gy, i, j, k) * b;
          AT(bx[VO_W], i, j, k) -= AT(gz, i, j, k) * b;
        }
    free(gx.d); free(gy.d); free(gz.d);
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) AT(bx[VO_RHO], i, j, k) -= AT(div, i, j, k) * AT(*bo, i, j, k);
    dop_ad_f(m, 2, wb, &bx[VO_RHO], bo, -1.0);
    dop_ad_f(m, 1, vb, &bx[VO_RHO], bo, -1.0);
    dop_ad_f(m, 0, ub, &bx[VO_RHO], bo, -1.0);
    dop_ad_f(m, 2, rhob, &bx[VO_W], bo, -1.0);
    dop_ad_f(m, 1, rhob, &bx[VO_V], bo, -1.0);
    dop_ad_f(m, 0, rhob, &bx[VO_U], bo, -1.0);
  }
  for (int si = 6; si >= 0; --si) {
    const int sp = kTlScalars[si];
    fld *sb = &xb[sp], *bs = &bx[sp], *bo = &bd[sp];
    dop_ad_c(m, 2, sb, &bx[VO_W], bo, -1.0);
    dop_ad_c(m, 1, sb, &bx[VO_V], bo, -1.0);
    dop_ad_c(m, 0, sb, &bx[VO_U], bo, -1.0);
    dop_ad_f(m, 2, wb, bs, bo, -1.0);
    dop_ad_f(m, 1, vb, bs, bo, -1.0);
    dop_ad_f(m, 0, ub, bs, bo, -1.0);
  }
  free(div.d);
}

static void views12(const vo_model *m, const double *const *p, fld *out) {
  for (int sp = 0; sp < VO_NSPECIES; ++sp) out[sp] = sp_view(m, sp, p[sp]);
}
static void alloc12(const vo_model *m, fld *out) {
  for (int sp = 0; sp < VO_NSPECIES; ++sp) fld_alloc(&out[sp], m->nx, m->ny, m->nz, stagger_of(sp));
}
static void free12(fld *f) { for (int sp = 0; sp < VO_NSPECIES; ++sp) free(f[sp].d); }

void vo_tl_tendency(const vo_model *m, const double *const *xb, const double *const *dx, double *const *d) {
  fld X[VO_NSPECIES], D[VO_NSPECIES], O[VO_NSPECIES];
  views12(m, xb, X); views12(m, dx, D); views12(m, (const double *const *)d, O);
  tl_tendency(m, X, D, O);
}
void vo_ad_tendency(const vo_model *m, const double *const *xb, const double *const *bar_d, double *const *bar_dx) {
  fld X[VO_NSPECIES], B[VO_NSPECIES], O[VO_NSPECIES];
  views12(m, xb, X); views12(m, bar_d, B); views12(m, (const double *const *)bar_dx, O);
  ad_tendency(m, X, B, O);
}

/* nl_tendency of the reference's TL/AD test (tests/unit/test_tl_ad.cpp:100-180):
 * the nonlinear collocated tendency whose Jacobian at xb is tl_tendency; the
 * buoyancy g (theta/max(theta_b, 1) - 1) takes theta_b from the base xb. */
static void nl_tendency(const vo_model *m, fld *xb, fld *x, fld *d) {
  const int nx = m->nx, ny = m->ny, nz = m->nz;
  const double rdcv = K_RD / K_CV, fc = tl_coriolis();
  for (int sp = 0; sp < VO_NSPECIES; ++sp) fld_zero(&d[sp]);
  fld *u = &x[VO_U], *v = &x[VO_V], *w = &x[VO_W], *rho = &x[VO_RHO], *th = &x[VO_THETA], *pi = &x[VO_PI];
  for (int si = 0; si < 7; ++si) {
    const int sp = kTlScalars[si];
    fld *q = &x[sp], *out = &d[sp];
    dop(m, 0, q, u, out, -1.0); dop(m, 1, q, v, out, -1.0); dop(m, 2, q, w, out, -1.0);
  }
  {
    fld *out = &d[VO_RHO];
    dop(m, 0, u, rho, out, -1.0); dop(m, 1, v, rho, out, -1.0); dop(m, 2, w, rho, out, -1.0);
    dop(m, 0, rho, u, out, -1.0); dop(m, 1, rho, v, out, -1.0); dop(m, 2, rho, w, out, -1.0);
  }
  {
    fld *out = &d[VO_PI];
    dop(m, 0, pi, u, out, -1.0); dop(m, 1, pi, v, out, -1.0); dop(m, 2, pi, w, out, -1.0);
    dop(m, 0, u, pi, out, -rdcv); dop(m, 1, v, pi, out, -rdcv); dop(m, 2, w, pi, out, -rdcv);
  }
  {
    fld *out = &d[VO_U];
    dop(m, 0, u, u, out, -1.0); dop(m, 1, u, v, out, -1.0); dop(m, 2, u, w, out, -1.0);
    dop(m, 0, pi, th, out, -K_CP);
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) AT(*out, i, j, k) += fc * AT(*v, i, j, k);
  }
  {
    fld *out = &d[VO_V];
    dop(m, 0, v, u, out, -1.0); dop(m, 1, v, v, out, -1.0); dop(m, 2, v, w, out, -1.0);
    dop(m, 1, pi, th, out, -K_CP);
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) AT(*out, i, j, k) -= fc * AT(*u, i, j, k);
  }
  {
    fld *out = &d[VO_W];
    dop(m, 0, w, u, out, -1.0); dop(m, 1, w, v, out, -1.0); dop(m, 2, w, w, out, -1.0);
    dop(m, 2, pi, th, out, -K_CP);
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
          const double tb = dmax(AT(xb[VO_THETA], i, j, k), 1.0);
          AT(*out, i, j, k) += K_GRAVITY * (AT(*th, i, j, k) / tb - 1.0);
        }
  }
}

void vo_nl_tendency(const vo_model *m, const double *const *xb, const double *const *x, double *const *d) {
  fld X[VO_NSPECIES], XN[VO_NSPECIES], D[VO_NSPECIES];
  views12(m, xb, X); views12(m, x, XN); views12(m, (const double *const *)d, D);
  nl_tendency(m, X, XN, D);
}

/* nl_rk3 of the same test (test_tl_ad.cpp:186-199): one step */
void vo_nl_step(const vo_model *m, const double *const *xb, const double *const *x, double dt, double *const *out) {
  fld X[VO_NSPECIES], XN[VO_NSPECIES], OUT[VO_NSPECIES], d[VO_NSPECIES], s1[VO_NSPECIES];
  views12(m, xb, X); views12(m, x, XN); views12(m, (const double *const *)out, OUT);
  alloc12(m, d); alloc12(m, s1);
  const double a[3] = {dt / 3.0, dt / 2.0, dt};
  fld *in = XN;
  for (int st = 0; st < 3; ++st) {
    nl_tendency(m, X, in, d);
    fld *dst = (st == 2) ? OUT : s1;
    for (int sp = 0; sp < VO_NSPECIES; ++sp) {
      fld_copy(&dst[sp], &XN[sp]);
      add_scaled(&dst[sp], a[st], &d[sp]);
    }
    in = s1;
  }
  free12(d); free12(s1);
}

/* rk3_tl, tangent_linear.cpp:559-572 (state_add_tendency over all storage) */
void vo_tl_step(const vo_model *m, const double *const *xb, const double *const *dx, double dt, double *const *out) {
  fld X[VO_NSPECIES], DX[VO_NSPECIES], OUT[VO_NSPECIES], d[VO_NSPECIES], s1[VO_NSPECIES];
  views12(m, xb, X); views12(m, dx, DX); views12(m, (const double *const *)out, OUT);
  alloc12(m, d); alloc12(m, s1);
  const double a[3] = {dt / 3.0, dt / 2.0, dt};
  fld *in = DX;
  for (int st = 0; st < 3; ++st) {
    tl_tendency(m, X, in, d);
    fld *dst = (st == 2) ? OUT : s1;
    for (int sp = 0; sp < VO_NSPECIES; ++sp) {
      fld_copy(&dst[sp], &DX[sp]);
      add_scaled(&dst[sp], a[st], &d[sp]);
    }
    in = s1;
  }
  free12(d); free12(s1);
}

/* rk3_ad, tangent_linear.cpp:574-603 */
void vo_ad_step(const vo_model *m, const double *const *xb, const double *const *bar_out, double dt,
                double *const *bar_in) {
  fld X[VO_NSPECIES], BO[VO_NSPECIES], BI[VO_NSPECIES], bd[VO_NSPECIES], bx[VO_NSPECIES];
  views12(m, xb, X); views12(m, bar_out, BO); views12(m, (const double *const *)bar_in, BI);
  alloc12(m, bd); alloc12(m, bx);
  for (int sp = 0; sp < VO_NSPECIES; ++sp) fld_copy(&BI[sp], &BO[sp]);
  const double a[3] = {dt, dt / 2.0, dt / 3.0};
  fld *src = BO;
  fld prev[VO_NSPECIES];
  alloc12(m, prev);
  for (int st = 0; st < 3; ++st) {
    for (int sp = 0; sp < VO_NSPECIES; ++sp) {
      fld_zero(&bd[sp]);
      add_scaled(&bd[sp], a[st], &src[sp]);
      fld_zero(&bx[sp]);
    }
    ad_tendency(m, X, bd, bx);
    for (int sp = 0; sp < VO_NSPECIES; ++sp) {
      add_scaled(&BI[sp], 1.0, &bx[sp]);
      fld_copy(&prev[sp], &bx[sp]);
    }
    src = prev;
  }
  free12(bd); free12(bx); free12(prev);
}

/* ------------------------------------------------------------------------ */
/* Time-step diagnostics                                                     */
/* ------------------------------------------------------------------------ */
void vo_cfl(const vo_model *m, double dt, double dtau, double *adv_cfl, double *max_sound_speed,
            double *acoustic_cfl) {
  const fld *u = &m->st[VO_U], *v = &m->st[VO_V], *w = &m->st[VO_W], *th = &m->st[VO_THETA], *pi = &m->st[VO_PI];
  double worst = 0.0, best = 0.0, ac = 0.0;
  for (int k = 0; k < m->nz; ++k)
    for (int j = 0; j < m->ny; ++j)
      for (int i = 0; i < m->nx; ++i) {
        const double dx = m->s.dx, dy = m->s.dy;
        const double scale = m->s.z_top - g_terrain(m, i, j);
        const double dz = dmax(g_dzeta(m, k) * scale, 1.0);
        const double uu = 0.5 * (AT(*u, i, j, k) + AT(*u, i + 1, j, k));
        const double vv = 0.5 * (AT(*v, i, j, k) + AT(*v, i, j + 1, k));
        const double ww = 0.5 * (AT(*w, i, j, k) + AT(*w, i, j, k + 1));
        /* cfl_number, advection.cpp:325-340 */
        worst = dmax(worst, dt * (fabs(uu) / dx + fabs(vv) / dy + fabs(ww) / dz));
        /* max_sound_speed, equations.cpp:238-249 */
        const double t = AT(*th, i, j, k) * AT(*pi, i, j, k);
        const double cs = sqrt((K_CP / K_CV) * K_RD * dmax(t, 1.0));
        best = dmax(best, cs);
        /* acoustic_cfl, acoustic_substep.cpp:151-168 */
        ac = dmax(ac, dtau * ((cs + fabs(uu)) / dx + (cs + fabs(vv)) / dy + (cs + fabs(ww)) / dz));
      }
  if (adv_cfl) *adv_cfl = worst;
  if (max_sound_speed) *max_sound_speed = best;
  if (acoustic_cfl) *acoustic_cfl = ac;
}

/* RungeKutta3Integrator::max_stable_dt, runge_kutta.cpp:121-140 */
double vo_max_stable_dt(const vo_model *m) {
  double adv = 0.0, cs = 0.0;
  vo_cfl(m, 1.0, 1.0, &adv, &cs, NULL);
  double rate = 0.0;
  for (int k = 0; k < m->nz; ++k)
    for (int j = 0; j < m->ny; ++j)
      for (int i = 0; i < m->nx; ++i) {
        const double scale = m->s.z_top - g_terrain(m, i, j);
        const double dz = dmax(g_dzeta(m, k) * scale, 1.0);
        rate = dmax(rate, cs * (1.0 / m->s.dx + 1.0 / m->s.dy + 1.0 / dz));
      }
  const double dt_adv = (adv > 0.0) ? 0.8 / adv : 1e9;
  const double dt_ac = (rate > 0.0) ? 2.0 / rate : 1e9;
  return dmin(dt_adv, dt_ac);
}

/* ------------------------------------------------------------------------ */
/* Nest transfers: src/grid/nest.cpp:34-124                                  */
/* ------------------------------------------------------------------------ */
static fld fld_of(int nx, int ny, int nz, int stagger, const double *p) {
  fld f;
  f.nx = nx; f.ny = ny; f.nz = nz;
  f.nsx = nx + 2 * VO_HALO + (stagger == 1);
  f.nsy = ny + 2 * VO_HALO + (stagger == 2);
  f.nsz = nz + 2 * VO_HALO + (stagger == 3);
  f.d = (double *)p;
  return f;
}

/* davies_profile, nest.cpp:34-44 */
void vo_davies_profile(int n_zone, double alpha_max, double *out) {
  for (int n = 0; n < n_zone; ++n) {
    const double arg = K_PI * (double)(n_zone - n) / (double)n_zone;
    out[n] = alpha_max * 0.5 * (1.0 - cos(arg));
  }
}

/* Nest::interpolate_from_parent, nest.cpp:58-84: child point (i, j) at
 * parent coordinate ((i0 + i) + 0.5)/r - 0.5, bilinear with the parent's
 * clamp; every stagger uses the cell-centre formula over the grid's nx x ny */
void vo_nest_interpolate_from_parent(const vo_nest_placement *p, int nvars, const int *stagger, int pnx, int pny,
                                     int pnz, const double *const *parent, int cnx, int cny, int cnz,
                                     double *const *child) {
  const double inv = 1.0 / (double)p->ratio;
  for (int v = 0; v < nvars; ++v) {
    const fld src = fld_of(pnx, pny, pnz, stagger[v], parent[v]);
    fld dst = fld_of(cnx, cny, cnz, stagger[v], child[v]);
    for (int k = 0; k < cnz; ++k)
      for (int j = 0; j < cny; ++j)
        for (int i = 0; i < cnx; ++i) {
          const double xp = ((double)(p->i0 + i) + 0.5) * inv - 0.5;
          const double yp = ((double)(p->j0 + j) + 0.5) * inv - 0.5;
          const int ip = (int)floor(xp), jp = (int)floor(yp);
          const double wx = xp - (double)ip, wy = yp - (double)jp;
          AT(dst, i, j, k) = lerp(lerp(CL(&src, ip, jp, k), CL(&src, ip + 1, jp, k), wx),
                                  lerp(CL(&src, ip, jp + 1, k), CL(&src, ip + 1, jp + 1, k), wx), wy);
        }
  }
}

/* Nest::restrict_to_parent, nest.cpp:86-105: parent (i0+i, j0+j, k) = mean of
 * the child's r x r points (jj outer, ii inner), i < iext, j < jext, k < the
 * parent's nz */
void vo_nest_restrict_to_parent(const vo_nest_placement *p, int nvars, const int *stagger, int cnx, int cny,
                                int cnz, const double *const *child, int pnx, int pny, int pnz,
                                double *const *parent) {
  const int r = p->ratio;
  const double w = 1.0 / (double)(r * r);
  for (int v = 0; v < nvars; ++v) {
    const fld src = fld_of(cnx, cny, cnz, stagger[v], child[v]);
    fld dst = fld_of(pnx, pny, pnz, stagger[v], parent[v]);
    for (int j = 0; j < p->jext; ++j)
      for (int i = 0; i < p->iext; ++i)
        for (int k = 0; k < pnz; ++k) {
          double acc = 0.0;
          for (int jj = 0; jj < r; ++jj)
            for (int ii = 0; ii < r; ++ii) acc += CL(&src, i * r + ii, j * r + jj, k);
          AT(dst, p->i0 + i, p->j0 + j, k) = acc * w;
        }
  }
}

/* Nest::apply_lateral_boundary, nest.cpp:107-124 */
void vo_nest_apply_lateral_boundary(const vo_nest_placement *p, int nvars, const int *stagger, int cnx, int cny,
                                    int cnz, double *const *child, const double *const *parent_interp) {
  const int nzone = p->boundary_zone > 0 ? p->boundary_zone : 0;
  double *davies = (double *)calloc((size_t)nzone + 1, sizeof(double));
  vo_davies_profile(nzone, 1.0, davies);
  for (int v = 0; v < nvars; ++v) {
    fld c = fld_of(cnx, cny, cnz, stagger[v], child[v]);
    const fld pi = fld_of(cnx, cny, cnz, stagger[v], parent_interp[v]);
    for (int k = 0; k < cnz; ++k)
      for (int j = 0; j < cny; ++j)
        for (int i = 0; i < cnx; ++i) {
          const int d = imin(imin(i, cnx - 1 - i), imin(j, cny - 1 - j));
          if (d >= nzone) continue;
          const double alpha = davies[d];
          AT(c, i, j, k) = (1.0 - alpha) * AT(c, i, j, k) + alpha * AT(pi, i, j, k);
        }
  }
  free(davies);
}

/* ------------------------------------------------------------------------ */
/* C-ABI kernels: src/common/c_kernels.c                                     */
/* ------------------------------------------------------------------------ */
int vo_tridiagonal_solve(const double *a, const double *b, const double *c, const double *d, int n,
                         double *x, double *ws) {
  /* argument checks and n==1 branch: c_kernels.c:22-29 */
  if (n <= 0 || b == NULL || d == NULL || x == NULL || ws == NULL) return 2;
  if (n == 1) {
    if (b[0] == 0.0) return 1;
    x[0] = d[0] / b[0];
    return 0;
  }
  /* contract c_kernels.h:38-55 (NULL a/c = 0) solved with the recurrence of
   * thomas_solve, helmholtz.cpp:71-85; ws holds the modified super-diagonal */
  double denom = b[0];
  if (denom == 0.0) return 1;
  ws[0] = (c != NULL ? c[0] : 0.0) / denom;
  x[0] = d[0] / denom;
  for (int k = 1; k < n; ++k) {
    const double am = (a != NULL) ? a[k - 1] : 0.0;
    denom = b[k] - am * ws[k - 1];
    if (denom == 0.0) return 1;
    x[k] = (d[k] - am * x[k - 1]) / denom;
    if (k < n - 1) ws[k] = (c != NULL ? c[k] : 0.0) / denom;
  }
  for (int k = n - 1; k-- > 0;) x[k] = x[k] - ws[k] * x[k + 1];
  return 0;
}

void vo_weno5_reconstruct(double qm2, double qm1, double q0, double q1, double q2, double *q_left,
                          double *q_right) {
  if (q_left == NULL || q_right == NULL) return; /* c_kernels.c:71 */
  weno5(qm2, qm1, q0, q1, q2, q_left, q_right);   /* c_kernels.c:64-104 == advection.cpp:62-98 */
}

double vo_bilinear(const double *f, int halo, int nsx, int nsy, int nz, double xi, double yj, int k) {
  /* c_kernels.c:108-144 */
  const int nxi = nsx - 2 * halo, nyi = nsy - 2 * halo;
  if (f == NULL || nz <= 0) return 0.0;
  if (k < 0) k = 0;
  if (k >= nz) k = nz - 1;
  const int i0 = (int)floor(xi), j0 = (int)floor(yj);
  const double wx = xi - (double)i0, wy = yj - (double)j0;
  /* c_kernels.c:128-135 clamps up to 0 first and then down to n-1 (with
   * n <= 0 the index ends at n-1, a halo point) */
  int ia = i0 < 0 ? 0 : i0, ib = i0 + 1 < 0 ? 0 : i0 + 1, ja = j0 < 0 ? 0 : j0, jb = j0 + 1 < 0 ? 0 : j0 + 1;
  if (ia > nxi - 1) ia = nxi - 1;
  if (ib > nxi - 1) ib = nxi - 1;
  if (ja > nyi - 1) ja = nyi - 1;
  if (jb > nyi - 1) jb = nyi - 1;
#define F_AT(I, J) f[(((size_t)(k + halo) * (size_t)nsy + (size_t)((J) + halo)) * (size_t)nsx) + (size_t)((I) + halo)]
  const double q00 = F_AT(ia, ja), q10 = F_AT(ib, ja), q01 = F_AT(ia, jb), q11 = F_AT(ib, jb);
#undef F_AT
  return (q00 + wx * (q10 - q00)) + wy * ((q01 + wx * (q11 - q01)) - (q00 + wx * (q10 - q00)));
}

double vo_cfl_scan(const double *u, const double *v, const double *w, const double *dzeta, const double *zs,
                   int nx, int ny, int nz, double dx, double dy, double z_top, double dt, double *max_wind_out,
                   double *min_dz_out) {
  /* c_kernels.c:148-186 */
  double worst = 0.0, max_wind = 0.0, min_dz = 1e30;
  const size_t nxy = (size_t)nx * (size_t)ny;
  if (u == NULL || v == NULL || w == NULL || dzeta == NULL) return 0.0;
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const size_t idx = (size_t)k * nxy + (size_t)j * (size_t)nx + (size_t)i;
        const double uu = u[idx], vv = v[idx], ww = w[idx];
        const double scale = (zs != NULL) ? (z_top - zs[(size_t)j * (size_t)nx + (size_t)i]) : z_top;
        double dz = dzeta[k] * scale;
        if (dz < 1.0) dz = 1.0;
        if (dz < min_dz) min_dz = dz;
        const double speed = sqrt(uu * uu + vv * vv + ww * ww);
        if (speed > max_wind) max_wind = speed;
        const double cfl = dt * (fabs(uu) / dx + fabs(vv) / dy + fabs(ww) / dz);
        if (cfl > worst) worst = cfl;
      }
  if (max_wind_out != NULL) *max_wind_out = max_wind;
  if (min_dz_out != NULL) *min_dz_out = (min_dz > 1e29) ? 0.0 : min_dz;
  return worst;
}

double vo_neumaier_sum(const double *x, size_t n) { /* c_kernels.c:190-205 */
  double sum = 0.0, c = 0.0;
  if (x == NULL) return 0.0;
  for (size_t i = 0; i < n; ++i) {
    const double t = sum + x[i];
    if (fabs(sum) >= fabs(x[i])) c += (sum - t) + x[i];
    else c += (x[i] - t) + sum;
    sum = t;
  }
  return sum + c;
}

void vo_advect_scalar_flux(const double *q, const double *rho, const double *u, const double *v, const double *w,
                           const double *dzeta, const double *zs, int nx, int ny, int nz, double dx, double dy,
                           double z_top, double *dqdt) {
  /* c_kernels.c:209-286 */
  const size_t nxy = (size_t)nx * (size_t)ny;
  const double inv_dx = 1.0 / dx, inv_dy = 1.0 / dy;
  if (q == NULL || rho == NULL || u == NULL || v == NULL || w == NULL || dzeta == NULL || dqdt == NULL) return;
  for (int k = 0; k < nz; ++k) {
    const size_t base_k = (size_t)k * nxy;
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const size_t idx = base_k + (size_t)j * (size_t)nx + (size_t)i;
        const double scale = (zs != NULL) ? (z_top - zs[(size_t)j * (size_t)nx + (size_t)i]) : z_top;
        double dz = dzeta[k] * scale;
        double fxE, fxW, fyN, fyS, fzT, fzB;
        if (dz < 1.0) dz = 1.0;
        {
          const size_t e = base_k + (size_t)j * (size_t)nx + (size_t)((i + 1) % nx);
          const size_t c = idx;
          const size_t ws = base_k + (size_t)j * (size_t)nx + (size_t)((i + nx - 1) % nx);
          fxE = u[e] * (0.5 * (rho[c] + rho[e])) * (0.5 * (q[c] + q[e]));
          fxW = u[c] * (0.5 * (rho[ws] + rho[c])) * (0.5 * (q[ws] + q[c]));
        }
        {
          const size_t e = base_k + (size_t)((j + 1) % ny) * (size_t)nx + (size_t)i;
          const size_t c = idx;
          const size_t s = base_k + (size_t)((j + ny - 1) % ny) * (size_t)nx + (size_t)i;
          fyN = v[e] * (0.5 * (rho[c] + rho[e])) * (0.5 * (q[c] + q[e]));
          fyS = v[c] * (0.5 * (rho[s] + rho[c])) * (0.5 * (q[s] + q[c]));
        }
        if (k > 0 && k + 1 < nz) {
          const size_t t = base_k + nxy + (size_t)j * (size_t)nx + (size_t)i;
          const size_t c = idx;
          const size_t b = base_k - nxy + (size_t)j * (size_t)nx + (size_t)i;
          fzT = w[t] * (0.5 * (rho[c] + rho[t])) * (0.5 * (q[c] + q[t]));
          fzB = w[c] * (0.5 * (rho[b] + rho[c])) * (0.5 * (q[b] + q[c]));
        } else {
          fzT = 0.0;
          fzB = 0.0;
        }
        const double div = (fxE - fxW) * inv_dx + (fyN - fyS) * inv_dy + (fzT - fzB) / dz;
        const double rr = (rho[idx] > 1e-12) ? rho[idx] : 1e-12;
        dqdt[idx] = -div / rr;
      }
  }
}


/* ---- .vibebin restart files (io::write_restart / read_restart,
 * src/io/field_io.cpp:175-250; byte layout src/io/binary_writer.cpp:1-20,
 * 271-320): header "VIBEBIN1", int32 nx ny nz real_kind(0), float64 time,
 * int32 nvars nlevels(=nz), then per variable char name[32] and its
 * float64 values over the stagger's points (u: nx+1 in i, v: ny+1 in j,
 * w: nz+1 in k; "__restart_info__" = [time, step]), i fastest; all
 * little-endian, assembled byte by byte. ---- */
static const char *const kSpeciesName[VO_NSPECIES] = {"u", "v", "w", "rho", "theta", "pi",
                                                      "qv", "qc", "qr", "qi", "qs", "qg"};
static void put_i32(FILE *f, int v) {
  const unsigned u = (unsigned)v;
  unsigned char b[4] = {(unsigned char)(u & 0xFFu), (unsigned char)((u >> 8) & 0xFFu),
                        (unsigned char)((u >> 16) & 0xFFu), (unsigned char)((u >> 24) & 0xFFu)};
  fwrite(b, 1, 4, f);
}
static void put_f64(FILE *f, double v) {
  unsigned long long u;
  unsigned char b[8];
  memcpy(&u, &v, 8);
  for (int i = 0; i < 8; ++i) b[i] = (unsigned char)((u >> (8 * i)) & 0xFFu);
  fwrite(b, 1, 8, f);
}
static int get_i32(FILE *f, int *v) {
  unsigned char b[4];
  if (fread(b, 1, 4, f) != 4) return 0;
  *v = (int)((unsigned)b[0] | ((unsigned)b[1] << 8) | ((unsigned)b[2] << 16) | ((unsigned)b[3] << 24));
  return 1;
}
static int get_f64(FILE *f, double *v) {
  unsigned char b[8];
  unsigned long long u = 0;
  if (fread(b, 1, 8, f) != 8) return 0;
  for (int i = 0; i < 8; ++i) u |= (unsigned long long)b[i] << (8 * i);
  memcpy(v, &u, 8);
  return 1;
}
static void shape_of(int sp, int nx, int ny, int nz, int *ni, int *nj, int *nk) {
  *ni = nx + (sp == VO_U);
  *nj = ny + (sp == VO_V);
  *nk = nz + (sp == VO_W);
}

int vo_write_restart(const vo_model *m, const char *path, double time, int step) {
  FILE *f = fopen(path, "wb");
  if (!f) return 1;
  fwrite("VIBEBIN1", 1, 8, f);
  put_i32(f, m->nx);
  put_i32(f, m->ny);
  put_i32(f, m->nz);
  put_i32(f, 0);
  put_f64(f, time);
  put_i32(f, 1 + VO_NSPECIES);
  put_i32(f, m->nz);
  char name[32];
  memset(name, 0, sizeof name);
  strcpy(name, "__restart_info__");
  fwrite(name, 1, 32, f);
  put_f64(f, time);
  put_f64(f, (double)step);
  for (int sp = 0; sp < VO_NSPECIES; ++sp) {
    memset(name, 0, sizeof name);
    strcpy(name, kSpeciesName[sp]);
    fwrite(name, 1, 32, f);
    int ni, nj, nk;
    shape_of(sp, m->nx, m->ny, m->nz, &ni, &nj, &nk);
    for (int k = 0; k < nk; ++k)
      for (int j = 0; j < nj; ++j)
        for (int i = 0; i < ni; ++i) put_f64(f, AT(m->st[sp], i, j, k));
  }
  return fclose(f) == 0 ? 0 : 1;
}

int vo_read_restart(vo_model *m, const char *path, double *time, int *step) {
  FILE *f = fopen(path, "rb");
  if (!f) return 1;
  char magic[8];
  int nx, ny, nz, kind, nvars, nlev;
  double t;
  int ok = fread(magic, 1, 8, f) == 8 && memcmp(magic, "VIBEBIN1", 8) == 0 && get_i32(f, &nx) && get_i32(f, &ny) &&
           get_i32(f, &nz) && get_i32(f, &kind) && get_f64(f, &t) && get_i32(f, &nvars) && get_i32(f, &nlev);
  ok = ok && nx == m->nx && ny == m->ny && nz == m->nz;
  double info[2] = {0.0, 0.0};
  for (int v = 0; ok && v < nvars; ++v) {
    char name[33];
    name[32] = 0;
    if (fread(name, 1, 32, f) != 32) { ok = 0; break; }
    if (strcmp(name, "__restart_info__") == 0) {
      ok = get_f64(f, &info[0]) && get_f64(f, &info[1]);
      continue;
    }
    int sp = -1;
    for (int q = 0; q < VO_NSPECIES; ++q)
      if (strcmp(name, kSpeciesName[q]) == 0) sp = q;
    /* the shape follows from the name (binary_writer.cpp:100-118) */
    const int st = (strcmp(name, "u") == 0 || strcmp(name, "u_facex") == 0) ? 1
                   : (strcmp(name, "v") == 0 || strcmp(name, "v_facey") == 0) ? 2
                   : (strcmp(name, "w") == 0 || strcmp(name, "zeta") == 0 || strcmp(name, "w_facez") == 0) ? 3 : 0;
    const int ni = nx + (st == 1), nj = ny + (st == 2), nk = nz + (st == 3);
    for (int k = 0; ok && k < nk; ++k)
      for (int j = 0; ok && j < nj; ++j)
        for (int i = 0; ok && i < ni; ++i) {
          double x;
          ok = get_f64(f, &x);
          if (ok && sp >= 0) AT(m->st[sp], i, j, k) = x;
        }
  }
  fclose(f);
  if (!ok) return 1;
  if (time) *time = info[0];
  if (step) *step = (int)llround(info[1]);
  return 0;
}


/* dyn::energy_budget (src/dyn/diagnostics.cpp:255-277), serial FP64 sums in
 * the reference's loop order; out6 = {kinetic, internal, potential, latent,
 * total, mass}. cell_volume = dx dy jacobian dzeta z_top (geometry.hpp:
 * 145-147), z_center = height(k + 1/2) (geometry.hpp:135-137). */
void vo_energy_budget(const vo_model *m, double *out6) {
  const int nx = m->nx, ny = m->ny, nz = m->nz;
  const double H = m->s.z_top, Lv = 2.501e6;
  double ke = 0, ie = 0, pe = 0, le = 0, mass = 0;
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const double zs = m->zs[(size_t)j * nx + i];
        const double dzeta = m->zeta[k + 1] - m->zeta[k];
        const double dv = m->s.dx * m->s.dy * ((H - zs) / H) * dzeta * H;
        const double rho = AT(m->st[VO_RHO], i, j, k);
        const double uc = 0.5 * (AT(m->st[VO_U], i, j, k) + AT(m->st[VO_U], i + 1, j, k));
        const double vc = 0.5 * (AT(m->st[VO_V], i, j, k) + AT(m->st[VO_V], i, j + 1, k));
        const double wc = 0.5 * (AT(m->st[VO_W], i, j, k) + AT(m->st[VO_W], i, j, k + 1));
        const double T = AT(m->st[VO_THETA], i, j, k) * AT(m->st[VO_PI], i, j, k);
        const double z = zs + 0.5 * (m->zeta[k] + m->zeta[k + 1]) * (H - zs);
        mass += rho * dv;
        ke += 0.5 * rho * (uc * uc + vc * vc + wc * wc) * dv;
        ie += rho * K_CV * T * dv;
        pe += rho * K_GRAVITY * z * dv;
        le += rho * Lv * dmax(AT(m->st[VO_QV], i, j, k), 0.0) * dv;
      }
  out6[0] = ke; out6[1] = ie; out6[2] = pe; out6[3] = le; out6[4] = ke + ie + pe + le; out6[5] = mass;
}
