"""Shared Helmholtz problems for the CPU and GPU tests: the semi-implicit
step's operator on a small grid over a Gaussian hill (a = (dt/2)^2 (Rd/cv)
pi0 cp theta0, b = 1, f = the assembled right-hand side), and a mildly
scaled random operator on which the reference's Jacobi-BiCGSTAB converges."""
import numpy as np


def si_setup(oc, nx=32, ny=24, nz=16, **kw):
    s = oc.defaults()
    base = dict(nx=nx, ny=ny, nz=nz, dx=2000.0, dy=2000.0, z_top=20000.0, zeta_first=150.0, zeta_stretch=1.12,
                terrain_kind=1, hill_h=800.0, hill_a=10000.0, hill_xc=nx * 1000.0, hill_yc=ny * 1000.0,
                ref_kind=1, bv_n=0.01, profile_dz=250.0, u_background=15.0, shear_u=0.0,
                bubble_amplitude=0.5, bubble_xc=nx * 700.0, bubble_yc=ny * 1000.0, bubble_zc=3000.0,
                bubble_radius_x=6000.0, bubble_radius_z=2000.0,
                pgf_perturbation=0, split_fast=0, weno_advective=0, acoustic_mode=0, moist=0, qv_surface=0.0)
    base.update(kw)
    for k, v in base.items():
        setattr(s, k, v)
    return s


def si_problem(oc, s, dt=30.0):
    """(a, b, f, dzeta, zs) of one semi-implicit step's Helmholtz solve."""
    m = oc.Model(s, "port")
    rc, it, res, pin, rhs, acoef = m.si_step(dt, kind=0)
    assert rc == 0
    b = np.zeros_like(acoef)
    oc.interior(s, 3, b)[...] = 1.0
    return acoef, b, rhs, np.diff(m.zeta()), m.terrain()


def random_problem(oc, s, seed=0, scale=1e4):
    rng = np.random.default_rng(seed)
    n = int(np.prod(oc.storage_shape(s, 3)))
    a, b, f = np.zeros(n), np.zeros(n), np.zeros(n)
    oc.interior(s, 3, a)[...] = scale * (1 + rng.random(oc.interior(s, 3, a).shape))
    oc.interior(s, 3, b)[...] = 1.0
    oc.interior(s, 3, f)[...] = rng.standard_normal(oc.interior(s, 3, f).shape)
    return a, b, f
