"""Inputs of the TL/AD tests: a base state from the model's own set-up (warm
bubble over a stretched grid and a hill, with wind and shear) plus seeded
perturbations, and seeded TL inputs scaled per variable as the 4D-Var
configuration states (u, v, w: 1, 1, 0.1 m/s; theta 0.5 K; pi' from a 50 Pa
pressure perturbation)."""
import numpy as np

SCALE = [1.0, 1.0, 0.1, 1e-4, 0.5, 50.0 / 1e5 * 0.2857, 1e-4, 1e-5, 1e-5, 1e-5, 1e-5, 1e-5]


def tl_setup(oc, nx=14, ny=12, nz=10, **kw):
    s = oc.defaults()
    base = dict(nx=nx, ny=ny, nz=nz, dx=3000.0, dy=3000.0, z_top=15000.0, zeta_first=200.0, zeta_stretch=1.1,
                terrain_kind=1, hill_h=600.0, hill_a=9000.0, hill_xc=nx * 1500.0, hill_yc=ny * 1500.0,
                ref_kind=1, bv_n=0.01, u_background=10.0, shear_u=0.002, bubble_amplitude=1.5,
                bubble_xc=nx * 1200.0, bubble_yc=ny * 1600.0, bubble_zc=3000.0, bubble_radius_x=9000.0,
                bubble_radius_z=3000.0, qv_surface=0.01, moist=1)
    base.update(kw)
    for k, v in base.items():
        setattr(s, k, v)
    return s


def base_state(oc, model, seed=11):
    s = model.setup
    rng = np.random.default_rng(seed)
    xb = model.state()
    for sp, amp in ((0, 0.5), (1, 0.5), (2, 0.05), (4, 0.3)):
        oc.interior(s, sp, xb[sp])[...] += amp * rng.standard_normal(oc.interior(s, sp, xb[sp]).shape)
    for sp in range(7, 12):
        oc.interior(s, sp, xb[sp])[...] = 1e-4 * rng.random(oc.interior(s, sp, xb[sp]).shape)
    return xb


def perturbation(oc, model, seed):
    s = model.setup
    rng = np.random.default_rng(seed)
    dx = [np.zeros(model.size(sp)) for sp in range(12)]
    for sp in range(12):
        oc.interior(s, sp, dx[sp])[...] = SCALE[sp] * rng.standard_normal(oc.interior(s, sp, dx[sp]).shape)
    return dx


def dot(oc, s, a, b):
    return float(sum(np.sum(oc.interior(s, sp, a[sp]) * oc.interior(s, sp, b[sp])) for sp in range(12)))
