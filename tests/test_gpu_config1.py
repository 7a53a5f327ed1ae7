"""The CPU-runnable warm-bubble case over its full length: 64 x 64 x 40,
dx = dy = dz = 250 m, isentropic theta0 = 300 K, +2 K bubble of radius 2 km at
(8 km, 8 km, 2 km), WENO5 scalars, dt = 2 s with 6 acoustic substeps per
stage, 100 steps, compared field by field against the oracle's FP64 run of
the same composition (the stable one: the reference's own composition is
non-finite within ~7 steps). Both acoustic solvers: the HEVI column
(Thomas) solve the case names (acoustic_mode 2, centred) and the explicit
forward-backward substep.

Bounds (relative to each field's scale; velocities to the common velocity
scale) after 100 steps: FP64 path 1e-11 (measured 2.4e-13 explicit), mixed
path 1e-5 (measured 6.8e-7 explicit)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STEPS = 100


def config1(vg):
    return vg.Setup.defaults(nx=64, ny=64, nz=40, dx=250.0, dy=250.0, z_top=10000.0, zeta_first=1.0,
                             zeta_stretch=1.0, ref_kind=0, theta0=300.0, p_surf=100000.0, bubble_amplitude=2.0,
                             bubble_radius_x=2000.0, bubble_radius_z=2000.0, bubble_xc=8000.0, bubble_yc=8000.0,
                             bubble_zc=2000.0, qv_surface=0.0, advection=5, weno_scalars=1, weno_advective=1,
                             pgf_perturbation=1, split_fast=1, acoustic_mode=0, u_background=0.0, shear_u=0.0)


def errors(vg, s, got, ref):
    ins = [vg.interior(s, q, ref[q]) for q in range(7)]
    vs = max(float(np.abs(ins[q]).max()) for q in range(3))
    out = {}
    for q in range(7):
        scale = vs if q < 3 else float(np.abs(ins[q]).max())
        d = vg.interior(s, q, got[q]) - ins[q]
        out[vg.SPECIES[q]] = (float(np.abs(d).max() / scale) if scale > 0 else float(np.abs(d).max()),
                              float(np.sqrt(np.mean(d * d)) / scale) if scale > 0 else 0.0)
    return out


@pytest.mark.parametrize("acoustic_mode", [2, 0], ids=["hevi", "explicit"])
def test_config1_100_steps(vg, oc, acoustic_mode):
    s = config1(vg)
    s.acoustic_mode = acoustic_mode
    s.hevi_beta = 0.5
    t = oc.Setup()
    for name, _ in oc.Setup._fields_:
        setattr(t, name, getattr(s, name))
    o = oc.Model(t, "port")
    for _ in range(STEPS):
        assert o.rk3_step(2.0, 6) == 0
    ref = [o.get(q) for q in range(7)]
    for prec, tol in ((vg.FP64, 1e-11), (vg.MIXED, 1e-5)):
        with vg.Model(s, prec) as m:
            m.step(2.0, 6, STEPS)
            err = errors(vg, s, m.state(), ref)
            print("config 1, acoustic mode %d, precision %d, max/rms relative error after %d steps: %s"
                  % (acoustic_mode, prec, STEPS, err))
            assert all(e[0] <= tol for e in err.values()), err


def test_config1_reference_composition_until_it_diverges(vg, oc):
    """O-RK3 as the reference writes it (every composition flag 0, 2nd-order
    advection, explicit substeps) on the same case: it stays finite for 6
    steps and is non-finite at the 7th, as the reference is. All 12 fields:
    the FMA-free build bit for bit after 5 steps; the FP64 path within 1e-11
    after 2 steps (the growing mode amplifies FMA rounding differences after
    that)."""
    s = config1(vg)
    for name, v in dict(advection=2, weno_scalars=0, weno_advective=0, pgf_perturbation=0, split_fast=0).items():
        setattr(s, name, v)
    t = oc.Setup()
    for name, _ in oc.Setup._fields_:
        setattr(t, name, getattr(s, name))
    o = oc.Model(t, "port")
    for _ in range(2):
        assert o.rk3_step(2.0, 6) == 0
    ref2 = [o.get(q) for q in range(12)]
    for _ in range(3):
        assert o.rk3_step(2.0, 6) == 0
    ref = [o.get(q) for q in range(12)]
    with vg.Model(s, vg.FP64_EXACT) as m:
        m.step(2.0, 6, 5)
        for q, a in enumerate(m.state()):
            assert np.array_equal(vg.interior(s, q, a), vg.interior(s, q, ref[q])), vg.SPECIES[q]
    with vg.Model(s, vg.FP64) as m:
        m.step(2.0, 6, 2)
        got = m.state()
        for q in range(12):
            r = vg.interior(s, q, ref2[q])
            scale = max(float(np.abs(r).max()), 1e-300)
            assert np.abs(vg.interior(s, q, got[q]) - r).max() <= 1e-11 * scale, vg.SPECIES[q]
