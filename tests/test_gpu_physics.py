"""Physics coupling (vibe_gb300_set_physics; RungeKutta3Integrator::
slow_tendency, runge_kutta.cpp:46-63) with the built-in Kessler warm-rain
package, against the oracle's restatement (KesslerMicrophysics::step_column,
pinned bit for bit to the compiled reference on the CPU, through
state_to_column and the microphysics step of PhysicsDriver)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# tendencies: device pow/exp differ from the host libm by an ulp or two, and
# the saturation adjustment's Newton stops on a residual test, so FP64 agrees
# to ~1e-12 of each field's scale; the mixed path computes in FP32
TOL_TEND64, TOL_TEND32 = 1e-9, 2e-4
TOL_STEP64, TOL_STEP32 = 1e-9, 2e-4
FIELDS = {4: "theta", 6: "qv", 7: "qc", 8: "qr"}


def setup(vg, **kw):
    base = dict(nx=20, ny=16, nz=14, dx=250.0, dy=250.0, z_top=3500.0, zeta_first=1.0, zeta_stretch=1.06,
                bubble_xc=2500.0, bubble_yc=2000.0, bubble_zc=1000.0, bubble_radius_x=1500.0,
                bubble_radius_z=1000.0, u_background=5.0, shear_u=0.001, moist=1, qv_surface=0.018,
                qv_decay_height=2500.0, ref_kind=1, acoustic_mode=2, terrain_kind=1, hill_h=200.0, hill_a=1000.0,
                hill_xc=2500.0, hill_yc=2000.0)
    base.update(kw)
    return vg.Setup.defaults(**base)


def oracle_setup(oc, s):
    t = oc.Setup()
    for name, _ in oc.Setup._fields_:
        setattr(t, name, getattr(s, name))
    return t


def with_clouds(vg, s, state):
    """qc in a blob above the bubble, rain in a shaft beside it, and a
    supersaturated blob of vapour (qv x 1.6) low down (seeded)."""
    rng = np.random.default_rng(7)
    st = [a.copy() for a in state]
    k, j, i = np.meshgrid(np.arange(s.nz), np.arange(s.ny), np.arange(s.nx), indexing="ij")
    qv = vg.interior(s, 6, st[6])
    qv[...] *= 1.0 + 0.6 * np.exp(-(((i - 5) / 3.0) ** 2 + ((j - 10) / 3.0) ** 2 + ((k - 3) / 2.0) ** 2))
    for sp, amp, (ci, cj, ck) in ((7, 2.5e-3, (8, 8, 6)), (8, 3e-3, (13, 6, 9))):
        a = vg.interior(s, sp, st[sp])
        k, j, i = np.meshgrid(np.arange(s.nz), np.arange(s.ny), np.arange(s.nx), indexing="ij")
        r2 = ((i - ci) / 4.0) ** 2 + ((j - cj) / 4.0) ** 2 + ((k - ck) / 3.0) ** 2
        a[...] = amp * np.exp(-r2) * (1.0 + 0.1 * rng.standard_normal(a.shape))
    return st


def kessler(vg, oc, offset):
    return vg.Kessler.defaults(exner_offset=offset), oc.Kessler.defaults(exner_offset=offset)


def close(vg, s, got, ref, tol, what):
    for sp, name in FIELDS.items():
        g, r = vg.interior(s, sp, got[sp]), vg.interior(s, sp, ref[sp])
        scale = max(np.abs(r).max(), 1e-30)
        err = np.abs(g - r).max() / scale
        assert err <= tol, (what, name, err)


@pytest.mark.parametrize("offset", [0, 1])
@pytest.mark.parametrize("prec", ["FP64", "MIXED"])
def test_kessler_tendency_matches_oracle(vg, oc, prec, offset):
    """The package's PhysicsTendency for a cloudy, raining state: FP64 to
    1e-9, mixed (FP32 arithmetic) to 2e-4 of each field's scale; offset 0
    condenses (realistic column pressure), offset 1 is the reference's
    state_to_column (pressure from pi0 + pi)."""
    s = setup(vg, **({} if prec == "FP64" else dict(terrain_kind=0, ref_kind=0)))
    kg, ko = kessler(vg, oc, offset)
    with vg.Model(s, getattr(vg, prec)) as m:
        o = oc.Model(oracle_setup(oc, s), "port")
        st = with_clouds(vg, s, m.state())
        m.set_state(st)
        o.set_state(st)
        m.set_physics_kessler(kg)
        got = m.physics_tendency(6.0)
        ref = dict(zip((4, 6, 7, 8), oc.kessler_tendency(o, ko, 6.0)))
        close(vg, s, got, ref, TOL_TEND64 if prec == "FP64" else TOL_TEND32, "tendency")
        for sp in (0, 1, 9, 10, 11):  # u, v and the ice species: untouched by the scheme
            assert not np.any(got[sp])
        assert np.abs(vg.interior(s, 8, got[8])).max() > 0.0  # rain falls
        if offset == 0:
            assert vg.interior(s, 7, got[7]).max() > 0.0  # condensation somewhere


@pytest.mark.parametrize("prec", ["FP64", "MIXED"])
def test_rk3_steps_with_kessler_match_oracle(vg, oc, prec):
    """Two RK3 steps with the package coupled at every stage against the
    oracle's vo_rk3_step with the same coupling."""
    s = setup(vg, **({} if prec == "FP64" else dict(terrain_kind=0, ref_kind=0)))
    kg, ko = kessler(vg, oc, 0)
    with vg.Model(s, getattr(vg, prec)) as m:
        o = oc.Model(oracle_setup(oc, s), "port")
        st = with_clouds(vg, s, m.state())
        m.set_state(st)
        o.set_state(st)
        m.set_physics_kessler(kg)
        oc.set_physics_kessler(o, ko)
        m.step(2.0, 4, 2)
        assert o.rk3_step(2.0, 4) == 0 and o.rk3_step(2.0, 4) == 0
        got, ref = m.state(), o.state()
        tol = TOL_STEP64 if prec == "FP64" else TOL_STEP32
        for sp in (0, 1, 2, 3, 4, 5, 6, 7, 8):
            g, r = vg.interior(s, sp, got[sp]), vg.interior(s, sp, ref[sp])
            if sp in (4, 5, 3):  # compare the departures from the state's mean for the large fields
                r0 = np.mean(r)
                g, r = g - r0, r - r0
            scale = max(np.abs(r).max(), 1e-30)
            assert np.abs(g - r).max() <= tol * scale, (vg.SPECIES[sp], np.abs(g - r).max() / scale)


def test_physics_in_graph_replay_and_removal(vg):
    """Graph replay of steps with physics gives the eager steps' bits; with
    the package removed the step is the plain step again."""
    s = setup(vg, terrain_kind=0, ref_kind=0)
    kg = vg.Kessler.defaults(exner_offset=0)
    with vg.Model(s, vg.MIXED) as a, vg.Model(s, vg.MIXED) as b, vg.Model(s, vg.MIXED) as c:
        st = with_clouds(vg, s, a.state())
        for m in (a, b, c):
            m.set_state(st)
        a.set_physics_kessler(kg)
        b.set_physics_kessler(kg)
        b.set_graph(0)
        a.step(2.0, 4, 3)
        b.step(2.0, 4, 3)
        for x, y in zip(a.state(), b.state()):
            assert np.array_equal(x, y)
        a.set_physics_kessler(None)
        a.set_state(st)
        a.step(2.0, 4, 2)
        c.step(2.0, 4, 2)
        for x, y in zip(a.state(), c.state()):
            assert np.array_equal(x, y)


def test_kessler_needs_moisture(vg):
    s = setup(vg, moist=0)
    with vg.Model(s, vg.FP64) as m:
        m.set_physics_kessler(vg.Kessler.defaults())
        with pytest.raises(vg.VibeError):
            m.step(2.0, 4, 1)


def test_groups_refuse_models_with_physics(vg):
    """The work-list launches of a group have no physics call: a member with a
    package installed is refused rather than stepped without it."""
    s = setup(vg, terrain_kind=0, ref_kind=0)
    with vg.Model(s, vg.MIXED) as a, vg.Model(s, vg.MIXED) as b:
        a.set_physics_kessler(vg.Kessler.defaults())
        with pytest.raises(vg.VibeError):
            vg.Group([a, b])
        a.set_physics_kessler(None)
        with vg.Group([a, b]) as g:
            g.step(2.0, 4, 1)


def test_fp64_physics_graph_replay_and_errors(vg):
    """FP64 model: graph replay with the package equals eager steps bit for
    bit; asking for a tendency without a package is an error."""
    s = setup(vg)
    kg = vg.Kessler.defaults(exner_offset=0)
    with vg.Model(s, vg.FP64) as a, vg.Model(s, vg.FP64) as b:
        with pytest.raises(vg.VibeError):
            a.physics_tendency(1.0)
        st = with_clouds(vg, s, a.state())
        a.set_state(st)
        b.set_state(st)
        a.set_physics_kessler(kg)
        b.set_physics_kessler(kg)
        b.set_graph(0)
        a.step(2.0, 4, 3)
        b.step(2.0, 4, 3)
        for x, y in zip(a.state(), b.state()):
            assert np.array_equal(x, y)
