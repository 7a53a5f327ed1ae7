"""Groups (vibe_gb300_group_*): several mixed models of different sizes
advanced with one launch per kernel for all of them match the same models
stepped one by one. The work-list kernels run the single-domain kernel bodies
compiled in another kernel, whose FMA contraction may differ: the bound is
FP32 rounding, 1e-6 of each field's scale (velocities: the common velocity
scale) after five steps."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL_GROUP = 1e-6


def assert_rounding_close(vg, s, got, ref, tol=TOL_GROUP, what=""):
    """got, ref: lists of 7 FieldT arrays (u v w rho theta pi qv)."""
    ins = [vg.interior(s, q, ref[q]) for q in range(7)]
    vs = max(float(np.abs(ins[q]).max()) for q in range(3))
    for q in range(7):
        scale = vs if q < 3 else float(np.abs(ins[q]).max())
        err = float(np.abs(vg.interior(s, q, got[q]) - ins[q]).max())
        assert err <= tol * max(scale, 1e-30) or err == 0.0, (what, vg.SPECIES[q], err, scale)


def member(vg, nx, ny, seed):
    s = vg.Setup.defaults(nx=nx, ny=ny, nz=14, dx=500.0, dy=500.0, z_top=6000.0, zeta_first=1.0,
                          zeta_stretch=1.05, ref_kind=1, acoustic_mode=2, u_background=8.0, shear_u=0.001,
                          bubble_xc=nx * 250.0, bubble_yc=ny * 250.0, bubble_zc=1500.0, bubble_radius_x=2000.0,
                          bubble_radius_z=1000.0, bubble_amplitude=1.0 + 0.3 * seed, qv_surface=0.0)
    return s


@pytest.mark.parametrize("sizes", [[(40, 24), (17, 33), (64, 8)], [(33, 33)]])
def test_group_step_equals_individual_steps(vg, sizes):
    setups = [member(vg, nx, ny, q) for q, (nx, ny) in enumerate(sizes)]
    grouped = [vg.Model(s, vg.MIXED) for s in setups]
    single = [vg.Model(s, vg.MIXED) for s in setups]
    try:
        with vg.Group(grouped) as g:
            g.step(2.0, 6, 3)
            # per stage 1 stage + 6 column launches; after stages 1 and 2 the
            # fix-up of the deferred column kernel (u/v update, w/rho'
            # corrections); stage 3's is in the finish
            assert g.launches_per_step() == 3 * (1 + 6) + 2 + 1
            g.step(2.0, 6, 2)
        for m in single:
            m.step(2.0, 6, 5)
        for a, b, s in zip(grouped, single, setups):
            assert_rounding_close(vg, s, [a.get(sp) for sp in range(7)], [b.get(sp) for sp in range(7)],
                                  what="group vs single")
    finally:
        for m in grouped + single:
            m.close()


def test_group_rejects_unsupported_members(vg):
    s = member(vg, 16, 16, 0)
    t = vg.Setup.defaults(nx=16, ny=16, nz=14, acoustic_mode=0)
    with vg.Model(s, vg.MIXED) as a, vg.Model(t, vg.MIXED) as b, vg.Model(s, vg.FP64) as c:
        for bad in ([a, b], [a, c]):
            with pytest.raises(vg.VibeError):
                vg.Group(bad)


def test_group_after_members_reconfigured_for_another_dt(vg):
    """A member stepped alone with another dt, and a member's FP32 HEVI
    tangent-linear (which builds its column factors for 3*dtau), rewrite
    that member's per-model dt tables in place; the group's next step must
    put them back for its own dt, or its cached graph replays with the
    wrong HEVI factors and sponge weights."""
    setups = [member(vg, 40, 24, 0), member(vg, 17, 33, 1)]
    grouped = [vg.Model(s, vg.MIXED) for s in setups]
    single = [vg.Model(s, vg.MIXED) for s in setups]
    try:
        pert = [np.random.default_rng(3).standard_normal(grouped[1].size(sp)) for sp in (0, 1, 2, 3, 5)]
        with vg.Group(grouped) as g:
            g.step(2.0, 6, 2)
            grouped[0].step(1.0, 6, 2)       # stepped alone with another dt (parity kept)
            grouped[1].hevi_tl_f32(0.7, 2, pert)
            g.step(2.0, 6, 2)
        single[0].step(2.0, 6, 2)
        single[0].step(1.0, 6, 2)
        single[0].step(2.0, 6, 2)
        single[1].step(2.0, 6, 4)
        for a, b, s in zip(grouped, single, setups):
            assert_rounding_close(vg, s, [a.get(sp) for sp in range(7)], [b.get(sp) for sp in range(7)],
                                  what="group after reconfiguration vs single")
    finally:
        for m in grouped + single:
            m.close()
