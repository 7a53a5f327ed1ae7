"""Groups (vibe_gb300_group_*): several mixed models of different sizes
advanced with one launch per kernel for all of them give the bits of the same
models stepped one by one."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


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
            assert g.launches_per_step() == 3 * (1 + 6 + 1) + 1
            g.step(2.0, 6, 2)
        for m in single:
            m.step(2.0, 6, 5)
        for a, b in zip(grouped, single):
            for sp in range(7):
                assert np.array_equal(a.get(sp), b.get(sp)), vg.SPECIES[sp]
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
