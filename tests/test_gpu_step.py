"""GPU parity of the dynamics step against the CPU oracle (oracle/vibe_oracle.c,
itself pinned bit for bit to the reference compiled unchanged).

Error measure: max |gpu - oracle| over the compared points divided by the
field's magnitude scale -- max |value| for rho, theta, pi, q; for u, v, w the
common velocity scale max(|u|, |v|, |w|) (v and w start at zero, so their own
maxima say nothing about precision).
Tolerances:
  FP64_EXACT GPU path  bit-exact (no FMA contraction, reference operation order)
  FP64 GPU path        <= 1e-12 per substep kernel and per step of the stable
                       composition; <= 1e-11 per step of the reference's
                       total-Exner compositions, where w and v are driven by
                       differences of pi ~1e-3 of pi and FMA contraction alone
                       moves the result by a few 1e-12
  mixed GPU path       <= 1e-5  per step
Integer/index work (the set-up on the host) must be bit-exact.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOLMX = 1e-5
# Tendencies are differences of totals (theta ~ 300 K through up to 7-point
# stencils): the reference's own rounding there is ~1e-13 of the result, so
# kernel-level tendency checks use 1e-10, normalised by max(|R|, 1e-3/s *
# max|field|) so that fields whose exact tendency is zero (uniform qv, w = 0)
# compare rounding noise against a physical scale, not against itself.
TOL_TEND = 1e-10


def small_setup(vg, **kw):
    base = dict(nx=20, ny=16, nz=12, dx=250.0, dy=250.0, z_top=3000.0, zeta_first=1.0, zeta_stretch=1.08,
                bubble_xc=2500.0, bubble_yc=2000.0, bubble_zc=1000.0, bubble_radius_x=1500.0,
                bubble_radius_z=1000.0, u_background=5.0, shear_u=0.001)
    base.update(kw)
    return vg.Setup.defaults(**base)


def oracle_setup(oc, s):
    t = oc.Setup()
    for name, _ in oc.Setup._fields_:
        setattr(t, name, getattr(s, name))
    return t


def rel_err(vg, s, sp, got, ref, floor=0.0):
    g = vg.interior(s, sp, got)
    r = vg.interior(s, sp, ref)
    scale = max(np.abs(r).max(), floor)
    if scale == 0.0:
        return float(np.abs(g).max())
    return float(np.abs(g - r).max() / scale)


def velocity_scale(vg, s, ref):
    return max(float(np.abs(vg.interior(s, sp, ref[sp])).max()) for sp in (0, 1, 2) if sp < len(ref))


def assert_state_close(vg, s, got, ref, tol, species=range(7), what="", floors=None, velocity=True):
    floors = dict(floors or {})
    if velocity and len(ref) >= 3:
        vs = velocity_scale(vg, s, ref)
        for sp in (0, 1, 2):
            floors.setdefault(sp, vs)
    errs = {vg.SPECIES[sp]: rel_err(vg, s, sp, got[sp], ref[sp], floors.get(sp, 0.0)) for sp in species}
    bad = {k: v for k, v in errs.items() if not v <= tol}
    assert not bad, "%s: relative error above %g: %s (all: %s)" % (what, tol, bad, errs)
    return errs


SCHEMES = [
    dict(advection=2, weno_scalars=0, pgf_perturbation=0, split_fast=0, weno_advective=0),
    dict(advection=4, weno_scalars=0, pgf_perturbation=0, split_fast=0, coriolis=1),
    dict(advection=6, weno_scalars=0, pgf_perturbation=1, split_fast=1, coriolis=2, moist=1, qv_surface=0.01),
    dict(advection=5, weno_scalars=1, pgf_perturbation=0, split_fast=0, weno_advective=0, ref_kind=1),
    dict(advection=5, weno_scalars=1, pgf_perturbation=1, split_fast=1, weno_advective=1,
         divergence_damping=50.0, divergence_order=4),
    dict(advection=2, weno_scalars=0, divergence_damping=50.0, divergence_order=2, moist=1),
]


def test_setup_bit_exact(vg, oc):
    s = small_setup(vg, ref_kind=1)
    with vg.Model(s, vg.FP64) as m:
        o = oc.Model(oracle_setup(oc, s), "port")
        for sp in range(12):
            assert np.array_equal(m.get(sp), o.get(sp)), vg.SPECIES[sp]
        for r in range(5):
            assert np.array_equal(m.reffield(r), o.reffield(r))
        assert np.array_equal(m.zeta(), o.zeta())
        assert np.array_equal(m.sponge_profile(), o.sponge_profile())


@pytest.mark.parametrize("scheme", range(len(SCHEMES)))
def test_slow_tendency_fp64(vg, oc, scheme):
    s = small_setup(vg, **SCHEMES[scheme])
    with vg.Model(s, vg.FP64) as m:
        o = oc.Model(oracle_setup(oc, s), "port")
        floors = {sp: 1e-3 * np.abs(vg.interior(s, sp, o.get(sp))).max() for sp in range(12)}
        vs = 1e-3 * velocity_scale(vg, s, o.state())
        for sp in (0, 1, 2):
            floors[sp] = max(floors[sp], vs)
        assert_state_close(vg, s, m.slow_tendency(), o.slow_tendency(), TOL_TEND, range(12), "slow tendency",
                           floors, velocity=False)


@pytest.mark.parametrize("scheme", range(len(SCHEMES)))
def test_slow_tendency_fp64_exact(vg, oc, scheme):
    s = small_setup(vg, **SCHEMES[scheme])
    with vg.Model(s, vg.FP64_EXACT) as m:
        o = oc.Model(oracle_setup(oc, s), "port")
        for sp, (a, b) in enumerate(zip(m.slow_tendency(), o.slow_tendency())):
            assert np.array_equal(vg.interior(s, sp, a), vg.interior(s, sp, b)), vg.SPECIES[sp]


MIXED_SCHEMES = [
    dict(),
    dict(advection=2, weno_scalars=0),
    dict(advection=4, weno_scalars=0, coriolis=1),
    dict(advection=6, weno_scalars=0, coriolis=2, moist=1, qv_surface=0.01),
    dict(weno_advective=0, ref_kind=1, divergence_damping=50.0, divergence_order=2),
    dict(moist=1, qv_surface=0.01, ref_kind=1, nz=26, z_top=6000.0, shear_u=0.004),
]


def assert_levels_close(vg, s, got, ref, tol, species, what, floors):
    """Error of every level relative to that level's largest value (or the
    species' floor): a wrong term confined to one level, e.g. the top or
    bottom boundary, cannot hide behind a larger tendency elsewhere."""
    for sp in species:
        g = vg.interior(s, sp, got[sp])
        r = vg.interior(s, sp, ref[sp])
        for k in range(r.shape[0]):
            scale = max(float(np.abs(r[k]).max()), floors[sp])
            err = float(np.abs(g[k] - r[k]).max())
            assert err <= tol * scale or (scale == 0.0 and err == 0.0), \
                "%s: %s level %d error %.3e scale %.3e" % (what, vg.SPECIES[sp], k, err, scale)


@pytest.mark.parametrize("scheme", range(len(MIXED_SCHEMES)))
@pytest.mark.parametrize("levels", ["", "3"])
def test_slow_tendency_mixed(vg, oc, scheme, levels, monkeypatch):
    """Mixed-path slow tendency (FP32) against the oracle, level by level.
    levels = "3" makes the stage kernel's blocks march 3 levels each, so the
    chunk starts (fresh column registers and vertical fluxes) are exercised."""
    monkeypatch.setenv("VIBE_GB300_STAGE_LEVELS", levels)
    s = small_setup(vg, **MIXED_SCHEMES[scheme])
    n = 12 if s.moist else 7
    with vg.Model(s, vg.MIXED) as m:
        o = oc.Model(oracle_setup(oc, s), "port")
        ref = o.slow_tendency()
        floors = {sp: 1e-3 * np.abs(vg.interior(s, sp, o.get(sp))).max() for sp in range(n)}
        vs = 1e-3 * velocity_scale(vg, s, o.state())
        for sp in (0, 1, 2):
            floors[sp] = max(floors[sp], vs)
        got = m.slow_tendency()
        assert_state_close(vg, s, got, ref, TOLMX, range(n), "mixed slow tendency", floors, velocity=False)
        lf = {sp: 1e-2 * floors[sp] for sp in range(n)}
        assert_levels_close(vg, s, got, ref, 1e-4, range(n), "mixed slow tendency per level", lf)


@pytest.mark.parametrize("pgf", [0, 1])
def test_acoustic_substep_fp64(vg, oc, pgf):
    s = small_setup(vg, pgf_perturbation=pgf)
    with vg.Model(s, vg.FP64) as m:
        o = oc.Model(oracle_setup(oc, s), "port")
        for _ in range(3):
            m.acoustic_substep(0.3)
            o.acoustic_substep(0.3)
        assert_state_close(vg, s, m.state(), o.state(), TOL64, range(7), "FB substep")


def test_reference_hevi_substep_fp64(vg, oc):
    s = small_setup(vg, acoustic_mode=1, pgf_perturbation=0)
    with vg.Model(s, vg.FP64) as m:
        o = oc.Model(oracle_setup(oc, s), "port")
        for _ in range(2):
            m.hevi_substep(0.7)
            o.hevi_substep(0.7)
        assert_state_close(vg, s, m.state(), o.state(), TOL64, range(7), "reference HEVI substep")


@pytest.mark.parametrize("beta", [0.5, 0.6])
def test_consistent_hevi_substep_fp64(vg, oc, beta):
    s = small_setup(vg, acoustic_mode=2, hevi_beta=beta)
    with vg.Model(s, vg.FP64) as m:
        o = oc.Model(oracle_setup(oc, s), "port")
        for _ in range(3):
            m.hevi_substep(1.0)
            o.hevi_substep(1.0)
        assert_state_close(vg, s, m.state(), o.state(), TOL64, range(7), "consistent HEVI substep")


def test_sponge_fp64(vg, oc):
    s = small_setup(vg, sponge_alpha=0.3, sponge_start_fraction=0.5)
    with vg.Model(s, vg.FP64) as m:
        o = oc.Model(oracle_setup(oc, s), "port")
        m.sponge(6.0)
        o.sponge(6.0)
        assert_state_close(vg, s, m.state(), o.state(), TOL64, range(7), "sponge")


STEP_CASES = [
    dict(pgf_perturbation=0, split_fast=0, weno_scalars=0, advection=2, weno_advective=0),  # reference composition
    dict(pgf_perturbation=0, split_fast=0, weno_scalars=1, advection=5, weno_advective=0),  # O-WENO
    dict(),                                                                                  # stable, FB
    dict(acoustic_mode=2, ref_kind=1),                                                        # stable, HEVI
    dict(acoustic_mode=1, pgf_perturbation=0, split_fast=0),                                  # O-HEVI
    dict(acoustic_mode=2, ref_kind=1, w_rigid=1, hevi_beta=0.6),                              # rigid ground/lid
]


@pytest.mark.parametrize("case", range(len(STEP_CASES)))
def test_rk3_step_fp64(vg, oc, case):
    s = small_setup(vg, **STEP_CASES[case])
    tol = TOL64 if s.pgf_perturbation else 1e-11
    with vg.Model(s, vg.FP64) as m:
        o = oc.Model(oracle_setup(oc, s), "port")
        m.step(2.0, 4, 1)
        assert o.rk3_step(2.0, 4) == 0
        assert_state_close(vg, s, m.state(), o.state(), tol, range(12), "rk3 step")


@pytest.mark.parametrize("case", range(len(STEP_CASES)))
def test_rk3_step_fp64_exact(vg, oc, case):
    """Without FMA contraction the FP64 path reproduces the reference's bits."""
    s = small_setup(vg, **STEP_CASES[case])
    nsteps = 2 if s.pgf_perturbation else 1  # the reference compositions diverge within a few steps
    with vg.Model(s, vg.FP64_EXACT) as m:
        o = oc.Model(oracle_setup(oc, s), "port")
        m.step(2.0, 4, nsteps)
        for _ in range(nsteps):
            assert o.rk3_step(2.0, 4) == 0
        for sp in range(12):
            assert np.array_equal(vg.interior(s, sp, m.get(sp)), vg.interior(s, sp, o.get(sp))), vg.SPECIES[sp]


@pytest.mark.parametrize("case", [2, 3, 5])
def test_rk3_step_mixed(vg, oc, case):
    s = small_setup(vg, **STEP_CASES[case])
    with vg.Model(s, vg.MIXED) as m:
        o = oc.Model(oracle_setup(oc, s), "port")
        m.step(2.0, 4, 1)
        assert o.rk3_step(2.0, 4) == 0
        assert_state_close(vg, s, m.state(), o.state(), TOLMX, range(7), "mixed rk3 step")


def test_mixed_many_steps_track_fp64(vg):
    """Mixed vs FP64 GPU over 10 steps of a HEVI case (error growth bound)."""
    s = small_setup(vg, acoustic_mode=2, ref_kind=1, nx=24, ny=24, nz=20, dx=1000.0, dy=1000.0, z_top=10000.0,
                    bubble_xc=12000.0, bubble_yc=12000.0, bubble_zc=3000.0, bubble_radius_x=4000.0,
                    bubble_radius_z=2000.0, bubble_amplitude=3.0, u_background=10.0, shear_u=0.0)
    with vg.Model(s, vg.FP64) as a, vg.Model(s, vg.MIXED) as b:
        a.step(6.0, 6, 10)
        b.step(6.0, 6, 10)
        errs = assert_state_close(vg, s, b.state(), a.state(), 1e-4, range(7), "10 mixed steps")
        print("mixed vs fp64 after 10 steps:", errs)


@pytest.mark.parametrize("dims", [(13, 7, 5), (9, 11, 3), (5, 4, 2), (1, 6, 4)])
def test_ragged_and_tiny_grids(vg, oc, dims):
    nx, ny, nz = dims
    s = small_setup(vg, nx=nx, ny=ny, nz=nz, bubble_xc=nx * 125.0, bubble_yc=ny * 125.0, bubble_zc=500.0)
    for prec, tol, case in ((vg.FP64, TOL64, 2), (vg.FP64, TOL64, 0), (vg.MIXED, TOLMX, 2)):
        t = small_setup(vg, nx=nx, ny=ny, nz=nz, bubble_xc=nx * 125.0, bubble_yc=ny * 125.0, bubble_zc=500.0,
                        **STEP_CASES[case])
        with vg.Model(t, prec) as m:
            o = oc.Model(oracle_setup(oc, t), "port")
            m.step(1.0, 2, 1)
            assert o.rk3_step(1.0, 2) == 0
            assert_state_close(vg, t, m.state(), o.state(), tol, range(7), "grid %s prec %d" % (dims, prec))


def test_halo_ghost_line_is_read(vg, oc):
    """The reference reads rho at i = nx and j = ny without a clamp
    (equations.cpp:120-123); a non-zero halo there must change the result
    the same way on both sides."""
    s = small_setup(vg, **STEP_CASES[0])
    with vg.Model(s, vg.FP64) as m:
        o = oc.Model(oracle_setup(oc, s), "port")
        rho = o.get(3)
        a = rho.reshape(vg.storage_shape(s, 3))
        a[4:4 + s.nz, 4:4 + s.ny, 4 + s.nx] = 1.1    # east ghost column
        a[4:4 + s.nz, 4 + s.ny, 4:4 + s.nx] = 0.9    # north ghost row
        o.set(3, a)
        m.set(3, a)
        assert_state_close(vg, s, m.slow_tendency(), o.slow_tendency(), TOL_TEND, [3], "ghost line")


def test_nonfinite_state_is_reported(vg):
    s = small_setup(vg)
    for prec in (vg.FP64, vg.MIXED):
        with vg.Model(s, prec) as m:
            th = m.get(4)
            th.reshape(vg.storage_shape(s, 4))[6, 6, 6] = np.nan
            m.set(4, th)
            with pytest.raises(vg.VibeError) as e:
                m.step(2.0, 4, 1)
            assert e.value.code == -3
            # the model stays usable after the error
            m.set(4, np.nan_to_num(th, nan=300.0))


def test_mixed_rejects_unsupported_setups(vg):
    with pytest.raises(vg.VibeError) as e:
        vg.Model(small_setup(vg, terrain_kind=1, hill_h=300.0, hill_a=1000.0, hill_xc=2500.0, hill_yc=2000.0),
                 vg.MIXED)
    assert e.value.code == -5
    with pytest.raises(vg.VibeError):
        vg.Model(small_setup(vg, split_fast=0), vg.MIXED)


def test_terrain_fp64_step(vg, oc):
    s = small_setup(vg, terrain_kind=1, hill_h=300.0, hill_a=1000.0, hill_xc=2500.0, hill_yc=2000.0,
                    acoustic_mode=2, ref_kind=1)
    with vg.Model(s, vg.FP64) as m:
        o = oc.Model(oracle_setup(oc, s), "port")
        assert np.array_equal(m.terrain(), o.terrain())
        m.step(2.0, 3, 1)
        assert o.rk3_step(2.0, 3) == 0
        assert_state_close(vg, s, m.state(), o.state(), TOL64, range(7), "terrain step")


def test_mixed_graph_replay_is_bitwise_identical(vg):
    """The CUDA-graph replay of the mixed step gives the eager launches' bits."""
    s = small_setup(vg, acoustic_mode=2, ref_kind=1)
    with vg.Model(s, vg.MIXED) as a, vg.Model(s, vg.MIXED) as b:
        b.set_graph(False)
        a.step(2.0, 6, 5)
        b.step(2.0, 6, 5)
        a.step(2.0, 6, 2)  # same dt: graphs reused
        b.step(2.0, 6, 2)
        a.step(1.0, 4, 3)  # new dt: eager step, new graphs
        b.step(1.0, 4, 3)
        for sp in range(7):
            assert np.array_equal(a.get(sp), b.get(sp)), vg.SPECIES[sp]


@pytest.mark.parametrize("prec", ["FP64", "MIXED"])
def test_cfl_diagnostics_bit_exact(vg, oc, prec):
    """cfl_number / max_sound_speed / acoustic_cfl / max_stable_dt of the
    device state equal the oracle's serial loops bit for bit (maxima)."""
    s = small_setup(vg, **STEP_CASES[0]) if prec == "FP64" else small_setup(vg)
    with vg.Model(s, getattr(vg, prec)) as m:
        o = oc.Model(oracle_setup(oc, s), "port")
        o.set_state(m.state())  # same state on both sides
        assert m.cfl(2.0, 0.3) == oc.cfl(o, 2.0, 0.3)
        assert m.max_stable_dt() == oc.max_stable_dt(o)


def test_snapshot_restart_is_bitwise(vg):
    """A run restarted from the device snapshot repeats itself bit for bit."""
    s = small_setup(vg, acoustic_mode=2, ref_kind=1, pgf_perturbation=1, split_fast=1)
    for prec in (vg.MIXED, vg.FP64):
        with vg.Model(s, prec) as m:
            m.save_snapshot()
            m.step(2.0, 4, 3)
            first = m.state()
            m.restore_snapshot()
            m.step(2.0, 4, 3)
            for sp, (a, b) in enumerate(zip(first, m.state())):
                assert np.array_equal(a, b), vg.SPECIES[sp]
        with vg.Model(s, prec) as m, pytest.raises(vg.VibeError):
            m.restore_snapshot()


def test_rigid_ground_and_lid(vg):
    """w_rigid: w is zero on the k = 0 and k = nz faces after every step (the
    reference moves them: a bubble touching the ground pushes mass through it)."""
    for prec in (vg.FP64, vg.MIXED):
        for rigid in (0, 1):
            s = small_setup(vg, acoustic_mode=2, ref_kind=1, w_rigid=rigid, bubble_zc=300.0)
            with vg.Model(s, prec) as m:
                m.step(2.0, 4, 2)
                w = vg.interior(s, 2, m.get(2))
                edge = max(np.abs(w[0]).max(), np.abs(w[-1]).max())
                assert (edge == 0.0) == bool(rigid), (prec, rigid, edge)


@pytest.mark.parametrize("column", [-1, 4])
@pytest.mark.parametrize("dims", [(13, 7, 5), (9, 11, 3), (1, 6, 4), (2, 3, 6), (67, 9, 7)])
def test_mixed_hevi_ragged_grids(vg, oc, dims, column):
    """The HEVI column kernels (built-in and TMA-fed) on odd and tiny
    horizontal sizes (a thread's second column falls on the ghost line when nx
    is odd; 67 columns leave a second block with three)."""
    nx, ny, nz = dims
    t = small_setup(vg, nx=nx, ny=ny, nz=nz, bubble_xc=nx * 125.0, bubble_yc=ny * 125.0, bubble_zc=500.0,
                    **STEP_CASES[3])
    with vg.Model(t, vg.MIXED) as m:
        m.set_tuning(column_kernel=column)
        try:
            o = oc.Model(oracle_setup(oc, t), "port")
            m.step(1.0, 3, 2)
            assert o.rk3_step(1.0, 3) == 0 and o.rk3_step(1.0, 3) == 0
            assert_state_close(vg, t, m.state(), o.state(), 2 * TOLMX, range(7), "mixed HEVI grid %s" % (dims,))
        finally:
            m.set_tuning()


def test_column_kernel_variants_agree(vg):
    """Every HEVI column kernel variant computes the built-in one's update to
    FP32 rounding (1e-6 of each field's scale) over 3 steps."""
    s = small_setup(vg, acoustic_mode=2, ref_kind=1, nx=45, ny=22, nz=24)
    with vg.Model(s, vg.MIXED) as m:
        m.save_snapshot()
        m.step(2.0, 4, 3)
        ref = m.state()
        try:
            for column in range(5):
                m.restore_snapshot()
                m.set_tuning(column_kernel=column)
                m.step(2.0, 4, 3)
                assert_state_close(vg, s, m.state(), ref, 1e-6, range(7), "column kernel %d" % column)
        finally:
            m.set_tuning()


def test_autotune_keeps_the_update(vg):
    """The autotuner only chooses among launch shapes of the same update: a run
    after tuning matches the run before it to FP32 rounding (1e-6 of each
    field's scale), and tuning leaves the model's state as it was."""
    s = small_setup(vg, acoustic_mode=2, ref_kind=1, nx=45, ny=22, nz=24)
    with vg.Model(s, vg.MIXED) as a:
        a.save_snapshot()
        a.step(2.0, 4, 3)
        before = a.state()
        a.restore_snapshot()
        t = a.autotune(2.0, 4)
        assert t["column_kernel"] in (-1, 0, 1, 2, 3, 4) and 1 <= t["stage_levels"] <= s.nz
        assert t["ms_per_step"] > 0.0 and t["ms_per_step"] <= t["default_ms_per_step"] and t["candidates"] >= 5
        a.step(2.0, 4, 3)
        assert_state_close(vg, s, a.state(), before, 1e-6, range(7), "tuned vs built-in launch shapes")
        a.set_tuning()
        # tuning leaves the state parity too: a fresh model joins it in a group
        a.restore_snapshot()
        a.autotune(2.0, 4)
        a.set_tuning()
        with vg.Model(s, vg.MIXED) as b, vg.Group([a, b]) as g:
            g.step(2.0, 4, 1)


def test_step_io_pipeline_matches_synchronous_steps(vg):
    """vibe_gb300_step_io: five pipelined calls (inputs A, B, A, C, B; the
    staging buffers are reused every other call) give the bits of the same
    steps done one at a time with set_state / step / get_state; a species
    passed as NULL is neither uploaded nor read back."""
    torch = pytest.importorskip("torch")
    s = small_setup(vg, acoustic_mode=2, ref_kind=1)
    with vg.Model(s, vg.MIXED) as m, vg.Model(s, vg.MIXED) as ref:
        base = m.state()
        rng = np.random.default_rng(4)
        inputs = []
        for _ in range(3):
            st = [a.copy() for a in base[:7]]
            th = st[4]
            th += 0.2 * rng.standard_normal(th.size) * (th != 0.0)
            inputs.append([torch.from_numpy(a).pin_memory() for a in st])
        order = [0, 1, 0, 2, 1]
        outs = [[torch.zeros(m.size(q), dtype=torch.float64).pin_memory() for q in range(7)] for _ in order]
        for n, which in enumerate(order):
            in_ptrs = [t.data_ptr() for t in inputs[which]]
            out_ptrs = [t.data_ptr() for t in outs[n]]
            out_ptrs[6] = None  # qv not read back
            m.step_io(in_ptrs, out_ptrs, 2.0, 4)
        m.sync()
        for n, which in enumerate(order):
            for q in range(7):
                ref.set(q, inputs[which][q].numpy())
            ref.step(2.0, 4, 1)
            for q in range(6):
                assert np.array_equal(outs[n][q].numpy(), ref.get(q)), (n, vg.SPECIES[q])
            assert not outs[n][6].numpy().any()


def test_restart_files_match_the_reference_format(vg, oc, tmp_path):
    """Restart files of the device state are the bytes the reference's
    io::write_restart writes for the same state (committed golden file), and
    reading one restores the state, its time and step."""
    import os
    golden = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_restart.vibebin")
    import test_oracle_cpu as tc
    s = tc.small(oc)
    t = vg.Setup.defaults()
    for name, _ in vg.Setup._fields_:
        setattr(t, name, getattr(s, name))
    with vg.Model(t, vg.FP64_EXACT) as m, vg.Model(t, vg.FP64_EXACT) as fresh:
        m.step(1.0, 2, 1)
        path = str(tmp_path / "gpu.vibebin")
        m.write_restart(path, 12.5, 3)
        assert open(path, "rb").read() == open(golden, "rb").read()
        assert fresh.read_restart(golden) == (12.5, 3)
        for sp in range(12):
            assert np.array_equal(fresh.get(sp), m.get(sp)), vg.SPECIES[sp]
    t.pgf_perturbation, t.split_fast, t.weno_advective = 1, 1, 1  # the mixed path's composition
    with vg.Model(t, vg.MIXED) as mx:
        mx.read_restart(golden)
        mx.step(1.0, 2, 1)  # the FP32 working copy follows the loaded state
        assert np.isfinite(mx.get(4)).all()


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_energy_budget_matches_oracle(vg, oc, prec):
    """Global FP64 sums of the state (dyn::energy_budget) on the device against
    the oracle's serial sums (pinned to the reference), with terrain and
    moisture: 1e-12 relative per component (summation order and FMA
    contraction aside the terms are the same)."""
    kw = dict(terrain_kind=1, hill_h=300.0, hill_a=1500.0, hill_xc=2500.0, hill_yc=2000.0, moist=1,
              qv_surface=0.01, ref_kind=1)
    if prec == "mixed":
        kw.update(acoustic_mode=2, terrain_kind=0)  # the mixed path runs on flat terrain
    s = small_setup(vg, **kw)
    with vg.Model(s, vg.FP64 if prec == "fp64" else vg.MIXED) as m:
        m.step(1.0, 2, 1)
        o = oc.Model(oracle_setup(oc, s), "port")
        for sp in range(12):
            o.set(sp, m.get(sp))
        got, ref = m.energy_budget(), oc.energy_budget(o)
        for key in ref:
            assert abs(got[key] - ref[key]) <= 1e-12 * abs(ref[key]) + 1e-300, (key, got[key], ref[key])
