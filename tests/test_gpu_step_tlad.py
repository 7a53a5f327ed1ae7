"""Tangent-linear and adjoint of the model's own step (vibe_gb300_tendency_tl /
_ad, vibe_gb300_step_tl / _ad, and windows with tlad = None) on the GPU.

The step is the one vibe_gb300_step takes (runge_kutta.cpp:77-119 composed
with WENO5 scalars in advective form, the pi' pressure gradient, the fast
terms only in the consistent HEVI substeps, the sponge and the rigid ground
and lid). Its nonlinear form is pinned to the oracle elsewhere
(test_gpu_step.py, test_gpu_config1.py, test_gpu_config2.py); here the
tangent-linear is checked against central differences of that nonlinear
model, and the adjoint against the tangent-linear by the dot-product test:
1e-10 with FP64 models, 1e-5 with mixed models (FP32 arithmetic).

Central differences of the nonlinear model are limited by its own rounding:
total theta (~300 K) enters the flux-form WENO fluxes, whose FP64 rounding
(~1e-13 of theta u) divided by 2 e sets the floor. The checks therefore take
the smallest error over e = 1e-2 .. 1e-6 (the bottom of the U-curve)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# perturbation scale per species (u, v, w in m/s, rho, theta in K, pi, qv..)
SCALE = [1.0, 1.0, 0.1, 1e-4, 0.5, 50.0 / 1e5 * 0.2857, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0]
DT, NSUB = 15.0, 6


def case(vg, prec, **kw):
    base = dict(nx=20, ny=16, nz=12, dx=3000.0, dy=3000.0, z_top=12000.0, zeta_first=1.0, zeta_stretch=1.05,
                ref_kind=1, bv_n=0.01, u_background=10.0, bubble_xc=30000.0, bubble_yc=24000.0,
                bubble_zc=3000.0, bubble_radius_x=9000.0, bubble_radius_z=2000.0, bubble_amplitude=2.0,
                qv_surface=0.0, advection=5, weno_scalars=1, weno_advective=1, pgf_perturbation=1, split_fast=1,
                acoustic_mode=2, hevi_beta=0.6, w_rigid=1)
    base.update(kw)
    s = vg.Setup.defaults(**base)
    m = vg.Model(s, prec)
    # seeded theta' noise everywhere: where theta is flat the WENO5 weights
    # sit at the smoothness floor (beta ~ 1e-6), their derivatives are
    # exact but finite differences never reach the linear regime
    th = m.get(4)
    rng = np.random.default_rng(99)
    vg.interior(s, 4, th)[...] += rng.uniform(-0.5, 0.5, vg.interior(s, 4, th).shape)
    m.set(4, th)
    m.step(DT, NSUB, 2)  # winds and theta' in every direction
    return s, m


def perturb(vg, s, m, seed):
    """Seeded interior perturbation (qv and the moisture species unperturbed:
    the dry state holds qv = 0, where its positivity clip is not differentiable)."""
    rng = np.random.default_rng(seed)
    out = []
    for sp in range(12):
        a = np.zeros(m.size(sp))
        v = vg.interior(s, sp, a)
        v[...] = SCALE[sp] * rng.standard_normal(v.shape)
        out.append(a)
    return out


def tendency_box(vg, s, sp, a):
    """Points the slow tendency writes: the staggered box of each species."""
    v = np.asarray(a).reshape(vg.storage_shape(s, sp))
    h = vg.HALO
    return v[h:h + s.nz + (sp == 2), h:h + s.ny + (sp == 1), h:h + s.nx + (sp == 0)]


def vdot(a, b):
    return float(sum(np.dot(x, y) for x, y in zip(a, b)))


def rel_max(a, b):
    num = max(float(np.max(np.abs(x - y))) for x, y in zip(a, b))
    den = max(float(np.max(np.abs(y))) for y in b)
    return num / den


EPS = [10.0 ** -k for k in range(2, 7)]


def u_curve(fn, x0, dx, tl, pick, fields):
    """Per field, max relative error of (fn(x0 + e dx) - fn(x0 - e dx)) / 2e
    against tl for every e of EPS."""
    curves = {sp: [] for sp in fields}
    for e in EPS:
        fp = fn([a + e * b for a, b in zip(x0, dx)])
        fm = fn([a - e * b for a, b in zip(x0, dx)])
        for sp in fields:
            got, ref = pick(sp, tl[sp]), pick(sp, (fp[sp] - fm[sp]) / (2 * e))
            curves[sp].append(float(np.max(np.abs(got - ref))) / max(float(np.max(np.abs(ref))), 1e-300))
    return curves


def test_tendency_tl_matches_central_differences(vg):
    """(R(x + e dx) - R(x - e dx)) / 2e -> TL(dx) (FP64 model, WENO5 scalars):
    the bottom of the U-curve below 1e-6 (theta: 1e-4, its FD rounding floor)."""
    s, m = case(vg, vg.FP64)
    with m:
        x0 = m.state()
        dx = perturb(vg, s, m, 1)
        tl = m.tendency_tl(dx)

        def tend(x):
            m.set_state(x)
            return m.slow_tendency()

        curves = u_curve(tend, x0, dx, tl, lambda sp, a: tendency_box(vg, s, sp, a), (0, 1, 2, 3, 4))
        m.set_state(x0)
        for sp, c in curves.items():
            assert min(c) < (1e-4 if sp == 4 else 1e-6), (vg.SPECIES[sp], c)


@pytest.mark.parametrize("mixed,tol", [(False, 1e-10), (True, 1e-5)])
@pytest.mark.parametrize("weno", [1, 0])
def test_tendency_dot_product(vg, mixed, tol, weno):
    """<TL dx, y> = <dx, AD y> for the slow tendency, WENO5 and 4th-order
    central scalars, with Coriolis on the central case."""
    kw = {} if weno else dict(weno_scalars=0, weno_advective=0, advection=4, coriolis=1)
    s, m = case(vg, vg.MIXED if mixed else vg.FP64, **kw)
    with m:
        dx = perturb(vg, s, m, 2)
        y = perturb(vg, s, m, 3)
        lhs = vdot(m.tendency_tl(dx), y)
        rhs = vdot(dx, m.tendency_ad(y))
        assert abs(lhs - rhs) <= tol * max(abs(lhs), abs(rhs)), (lhs, rhs)


def test_step_tl_matches_central_differences(vg):
    """(M(x + e dx) - M(x - e dx)) / 2e -> TL(dx) for one model step (FP64);
    the model's state is left as it was."""
    s, m = case(vg, vg.FP64)
    with m:
        x0 = m.state()
        dx = perturb(vg, s, m, 4)
        tl = m.step_tl(DT, NSUB, dx)
        for a, b in zip(m.state(), x0):
            assert np.array_equal(a, b)

        def step(x):
            m.set_state(x)
            m.step(DT, NSUB, 1)
            return m.state()

        curves = u_curve(step, x0, dx, tl, lambda sp, a: vg.interior(s, sp, a), (0, 1, 2, 3, 4, 5))
        m.set_state(x0)
        for sp, c in curves.items():
            assert min(c) < 1e-4, (vg.SPECIES[sp], c)


@pytest.mark.parametrize("mixed,tol", [(False, 1e-10), (True, 1e-5)])
def test_step_dot_product(vg, mixed, tol):
    s, m = case(vg, vg.MIXED if mixed else vg.FP64)
    with m:
        dx, y = perturb(vg, s, m, 5), perturb(vg, s, m, 6)
        lhs = vdot(m.step_tl(DT, NSUB, dx), y)
        rhs = vdot(dx, m.step_ad(DT, NSUB, y))
        assert abs(lhs - rhs) <= tol * max(abs(lhs), abs(rhs)), (lhs, rhs)


def test_mixed_step_tl_tracks_fp64(vg):
    """The mixed model's FP32 step TL agrees with the FP64 model's to 1e-4."""
    s, m64 = case(vg, vg.FP64)
    _, m32 = case(vg, vg.MIXED)
    with m64, m32:
        dx = perturb(vg, s, m64, 7)
        a, b = m32.step_tl(DT, NSUB, dx), m64.step_tl(DT, NSUB, dx)
        assert rel_max([vg.interior(s, sp, a[sp]) for sp in range(6)],
                       [vg.interior(s, sp, b[sp]) for sp in range(6)]) < 1e-4


def test_own_window_equals_stepwise_composition(vg):
    """A 5-step window of the model's own step TL (checkpoints every 2 steps)
    gives the bits of step_tl applied step by step along the trajectory, and
    leaves the model at its initial state."""
    s, m = case(vg, vg.FP64)
    with m:
        x0 = m.state()
        dx = perturb(vg, s, m, 8)
        with vg.Window(m, None, DT, NSUB, 5, every=2) as w:
            got = w.tl(dx)
        for a, b in zip(m.state(), x0):
            assert np.array_equal(a, b)
        ref = dx
        for _ in range(5):
            ref = m.step_tl(DT, NSUB, ref)
            m.step(DT, NSUB, 1)
        for sp in range(12):
            assert np.array_equal(got[sp], ref[sp]), vg.SPECIES[sp]


@pytest.mark.parametrize("mixed,tol", [(False, 1e-10), (True, 1e-5)])
def test_own_window_dot_product(vg, mixed, tol):
    """<L dx, dy> = <dx, L^T dy> over a 7-step window of the model's own step
    with checkpoints every 3 steps (ragged last segment) and recomputation."""
    s, m = case(vg, vg.MIXED if mixed else vg.FP64)
    with m:
        dx, dy = perturb(vg, s, m, 9), perturb(vg, s, m, 10)
        with vg.Window(m, None, DT, NSUB, 7, every=3) as w:
            lhs = vdot(w.tl(dx), dy)
            rhs = vdot(dx, w.ad(dy))
            ms, ck, sg = w.stats()
            assert ms > 0.0 and ck == 3 * sg // 9  # 3 checkpoints, 3 states x 3 steps per segment
        assert abs(lhs - rhs) <= tol * max(abs(lhs), abs(rhs)), (lhs, rhs)


def test_own_step_refusals(vg):
    """The reference HEVI substep has no adjoint here: a clear error (before
    any step is taken)."""
    s = vg.Setup.defaults(nx=12, ny=10, nz=8, acoustic_mode=1)
    with vg.Model(s, vg.FP64) as m:
        dx = perturb(vg, s, m, 11)
        with pytest.raises(vg.VibeError):
            m.step_tl(DT, NSUB, dx)
