"""Tangent-linear / adjoint on the GPU (include/vibe_tlad.h) against the
oracle's restatement of src/da/tangent_linear.cpp (pinned bit for bit to the
compiled reference), and the dot-product test of the reference's
check_adjoint (tangent_linear.cpp:761-790)."""
import numpy as np
import pytest

import tlad_cases as tc

pytestmark = pytest.mark.gpu


def setup(vg, oc, precision=0, **kw):
    s = tc.tl_setup(oc, **kw)
    port = oc.Model(s, "port")
    xb = tc.base_state(oc, port)
    t = vg.TLAD(s.nx, s.ny, s.nz, s.dx, s.dy, s.z_top, np.diff(port.zeta()), port.terrain(), precision)
    t.set_base(xb)
    return s, port, xb, t


def close(oc, s, got, ref, tol):
    for sp in range(12):
        g, r = oc.interior(s, sp, got[sp]), oc.interior(s, sp, ref[sp])
        scale = max(np.abs(r).max(), 1e-300)
        assert np.abs(g - r).max() <= tol * scale, (sp, np.abs(g - r).max() / scale)


def test_tl_and_ad_tendencies_match_oracle(vg, oc):
    s, port, xb, t = setup(vg, oc)
    with t:
        dx, by = tc.perturbation(oc, port, 1), tc.perturbation(oc, port, 2)
        close(oc, s, t.tl_tendency(dx), oc.tl_tendency(port, xb, dx), 1e-12)
        close(oc, s, t.ad_tendency(by), oc.ad_tendency(port, xb, by), 1e-12)


def test_tl_ad_propagate_match_oracle(vg, oc):
    s, port, xb, t = setup(vg, oc)
    with t:
        dx, dy = tc.perturbation(oc, port, 1), tc.perturbation(oc, port, 2)
        close(oc, s, t.tl_propagate(15.0, 3, dx), oc.tl_propagate(port, xb, dx, 15.0, 3), 1e-12)
        close(oc, s, t.ad_propagate(15.0, 3, dy), oc.ad_propagate(port, xb, dy, 15.0, 3), 1e-12)
        # halo points pass through
        out = t.tl_propagate(15.0, 1, dx)
        for sp in range(12):
            m = np.ones(dx[sp].size, bool)
            oc.interior(s, sp, m.view())[...] = False
            assert np.array_equal(out[sp][m], dx[sp][m])


@pytest.mark.parametrize("precision,tol", [(0, 1e-10), (1, 1e-5)])
def test_dot_product(vg, oc, precision, tol):
    """<M dx, dy> = <dx, M^T dy> over 5 steps: 1e-10 in FP64, 1e-5 with FP32
    arithmetic."""
    s, port, xb, t = setup(vg, oc, precision, nx=24, ny=20, nz=14)
    with t:
        dx, dy = tc.perturbation(oc, port, 3), tc.perturbation(oc, port, 4)
        lhs = tc.dot(oc, s, t.tl_propagate(15.0, 5, dx), dy)
        rhs = tc.dot(oc, s, dx, t.ad_propagate(15.0, 5, dy))
        assert abs(lhs - rhs) <= tol * max(abs(lhs), abs(rhs)), (lhs, rhs)


def test_fp32_tl_tracks_fp64(vg, oc):
    s, port, xb, t64 = setup(vg, oc, 0)
    _, _, _, t32 = setup(vg, oc, 1)
    with t64, t32:
        dx = tc.perturbation(oc, port, 5)
        close(oc, s, t32.tl_propagate(15.0, 4, dx), t64.tl_propagate(15.0, 4, dx), 1e-5)


def test_nonlinear_model_matches_oracle(vg, oc):
    """The nonlinear collocated RK3 of the FD check (nl_rk3 of the reference's
    test_tl_ad.cpp:100-199) against the oracle's restatement."""
    s, port, xb, t = setup(vg, oc)
    with t:
        x = [a + 0.1 * b for a, b in zip(xb, tc.perturbation(oc, port, 6))]
        close(oc, s, t.nl_tendency(x), oc.nl_tendency(port, xb, x), 1e-12)
        ref = x
        for _ in range(2):
            ref = oc.nl_step(port, xb, ref, 15.0)
        close(oc, s, t.nl_propagate(15.0, 2, x), ref, 1e-12)


def test_tangent_finite_difference_u_shape(vg, oc):
    """(N(xb + e dx) - N(xb)) / e -> F(xb, dx) on the GPU: U-shaped error in e
    with an interior minimum below 1e-6 (check_tangent, tangent_linear.cpp:832-880)."""
    s, port, xb, t = setup(vg, oc)
    with t:
        dx = tc.perturbation(oc, port, 41)
        f = t.tl_tendency(dx)
        n0 = t.nl_tendency(xb)
        nf = np.sqrt(sum(np.sum(a * a) for a in f))
        errs = []
        for e in [10.0 ** -k for k in range(1, 11)]:
            n1 = t.nl_tendency([a + e * b for a, b in zip(xb, dx)])
            fd = [(a - b) / e for a, b in zip(n1, n0)]
            errs.append(np.sqrt(sum(np.sum((a - b) ** 2) for a, b in zip(fd, f))) / nf)
        k = int(np.argmin(errs))
        assert 0 < k < len(errs) - 1 and errs[k] < 1e-6, errs


# ---- assimilation windows: TL/AD about the model's own trajectory ----------
def window_case(vg, prec, precision):
    s = vg.Setup.defaults(nx=20, ny=16, nz=12, dx=3000.0, dy=3000.0, z_top=12000.0, zeta_first=1.0,
                          zeta_stretch=1.0, ref_kind=1, bv_n=0.01, u_background=10.0, shear_u=0.0,
                          bubble_xc=30000.0, bubble_yc=24000.0, bubble_zc=3000.0, bubble_radius_x=9000.0,
                          bubble_radius_z=2000.0, bubble_amplitude=2.0, qv_surface=0.0, acoustic_mode=2,
                          pgf_perturbation=1, split_fast=1)
    m = vg.Model(s, prec)
    t = vg.TLAD(s.nx, s.ny, s.nz, s.dx, s.dy, s.z_top, np.diff(m.zeta()), m.terrain(), precision)
    return s, m, t


def perturb(vg, s, m, seed):
    rng = np.random.default_rng(seed)
    out = []
    for sp in range(12):
        a = np.zeros(m.size(sp))
        vg.interior(s, sp, a)[...] = tc.SCALE[sp] * rng.standard_normal(vg.interior(s, sp, a).shape)
        out.append(a)
    return out


def vdot(vg, s, a, b):
    return float(sum(np.sum(vg.interior(s, sp, a[sp]) * vg.interior(s, sp, b[sp])) for sp in range(12)))


DT_W, NSUB_W, TLSUB = 15.0, 6, 12


def test_window_tl_equals_stepwise_composition(vg):
    """Window TL (bases read in place from the model, checkpoints) gives the
    bits of the same sequence run through the host API: model step, state to
    the host, set_base, TL steps; the model is back at its initial state."""
    s, m, t = window_case(vg, vg.FP64, 0)
    with m, t:
        x0 = m.state()
        dx = perturb(vg, s, m, 1)
        with vg.Window(m, t, DT_W, NSUB_W, 7, every=3, tl_substeps=TLSUB) as w:
            got = w.tl(dx)
            for a, b in zip(m.state(), x0):
                assert np.array_equal(a, b)
        ref = dx
        for _ in range(7):
            t.set_base(m.state())
            ref = t.tl_propagate(DT_W / TLSUB, TLSUB, ref)
            m.step(DT_W, NSUB_W, 1)
        for sp in range(12):
            assert np.array_equal(got[sp], ref[sp]), vg.SPECIES[sp]


@pytest.mark.parametrize("mixed,tol", [(False, 1e-10), (True, 1e-5)])
def test_window_dot_product(vg, mixed, tol):
    """<L dx, dy> = <dx, L^T dy> over a 7-step window with checkpoints every 3
    steps (ragged last segment) and recomputation: 1e-10 with the FP64 model
    and TL/AD, 1e-5 with the mixed model and FP32-arithmetic TL/AD."""
    s, m, t = window_case(vg, vg.MIXED if mixed else vg.FP64, 1 if mixed else 0)
    with m, t:
        dx, dy = perturb(vg, s, m, 2), perturb(vg, s, m, 3)
        with vg.Window(m, t, DT_W, NSUB_W, 7, every=3, tl_substeps=TLSUB) as w:
            lhs = vdot(vg, s, w.tl(dx), dy)
            rhs = vdot(vg, s, dx, w.ad(dy))
            ms, ck, sg = w.stats()
            assert ck == 3 * sg // 6 and ms > 0.0
        assert abs(lhs - rhs) <= tol * max(abs(lhs), abs(rhs)), (lhs, rhs)


def test_window_automatic_checkpointing(vg):
    """every = 0: the small window fits in device memory, so every step is
    stored (no recomputation); TL and AD are the bits of the checkpointed and
    recomputed window."""
    s, m, t = window_case(vg, vg.FP64, 0)
    with m, t:
        dx, dy = perturb(vg, s, m, 5), perturb(vg, s, m, 6)
        with vg.Window(m, t, DT_W, NSUB_W, 7, every=0, tl_substeps=TLSUB) as w:
            tl0, ad0 = w.tl(dx), w.ad(dy)
            _, ck, sg = w.stats()
            assert ck == 7 * sg // 2  # 7 checkpoints, a one-step segment double-buffered
        with vg.Window(m, t, DT_W, NSUB_W, 7, every=3, tl_substeps=TLSUB) as w:
            tl3, ad3 = w.tl(dx), w.ad(dy)
        for a, b in zip(tl0 + ad0, tl3 + ad3):
            assert np.array_equal(a, b)
