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
