"""Helmholtz solvers on the GPU (include/vibe_helmholtz.h) against the
oracle's restatement of the reference's HelmholtzSolver family
(src/time/helmholtz.cpp:126-495)."""
import numpy as np
import pytest

import helmholtz_cases as hc

pytestmark = pytest.mark.gpu


def dev_layout(oc, s, arr):
    return np.ascontiguousarray(oc.interior(s, 3, arr))


def make(vg, s, kind, dzeta, zs, max_iter=200, tol=1e-8):
    return vg.Helmholtz(kind, s.nx, s.ny, s.nz, s.dx, s.dy, s.z_top, dzeta, zs, max_iter, tol)


def test_operator_bit_exact(vg, oc):
    torch = pytest.importorskip("torch")
    s = hc.si_setup(oc)
    a, b, f, dzeta, zs = hc.si_problem(oc, s)
    port = oc.Model(s, "port")
    x = np.zeros_like(f)
    oc.interior(s, 3, x)[...] = np.random.default_rng(1).standard_normal(oc.interior(s, 3, x).shape)
    y_ref = port.helmholtz_apply(a, b, x)
    with make(vg, s, vg.HZ_KRYLOV_JACOBI, dzeta, zs) as h:
        h.set_coefficients(a, b)
        xd = torch.tensor(dev_layout(oc, s, x), device="cuda")
        yd = torch.zeros_like(xd)
        h.apply_dev(xd.data_ptr(), yd.data_ptr())
        torch.cuda.synchronize()
        assert np.array_equal(yd.cpu().numpy(), dev_layout(oc, s, y_ref))
        assert h.residual_l2(f, x) == port.helmholtz_residual_l2(a, b, f, x) or \
            abs(h.residual_l2(f, x) / port.helmholtz_residual_l2(a, b, f, x) - 1) < 1e-14


def test_vertical_tridiagonal_bit_exact(vg, oc):
    s = hc.si_setup(oc)
    a, b, f, dzeta, zs = hc.si_problem(oc, s)
    port = oc.Model(s, "port")
    xp, ip, rp, cp = port.helmholtz_solve(0, 200, 1e-8, a, b, f)
    with make(vg, s, vg.HZ_VERTICAL_TRIDIAGONAL, dzeta, zs) as h:
        rc, x = h.solve(a, b, f)
        assert rc == 0 and cp == 0
        assert np.array_equal(x, xp)
        assert h.iterations() == ip == 1 and h.residual() == rp == 0.0


@pytest.mark.parametrize("kind", [1, 2])
def test_reference_krylov_matches_oracle(vg, oc, kind):
    """The reference's Jacobi-BiCGSTAB (and its refinement wrapper) where it
    converges: same iteration count, same solution to reduction-order
    rounding."""
    s = hc.si_setup(oc, nx=24, ny=20, nz=12)
    a, b, f = hc.random_problem(oc, s)
    port = oc.Model(s, "port")
    dzeta, zs = np.diff(port.zeta()), port.terrain()
    xp, ip, rp, _ = port.helmholtz_solve(kind, 200, 1e-8, a, b, f)
    with make(vg, s, kind, dzeta, zs) as h:
        rc, x = h.solve(a, b, f)
        assert rc == 0
        assert h.iterations() == ip
        assert abs(h.residual() - rp) <= 1e-6 * rp
        assert np.abs(x - xp).max() <= 1e-10 * np.abs(xp).max()


def test_reference_krylov_diverges_like_oracle(vg, oc):
    """On the semi-implicit operator the reference's Jacobi-BiCGSTAB diverges
    (x is moved by the unpreconditioned s); the GPU kind reproduces it."""
    s = hc.si_setup(oc, nx=24, ny=20, nz=12)
    a, b, f, dzeta, zs = hc.si_problem(oc, s)
    port = oc.Model(s, "port")
    for max_iter in (3, 200):
        xp, ip, rp, _ = port.helmholtz_solve(2, max_iter, 1e-8, a, b, f)
        with make(vg, s, vg.HZ_KRYLOV_JACOBI, dzeta, zs, max_iter=max_iter) as h:
            rc, x = h.solve(a, b, f)
            assert h.iterations() == ip
            if np.isfinite(rp):
                assert abs(h.residual() / rp - 1) < 1e-6
            else:
                assert not np.isfinite(h.residual())


@pytest.mark.parametrize("kind", [3, 4])
@pytest.mark.parametrize("dims", [(32, 24, 16), (20, 12, 9), (7, 5, 6)])
def test_multigrid_bicgstab_converges_to_1e10(vg, oc, kind, dims):
    """Kinds 3 (FP64) and 4 (FP32 inner, FP64 refinement): the solution
    satisfies the reference's own operator (the oracle's apply) to a relative
    residual below 1e-10, and the two kinds agree."""
    nx, ny, nz = dims
    s = hc.si_setup(oc, nx=nx, ny=ny, nz=nz)
    a, b, f, dzeta, zs = hc.si_problem(oc, s)
    port = oc.Model(s, "port")
    fn = np.sqrt(np.sum(oc.interior(s, 3, f) ** 2))
    sols = {}
    for k in (3, 4):
        with make(vg, s, k, dzeta, zs, tol=1e-10) as h:
            rc, x = h.solve(a, b, f)
            assert rc == 0
            rel = port.helmholtz_residual_l2(a, b, f, x) / fn
            assert rel < 1e-10, (k, rel, h.iterations())
            assert h.residual() < 1e-10 and h.iterations() > 0
            if nx == 32:
                assert h.levels() == 3
            sols[k] = x
    assert np.abs(sols[3] - sols[4]).max() <= 1e-8 * np.abs(sols[3]).max()


def test_bad_arguments(vg, oc):
    s = hc.si_setup(oc, nx=8, ny=8, nz=4)
    dzeta = np.full(4, 0.25)
    with pytest.raises(vg.HelmholtzError):
        vg.Helmholtz(9, 8, 8, 4, 1.0, 1.0, 1.0, dzeta)
    with make(vg, s, vg.HZ_MG_BICGSTAB_MIXED, dzeta, None) as h:
        f = np.zeros(int(np.prod(oc.storage_shape(s, 3))))
        with pytest.raises(vg.HelmholtzError):
            h.solve(None, None, f)  # no coefficients yet
