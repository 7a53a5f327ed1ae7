"""The semi-implicit step on the GPU (vibe_gb300_si_step) against the
oracle's O-SI restatement (src/time/semi_implicit.cpp:56-106,167-226)."""
import numpy as np
import pytest

import helmholtz_cases as hc

pytestmark = pytest.mark.gpu


def gpu_setup(vg, oc, s):
    return vg.Setup.defaults(**{name: getattr(s, name) for name, _ in oc.Setup._fields_})


def test_si_step_exact_matches_oracle_with_reference_solver(vg, oc):
    """FP64_EXACT with the reference's default solver: bitwise state over 3
    steps, same iteration counts, non-finite solver residual on both sides."""
    s = hc.si_setup(oc, nx=20, ny=16, nz=12)
    port = oc.Model(s, "port")
    with vg.Model(gpu_setup(vg, oc, s), vg.FP64_EXACT) as m:
        for _ in range(3):
            it, res, _ = m.si_step(30.0, kind=vg.HZ_KRYLOV_MULTIGRID)
            rc, pit, pres, _, _, _ = port.si_step(30.0, kind=1)
            assert rc == 0 and it == pit
            assert not np.isfinite(res) and not np.isfinite(pres)
            for sp in range(12):
                assert np.array_equal(m.get(sp), port.get(sp)), vg.SPECIES[sp]


def test_si_step_vertical_solver_bit_exact(vg, oc):
    s = hc.si_setup(oc, nx=20, ny=16, nz=12)
    port = oc.Model(s, "port")
    with vg.Model(gpu_setup(vg, oc, s), vg.FP64_EXACT) as m:
        it, res, pin = m.si_step(30.0, kind=vg.HZ_VERTICAL_TRIDIAGONAL, want_pi=True)
        rc, pit, pres, ppin, _, _ = port.si_step(30.0, kind=0)
        assert rc == 0 and (it, res) == (pit, pres)
        assert np.array_equal(pin, ppin)
        for sp in range(12):
            assert np.array_equal(m.get(sp), port.get(sp)), vg.SPECIES[sp]


@pytest.mark.parametrize("kind", [3, 4])
def test_si_step_multigrid_solution_satisfies_reference_operator(vg, oc, kind):
    """FP64 path with the GB300 solvers: the state matches the oracle to
    1e-12 (it does not depend on the solve) and the solution satisfies the
    assembled problem to a relative residual below 1e-10."""
    s = hc.si_setup(oc, nx=32, ny=24, nz=16)
    port = oc.Model(s, "port")
    with vg.Model(gpu_setup(vg, oc, s), vg.FP64) as m:
        it, res, pin = m.si_step(30.0, kind=kind, tol=1e-10, want_pi=True)
        rc, _, _, _, rhs, acoef = port.si_step(30.0, kind=0)
        assert rc == 0 and it > 0 and res < 1e-10
        b = np.zeros_like(acoef)
        oc.interior(s, 3, b)[...] = 1.0
        fn = np.sqrt(np.sum(oc.interior(s, 3, rhs) ** 2))
        assert port.helmholtz_residual_l2(acoef, b, rhs, pin) / fn < 1e-10
        for sp in range(7):
            g, r = oc.interior(s, sp, m.get(sp)), oc.interior(s, sp, port.get(sp))
            assert np.abs(g - r).max() <= 1e-12 * max(np.abs(r).max(), 1.0), vg.SPECIES[sp]


def test_si_step_rejects_mixed_precision(vg, oc):
    s = hc.si_setup(oc, nx=12, ny=10, nz=8, terrain_kind=0, ref_kind=1, pgf_perturbation=1, split_fast=1)
    with vg.Model(gpu_setup(vg, oc, s), vg.MIXED) as m:
        with pytest.raises(vg.VibeError):
            m.si_step(30.0)
