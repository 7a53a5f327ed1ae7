"""The single-domain 512 x 512 x 80 workload, on a 128 x 128 x 80 horizontal
sample the oracle steps in seconds: the same stretched levels (50 m at the
ground, 20 km top), the N = 0.01 profile, u = 10 m/s, the seeded theta'
white noise below 1 km and the 20 seeded warm bubbles (bench.perturbed_state),
WENO5 scalars, dt = 6 s with 6 consistent-HEVI substeps per stage, the
composition the bench times.

Each of 10 steps starts both GPU paths from the oracle's state at that step,
so the bound is per step: FP64 path within 1e-12, mixed path within 1e-5 of
each field's scale (velocities: the common velocity scale)."""
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
STEPS = 10
NS = 128


def _bench():
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    import bench
    return bench


def per_step_errors(vg, s, got, ref):
    ins = [vg.interior(s, q, ref[q]) for q in range(7)]
    vs = max(float(np.abs(ins[q]).max()) for q in range(3))
    out = {}
    for q in range(7):
        scale = vs if q < 3 else float(np.abs(ins[q]).max())
        scale = scale if scale > 0.0 else 1.0  # a field that is zero (qv of the dry case): absolute error
        d = vg.interior(s, q, got[q]) - ins[q]
        out[vg.SPECIES[q]] = (float(np.abs(d).max()) / scale, float(np.sqrt(np.mean(d * d))) / scale)
    return out


def test_workload_sample_per_step_against_oracle(vg, oc):
    b = _bench()
    s = b.case_setup(vg.Setup, NS, NS)
    t = oc.Setup()
    for name, _ in oc.Setup._fields_:
        setattr(t, name, getattr(s, name))
    o = oc.Model(t, "port")
    th, pi = b.perturbed_state(s, o.get(4), o.get(3), o.zeta(), seed=1, nx_full=NS, ny_full=NS)
    o.set(4, th)
    o.set(5, pi)
    worst = {vg.FP64: 0.0, vg.MIXED: 0.0}
    with vg.Model(s, vg.FP64) as m64, vg.Model(s, vg.MIXED) as mmx:
        for n in range(STEPS):
            x0 = [o.get(q) for q in range(7)]
            assert o.rk3_step(b.DT, b.NSUB) == 0
            ref = [o.get(q) for q in range(7)]
            for m, tol in ((m64, 1e-12), (mmx, 1e-5)):
                for q in range(7):
                    m.set(q, x0[q])
                m.step(b.DT, b.NSUB, 1)
                err = per_step_errors(vg, s, m.state()[:7], ref)
                worst[m.precision] = max(worst[m.precision], max(e[0] for e in err.values()))
                assert all(e[0] <= tol for e in err.values()), (n, m.precision, err)
    print("128x128x80 workload sample, worst per-step max relative error over %d steps: FP64 %.2e, mixed %.2e"
          % (STEPS, worst[vg.FP64], worst[vg.MIXED]))
