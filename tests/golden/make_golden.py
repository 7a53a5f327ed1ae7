"""Write the golden fixtures from the reference compiled unchanged.

Run where the reference tree is present (it builds oracle/_ref first):
    make -C oracle ref && python tests/golden/make_golden.py
Outputs (interior points of u v w rho theta pi qv, float64):
  ref_steps.npz    RK3 steps of the reference composition for several
                   schemes (RungeKutta3Integrator::step restated over the
                   reference's Equations/Advection/Damping objects)
  ref_kernels.npz  Equations::tendencies and AcousticSubstepper::step (HEVI)
  ref_restart.vibebin  io::write_restart of the small case after one RK3
                   step (dt 1, 2 substeps), time 12.5, step 3
  ref_kessler.npz  KesslerMicrophysics::step_column on the seeded columns of
                   tests/kessler_cases.py (theta, qv, qc, qr after the step and
                   the surface precipitation rate)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
import oracle_ctypes as oc  # noqa: E402
from test_oracle_cpu import small  # noqa: E402

CASES = [dict(advection=2, weno_scalars=0, coriolis=0, ref_kind=0),
         dict(advection=4, weno_scalars=0, coriolis=1, ref_kind=1),
         dict(advection=5, weno_scalars=1, coriolis=0, ref_kind=1, divergence_damping=50.0)]
KEYS = ["advection", "weno_scalars", "coriolis", "ref_kind", "divergence_damping"]
DT, NSUB, NSTEPS = 2.0, 3, 2


def main():
    if not oc.ref_available():
        sys.exit("oracle/_ref/libvibe_ref.so not built (make -C oracle ref)")
    out = {"ncases": len(CASES), "keys": np.array(KEYS), "dt": DT, "nsub": NSUB}
    for c, kw in enumerate(CASES):
        full = {k: kw.get(k, 0.0 if k == "divergence_damping" else 0) for k in KEYS}
        s = small(oc, **full)
        m = oc.Model(s, "ref")
        for _ in range(NSTEPS):
            assert m.rk3_step(DT, NSUB) == 0
        for k, v in full.items():
            out["case%d_%s" % (c, k)] = np.array(v)
        out["case%d_nsteps" % c] = NSTEPS
        for sp in range(7):
            out["case%d_sp%d" % (c, sp)] = oc.interior(s, sp, m.get(sp)).copy()
    np.savez_compressed(os.path.join(HERE, "ref_steps.npz"), **out)
    s = small(oc, acoustic_mode=1)
    m = oc.Model(s, "ref")
    kern = {}
    tend = m.slow_tendency()
    for sp in range(7):
        kern["tend_sp%d" % sp] = oc.interior(s, sp, tend[sp]).copy()
    m.hevi_substep(0.7)
    for sp in range(7):
        kern["hevi_sp%d" % sp] = oc.interior(s, sp, m.get(sp)).copy()
    np.savez_compressed(os.path.join(HERE, "ref_kernels.npz"), **kern)
    m = oc.Model(small(oc), "ref")
    assert m.rk3_step(1.0, 2) == 0
    assert oc.write_restart(m, os.path.join(HERE, "ref_restart.vibebin"), 12.5, 3) == 0
    from test_oracle_cpu import _kessler_runs
    runs = _kessler_runs(oc, "ref")
    kes = {"nruns": len(runs)}
    for r, run in enumerate(runs):
        for f, name in enumerate(("theta", "qv", "qc", "qr")):
            kes["run%d_%s" % (r, name)] = run[f]
        kes["run%d_precip" % r] = run[4]
    np.savez_compressed(os.path.join(HERE, "ref_kessler.npz"), **kes)
    print("wrote", os.listdir(HERE))


if __name__ == "__main__":
    main()
