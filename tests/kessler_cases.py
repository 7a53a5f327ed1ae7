"""Seeded single-column cases for the Kessler warm-rain step
(KesslerMicrophysics::step_column, src/physics/microphysics_kessler.cpp):
supersaturated air without cloud (condensation), cloud above the
autoconversion threshold in subsaturated air (cloud evaporation), heavy rain
falling into dry air (sedimentation and rain evaporation), a one-level column
and a mixed profile."""
import numpy as np

RD, CP, KAPPA, P0, T0, EPS = 287.05, 1004.64, 0.28571, 1.0e5, 273.15, 0.62197


def qsat(p, t):
    tc = np.maximum(t - T0, -80.0)
    es = 611.2 * np.exp(17.67 * tc / (tc + 243.5))
    return EPS * es / np.maximum(p - es, 1.0)


def column(seed, n, rh, qc, qr, dz=250.0):
    rng = np.random.default_rng(seed)
    z = 50.0 + dz * np.arange(n) + rng.uniform(-20.0, 20.0, n)
    z = np.sort(z)
    p = P0 * np.exp(-z / 8000.0)
    theta = 300.0 + 0.004 * z + rng.uniform(-0.5, 0.5, n)
    t = theta * (p / P0) ** KAPPA
    qv = rh(rng, n) * qsat(p, t)
    rho = p / (RD * t)
    return dict(z=z, p=p, rho=rho, theta=theta, qv=qv, qc=qc(rng, n), qr=qr(rng, n))


def cases():
    zero = lambda rng, n: np.zeros(n)  # noqa: E731
    return [
        column(1, 24, lambda r, n: r.uniform(1.02, 1.15, n), zero, zero),
        column(2, 24, lambda r, n: r.uniform(0.6, 0.95, n), lambda r, n: r.uniform(0.5e-3, 3e-3, n), zero),
        column(3, 30, lambda r, n: r.uniform(0.3, 0.7, n), zero, lambda r, n: r.uniform(1e-3, 6e-3, n)),
        column(4, 1, lambda r, n: np.full(n, 1.05), lambda r, n: np.full(n, 2e-3), lambda r, n: np.full(n, 1e-3)),
        column(5, 40, lambda r, n: r.uniform(0.5, 1.2, n), lambda r, n: r.uniform(0.0, 2.5e-3, n) * (r.random(n) < 0.5),
               lambda r, n: r.uniform(0.0, 4e-3, n) * (r.random(n) < 0.5)),
    ]


DTS = [10.0, 60.0]
