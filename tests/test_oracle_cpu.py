"""CPU tests of the oracle: the plain-C restatement against the reference
compiled unchanged (bit for bit) where the reference tree was available at
build time, against the committed golden fixtures everywhere, and the
reference's own known-answer tests for the C ABI."""
import ctypes
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def small(oc, **kw):
    s = oc.defaults()
    base = dict(nx=20, ny=16, nz=12, dx=250.0, dy=250.0, z_top=3000.0, zeta_first=1.0, zeta_stretch=1.08,
                bubble_xc=2500.0, bubble_yc=2000.0, bubble_zc=1000.0, bubble_radius_x=1500.0,
                bubble_radius_z=1000.0, u_background=5.0, shear_u=0.001,
                pgf_perturbation=0, split_fast=0, weno_advective=0, acoustic_mode=0)
    base.update(kw)
    for k, v in base.items():
        setattr(s, k, v)
    return s


REF_CASES = [dict(advection=a, weno_scalars=w, coriolis=c, ref_kind=r, moist=mo,
                  divergence_damping=dd, divergence_order=do)
             for (a, w, c, r, mo, dd, do) in [(2, 0, 0, 0, 0, 0.0, 2), (4, 0, 1, 1, 0, 100.0, 2),
                                              (6, 0, 2, 0, 1, 0.0, 2), (5, 1, 0, 1, 0, 50.0, 4),
                                              (5, 1, 1, 0, 1, 0.0, 2)]]


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(GOLDEN), "..", "oracle", "_ref",
                                                    "libvibe_ref.so")),
                    reason="reference-linked oracle not built (reference tree absent)")
@pytest.mark.parametrize("case", range(len(REF_CASES)))
def test_port_is_bit_exact_to_reference(oc, case):
    s = small(oc, **REF_CASES[case])
    a, b = oc.Model(s, "port"), oc.Model(s, "ref")
    for sp in range(12):
        assert np.array_equal(a.get(sp), b.get(sp))
    for r in range(5):
        assert np.array_equal(a.reffield(r), b.reffield(r))
    assert np.array_equal(a.sponge_profile(), b.sponge_profile())
    for x, y in zip(a.slow_tendency(), b.slow_tendency()):
        assert np.array_equal(x, y)
    a.acoustic_substep(0.2)
    b.acoustic_substep(0.2)
    assert a.rk3_step(2.0, 3) == b.rk3_step(2.0, 3) == 0
    for sp in range(12):
        assert np.array_equal(a.get(sp), b.get(sp)), oc.SPECIES[sp]
    t = small(oc, acoustic_mode=1)
    a, b = oc.Model(t, "port"), oc.Model(t, "ref")
    a.hevi_substep(0.7)
    b.hevi_substep(0.7)
    a.sponge(6.0)
    b.sponge(6.0)
    for sp in range(12):
        assert np.array_equal(a.get(sp), b.get(sp))


def _golden(name):
    path = os.path.join(GOLDEN, name + ".npz")
    if not os.path.exists(path):
        pytest.skip("golden fixture %s missing" % name)
    return np.load(path)


def test_port_matches_golden_steps(oc):
    """Fixtures written by tests/golden/make_golden.py from the reference
    compiled unchanged (oracle/_ref): the port must reproduce them bit for
    bit on this machine's libm (x86 and Arm glibc agree on these inputs)."""
    g = _golden("ref_steps")
    for case in range(int(g["ncases"])):
        s = small(oc, **{k: g["case%d_%s" % (case, k)].item() for k in g["keys"]})
        m = oc.Model(s, "port")
        for n in range(int(g["case%d_nsteps" % case])):
            assert m.rk3_step(float(g["dt"]), int(g["nsub"])) == 0
        for sp in range(7):
            got = oc.interior(s, sp, m.get(sp))
            ref = g["case%d_sp%d" % (case, sp)]
            assert np.allclose(got, ref, rtol=0, atol=1e-13 * max(np.abs(ref).max(), 1e-300)), (case, sp)


def test_port_matches_golden_kernels(oc):
    g = _golden("ref_kernels")
    s = small(oc, acoustic_mode=1)
    m = oc.Model(s, "port")
    tend = m.slow_tendency()
    for sp in range(7):
        assert np.array_equal(oc.interior(s, sp, tend[sp]), g["tend_sp%d" % sp])
    m.hevi_substep(0.7)
    for sp in range(7):
        assert np.array_equal(oc.interior(s, sp, m.get(sp)), g["hevi_sp%d" % sp])


def test_reference_composition_diverges_and_documented_one_does_not(oc):
    """The reference's own composition (total-Exner pressure gradient, fast
    terms counted twice) blows up within a few steps on a warm bubble; the
    documented composition (pi', fast terms once, advective WENO5) stays
    bounded. 32x32x20 at 250 m keeps this a few seconds."""
    base = dict(nx=32, ny=32, nz=20, dx=250.0, dy=250.0, z_top=5000.0, zeta_first=1.0, zeta_stretch=1.0,
                bubble_xc=4000.0, bubble_yc=4000.0, bubble_zc=1500.0, qv_surface=0.0, u_background=0.0,
                shear_u=0.0, advection=5, weno_scalars=1)
    bad = oc.Model(small(oc, **base), "port")
    rcs = [bad.rk3_step(2.0, 6) for _ in range(12)]
    assert 1 in rcs
    good_s = small(oc, **base, pgf_perturbation=1, split_fast=1, weno_advective=1)
    good = oc.Model(good_s, "port")
    for _ in range(12):
        assert good.rk3_step(2.0, 6) == 0
    w = oc.interior(good_s, 2, good.get(2))
    assert np.abs(w).max() < 5.0


# ---- the composition flags against the reference's own operators ----------
# oracle/ref/ref_driver.cpp composes pgf_perturbation, split_fast,
# weno_advective and w_rigid from Equations::tendencies / acoustic_tendencies
# and Advection::scalar, and the consistent HEVI (acoustic_mode = 2) from
# acoustic_tendencies (its column matrix probed from that operator) and
# timeint::thomas_solve; the port restates the same flags in plain C.
HEADLINE_FLAGS = dict(advection=5, weno_scalars=1, weno_advective=1, pgf_perturbation=1, split_fast=1, ref_kind=1)
FLAG_CASES = [dict(HEADLINE_FLAGS, acoustic_mode=0),
              dict(HEADLINE_FLAGS, acoustic_mode=0, moist=1, qv_surface=0.01, w_rigid=1),
              dict(advection=4, weno_scalars=0, pgf_perturbation=1, split_fast=1, acoustic_mode=0,
                   divergence_damping=50.0, moist=1, qv_surface=0.01, coriolis=1),
              dict(HEADLINE_FLAGS, acoustic_mode=0, split_fast=0, terrain_kind=1, hill_h=300.0, hill_a=1500.0,
                   hill_xc=2500.0, hill_yc=2000.0)]
HEVI_CASES = [dict(HEADLINE_FLAGS, acoustic_mode=2, hevi_beta=0.5),
              dict(HEADLINE_FLAGS, acoustic_mode=2, hevi_beta=0.6, w_rigid=1),
              dict(HEADLINE_FLAGS, acoustic_mode=2, hevi_beta=0.7, pgf_perturbation=0, ref_kind=0, terrain_kind=1,
                   hill_h=300.0, hill_a=1500.0, hill_xc=2500.0, hill_yc=2000.0)]


def _need_ref():
    if not os.path.exists(os.path.join(os.path.dirname(GOLDEN), "..", "oracle", "_ref", "libvibe_ref.so")):
        pytest.skip("reference-linked oracle not built (reference tree absent)")


@pytest.mark.parametrize("case", range(len(FLAG_CASES)))
def test_composition_flags_port_is_bit_exact_to_reference_operators(oc, case):
    """pgf_perturbation, split_fast, weno_advective and w_rigid with the
    explicit substep: slow tendency and two RK3 steps bit for bit."""
    _need_ref()
    s = small(oc, **FLAG_CASES[case])
    a, b = oc.Model(s, "port"), oc.Model(s, "ref")
    for x, y in zip(a.slow_tendency(), b.slow_tendency()):
        assert np.array_equal(x, y)
    for _ in range(2):
        assert a.rk3_step(2.0, 3) == b.rk3_step(2.0, 3) == 0
    for sp in range(12):
        assert np.array_equal(a.get(sp), b.get(sp)), oc.SPECIES[sp]


@pytest.mark.parametrize("case", range(len(HEVI_CASES)))
def test_consistent_hevi_port_matches_reference_operators(oc, case):
    """The consistent HEVI substep of the port against the one assembled from
    the reference's acoustic operator and thomas_solve: from the same state,
    every field's change agrees to 1e-11 of its size (the two differ only in
    operation order; pi' = pi - pi0 carries ~1e-16 of pi into u and v), and
    two full RK3 steps of the headline composition agree to 1e-9 of each
    field's size. A sign, weight or staggering error would differ at O(1)."""
    _need_ref()
    s = small(oc, **HEVI_CASES[case])
    a, b = oc.Model(s, "port"), oc.Model(s, "ref")
    for x, y in zip(a.slow_tendency(), b.slow_tendency()):
        assert np.array_equal(x, y)
    assert a.rk3_step(2.0, 3) == 0
    b.set_state(a.state())
    x0 = a.state()
    a.hevi_substep(0.7)
    b.hevi_substep(0.7)
    for sp in (0, 1, 2, 3, 5):
        x, y, z = (oc.interior(s, sp, f) for f in (a.get(sp), b.get(sp), x0[sp]))
        change = np.abs(x - z).max()
        assert change > 0
        assert np.abs(x - y).max() <= 1e-11 * change, oc.SPECIES[sp]
    for _ in range(2):
        assert a.rk3_step(2.0, 3) == b.rk3_step(2.0, 3) == 0
    for sp in range(7):
        x, y = oc.interior(s, sp, a.get(sp)), oc.interior(s, sp, b.get(sp))
        assert np.abs(x - y).max() <= 1e-9 * max(np.abs(x).max(), 1e-30), oc.SPECIES[sp]


K_RD, K_CP, K_CV = 287.05, 1004.64, 717.63


def _column_case(oc, beta, nz=16):
    """One column (nx = ny = 1, so the horizontal terms vanish) of the N =
    0.01 profile on stretched levels, with random pi' and interior w."""
    s = small(oc, nx=1, ny=1, nz=nz, dx=250.0, dy=250.0, z_top=4000.0, zeta_first=1.0, zeta_stretch=1.06,
              ref_kind=1, bubble_amplitude=0.0, u_background=0.0, shear_u=0.0, qv_surface=0.0,
              acoustic_mode=2, hevi_beta=beta, pgf_perturbation=1, split_fast=1)
    m = oc.Model(s, "port")
    rng = np.random.default_rng(7)
    for sp in (0, 1):
        m.set(sp, np.zeros(m.size(sp)))
    w = np.zeros(m.size(2))
    oc.interior(s, 2, w)[1:nz, 0, 0] = rng.uniform(-1.0, 1.0, nz - 1)
    m.set(2, w)
    pi = m.reffield(1).copy()
    oc.interior(s, 5, pi)[:, 0, 0] += rng.uniform(-1e-3, 1e-3, nz)
    m.set(5, pi)
    return s, m


def _acoustic_energy(oc, s, m):
    """E = 1/2 sum_k (dz_k / kappa_k) pi'_k^2 + 1/2 sum_f (r_f dzf_f / (cp t_f)) w_f^2:
    the quadratic form in which the linear column operator (w rate
    -cp t_f d(pi')/dz on interior faces, pi' rate kappa_k * (-d(r_f w)/dz))
    is skew-adjoint, so Crank-Nicolson at beta = 1/2 keeps it exactly."""
    nz = s.nz
    zeta = m.zeta()
    dzc = np.maximum(np.diff(zeta) * s.z_top, 1.0)
    th0 = oc.interior(s, 4, m.reffield(0))[:, 0, 0]
    pi0 = oc.interior(s, 5, m.reffield(1))[:, 0, 0]
    r0 = oc.interior(s, 3, m.reffield(2))[:, 0, 0]
    kap = (K_RD / K_CV) * pi0 / np.maximum(r0, 1e-8)
    f = np.arange(1, nz)
    rf = 0.5 * (r0[f - 1] + r0[f])
    tf = 0.5 * (th0[f - 1] + th0[f])
    dzf = dzc[f]
    pip = oc.interior(s, 5, m.get(5))[:, 0, 0] - pi0
    w = oc.interior(s, 2, m.get(2))[1:nz, 0, 0]
    return 0.5 * np.sum(dzc / kap * pip ** 2) + 0.5 * np.sum(rf * dzf / (K_CP * tf) * w ** 2)


def test_consistent_hevi_conserves_linear_acoustic_energy(oc):
    """Property of the consistent HEVI (no reference routine exists for it):
    at beta = 1/2 it is the trapezoidal rule of the linear column acoustics,
    so the column's acoustic energy is kept to rounding over 200 substeps
    at a vertical Courant number far above 1; off-centred (beta = 0.6) it
    decays monotonically; the ground and lid faces stay at rest."""
    s, m = _column_case(oc, 0.5)
    e0 = _acoustic_energy(oc, s, m)
    for _ in range(200):
        m.hevi_substep(2.0)
    assert abs(_acoustic_energy(oc, s, m) - e0) <= 1e-10 * e0
    w = oc.interior(s, 2, m.get(2))[:, 0, 0]
    assert w[0] == 0.0 and w[-1] == 0.0
    s, m = _column_case(oc, 0.6)
    es = [_acoustic_energy(oc, s, m)]
    for _ in range(20):
        m.hevi_substep(2.0)
        es.append(_acoustic_energy(oc, s, m))
    assert all(b < a for a, b in zip(es, es[1:])) and es[-1] < 0.9 * es[0]


def test_consistent_hevi_tends_to_forward_backward_as_dtau_shrinks(oc):
    """One off-centred HEVI substep and one explicit forward-backward
    substep from the same state integrate the same linear acoustics; their
    difference, relative to the substep's change, shrinks in proportion to
    dtau (first order), on the full 3-D state with terrain."""
    base = dict(HEADLINE_FLAGS, terrain_kind=1, hill_h=300.0, hill_a=1500.0, hill_xc=2500.0, hill_yc=2000.0)
    hs, fs = small(oc, acoustic_mode=2, hevi_beta=0.6, **base), small(oc, acoustic_mode=0, **base)
    start = oc.Model(hs, "port")
    assert start.rk3_step(1.0, 4) == 0
    x0 = start.state()
    ratios = []
    for dtau in (0.08, 0.04, 0.02, 0.01):
        h, f = oc.Model(hs, "port"), oc.Model(fs, "port")
        h.set_state(x0)
        f.set_state(x0)
        h.hevi_substep(dtau)
        f.acoustic_substep(dtau)
        num = sum(np.linalg.norm(oc.interior(hs, sp, h.get(sp)) - oc.interior(hs, sp, f.get(sp)))
                  / max(np.linalg.norm(oc.interior(hs, sp, x0[sp])), 1e-30) for sp in (0, 1, 2, 3, 5))
        den = sum(np.linalg.norm(oc.interior(hs, sp, f.get(sp)) - oc.interior(hs, sp, x0[sp]))
                  / max(np.linalg.norm(oc.interior(hs, sp, x0[sp])), 1e-30) for sp in (0, 1, 2, 3, 5))
        ratios.append(num / den)
    for a, b in zip(ratios, ratios[1:]):
        assert 0.4 <= b / a <= 0.6, ratios


# ---- C-ABI known answers on the oracle (test_common.cpp:163-266) -------------
def test_oracle_c_abi_known_answers(oc):
    L = oc.port_lib()
    n = 24
    a, c, b, d = np.ones(n - 1), np.ones(n - 1), np.full(n, -4.0), np.ones(n)
    x, ws = np.zeros(n), np.zeros(n)
    assert L.vo_tridiagonal_solve(a.ctypes.data, b.ctypes.data, c.ctypes.data, d.ctypes.data, n, x.ctypes.data,
                                  ws.ctypes.data) == 0
    lhs = -4.0 * x
    lhs[1:] += x[:-1]
    lhs[:-1] += x[1:]
    assert np.abs(lhs - 1).max() <= 1e-10
    z = np.zeros(2)
    o = np.ones(2)
    assert L.vo_tridiagonal_solve(None, z.ctypes.data, None, o.ctypes.data, 2, x.ctypes.data, ws.ctypes.data) == 1
    assert L.vo_tridiagonal_solve(None, None, None, None, 2, x.ctypes.data, ws.ctypes.data) == 2
    ql, qr = ctypes.c_double(), ctypes.c_double()
    L.vo_weno5_reconstruct(3.5, 3.5, 3.5, 3.5, 3.5, ctypes.byref(ql), ctypes.byref(qr))
    assert abs(ql.value - 3.5) <= 1e-12 and abs(qr.value - 3.5) <= 1e-12
    xs = np.ones(10000)
    xs[0], xs[-1] = 1e16, -1e16
    assert abs(L.vo_neumaier_sum(xs.ctypes.data, xs.size) - 9998.0) <= 1e-6


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(GOLDEN), "..", "oracle", "_ref",
                                                    "libvibe_ref.so")),
                    reason="reference-linked oracle not built (reference tree absent)")
def test_reference_c_thomas_is_wrong_port_is_right(oc):
    """The shipped vibe_tridiagonal_solve_f64 (c_kernels.c:18-60) misses its
    own contract; the oracle follows the contract."""
    ref = ctypes.CDLL(oc.REF_SO)
    ref.vibe_tridiagonal_solve_f64.restype = ctypes.c_int
    ref.vibe_tridiagonal_solve_f64.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_int] + [ctypes.c_void_p] * 2
    n = 24
    a, c, b, d = np.ones(n - 1), np.ones(n - 1), np.full(n, -4.0), np.ones(n)
    x, ws = np.zeros(n), np.zeros(n)
    ref.vibe_tridiagonal_solve_f64(a.ctypes.data, b.ctypes.data, c.ctypes.data, d.ctypes.data, n, x.ctypes.data,
                                   ws.ctypes.data)
    lhs = -4.0 * x
    lhs[1:] += x[:-1]
    lhs[:-1] += x[1:]
    assert np.abs(lhs - 1).max() > 1e-2


# ---- Helmholtz family and the semi-implicit step (src/time/helmholtz.cpp,
# src/time/semi_implicit.cpp) ----
REF_SO_PATH = os.path.join(os.path.dirname(GOLDEN), "..", "oracle", "_ref", "libvibe_ref.so")
need_ref = pytest.mark.skipif(not os.path.exists(REF_SO_PATH),
                              reason="reference-linked oracle not built (reference tree absent)")


@need_ref
@pytest.mark.parametrize("kind", [1, 2])
def test_helmholtz_krylov_port_is_bit_exact_to_reference(oc, kind):
    import helmholtz_cases as hc
    s = hc.si_setup(oc, nx=16, ny=12, nz=10)
    a, b, f = hc.random_problem(oc, s)
    p, r = oc.Model(s, "port"), oc.Model(s, "ref")
    assert p.helmholtz_residual_l2(a, b, f, f) == r.helmholtz_residual_l2(a, b, f, f)
    for max_iter in (1, 2, 3, 200):
        xp, ip, rp, cp = p.helmholtz_solve(kind, max_iter, 1e-8, a, b, f)
        xr, ir, rr, cr = r.helmholtz_solve(kind, max_iter, 1e-8, a, b, f)
        assert (cp, ip, rp) == (cr, ir, rr)
        assert np.array_equal(xp, xr)
    assert rp < 1e-8  # converges on this operator


@need_ref
def test_multigrid_transfers_port_is_bit_exact_to_reference(oc):
    import helmholtz_cases as hc
    s = hc.si_setup(oc, nx=14, ny=9, nz=5)
    p, r = oc.Model(s, "port"), oc.Model(s, "ref")
    x = np.random.default_rng(3).standard_normal(p.size(3))
    assert np.array_equal(p.multigrid_restrict(x), r.multigrid_restrict(x))
    assert np.array_equal(p.multigrid_prolong(x), r.multigrid_prolong(x))


@need_ref
def test_semi_implicit_step_port_is_bit_exact_to_reference(oc):
    """O-SI: three steps; the reference's default solver (krylov_multigrid)
    diverges on this operator (non-finite residual), which the port
    reproduces; the state itself stays finite (the solution is dropped)."""
    import helmholtz_cases as hc
    s = hc.si_setup(oc, nx=16, ny=12, nz=10)
    p, r = oc.Model(s, "port"), oc.Model(s, "ref")
    for _ in range(3):
        op, orf = p.si_step(30.0), r.si_step(30.0)
        assert op[0] == orf[0] == 0 and op[1] == orf[1]
        assert not np.isfinite(op[2]) and not np.isfinite(orf[2])
        assert np.array_equal(op[3], orf[3], equal_nan=True)
        assert np.array_equal(op[4], orf[4]) and np.array_equal(op[5], orf[5])
        for sp in range(12):
            assert np.array_equal(p.get(sp), r.get(sp)), sp


@need_ref
@pytest.mark.parametrize("case", range(4))
def test_nest_transfers_port_is_bit_exact_to_reference(oc, case):
    import nest_cases as nc
    pdims, cdims, pl = nc.CASES[case]
    assert np.array_equal(oc.davies_profile(pl["boundary_zone"], 1.0, "port"),
                          oc.davies_profile(pl["boundary_zone"], 1.0, "ref"))
    parent = nc.fields(oc, pdims, 1)
    out = {}
    for kind in ("port", "ref"):
        child = nc.fields(oc, cdims, 2)
        oc.nest_interpolate_from_parent(pl, nc.STAGGERS, pdims, parent, cdims, child, kind)
        interp = [c.copy() for c in child]
        inner = nc.fields(oc, cdims, 3)
        oc.nest_apply_lateral_boundary(pl, nc.STAGGERS, cdims, inner, interp, kind)
        par = [p.copy() for p in parent]
        oc.nest_restrict_to_parent(pl, nc.STAGGERS, cdims, inner, pdims, par, kind)
        out[kind] = (interp, inner, par)
    for a, b in zip(out["port"], out["ref"]):
        for x, y in zip(a, b):
            assert np.array_equal(x, y)


@need_ref
def test_tlad_port_is_bit_exact_to_reference(oc):
    """TangentLinearModel::step / propagate and AdjointModel::step_adjoint /
    propagate_with_trajectory (src/da/tangent_linear.cpp) against the port."""
    import tlad_cases as tc
    s = tc.tl_setup(oc)
    p, r = oc.Model(s, "port"), oc.Model(s, "ref")
    xb = tc.base_state(oc, p)
    dx, dy = tc.perturbation(oc, p, 1), tc.perturbation(oc, p, 2)
    for a, b in zip(oc.tl_step(p, xb, dx, 15.0), oc.tl_step(r, xb, dx, 15.0)):
        assert np.array_equal(a, b)
    for a, b in zip(oc.ad_step(p, xb, dy, 15.0), oc.ad_step(r, xb, dy, 15.0)):
        assert np.array_equal(a, b)
    for a, b in zip(oc.tl_propagate(p, xb, dx, 15.0, 3), oc.tl_propagate(r, xb, dx, 15.0, 3)):
        assert np.array_equal(a, b)
    for a, b in zip(oc.ad_propagate(p, xb, dy, 15.0, 3), oc.ad_propagate(r, xb, dy, 15.0, 3)):
        assert np.array_equal(a, b)


def test_tlad_port_dot_product(oc):
    """The port's AD is the transpose of its TL (the reference's check_adjoint)."""
    import tlad_cases as tc
    s = tc.tl_setup(oc)
    p = oc.Model(s, "port")
    xb = tc.base_state(oc, p)
    dx, dy = tc.perturbation(oc, p, 1), tc.perturbation(oc, p, 2)
    lhs = tc.dot(oc, s, oc.tl_propagate(p, xb, dx, 15.0, 2), dy)
    rhs = tc.dot(oc, s, dx, oc.ad_propagate(p, xb, dy, 15.0, 2))
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), abs(rhs))


@need_ref
@pytest.mark.parametrize("case", [0, 3])
def test_cfl_diagnostics_port_is_bit_exact_to_reference(oc, case):
    s = small(oc, **REF_CASES[case])
    p, r = oc.Model(s, "port"), oc.Model(s, "ref")
    assert p.rk3_step(1.0, 2) == r.rk3_step(1.0, 2) == 0
    assert oc.cfl(p, 2.0, 0.3) == oc.cfl(r, 2.0, 0.3)
    assert oc.max_stable_dt(p) == oc.max_stable_dt(r)


def fd_curve(oc, s, port, xb, dx, eps):
    """Relative error of (N(xb + e dx) - N(xb)) / e against F(xb, dx)."""
    t = oc.tl_tendency(port, xb, dx)
    f0 = oc.nl_tendency(port, xb, xb)
    nt = np.sqrt(sum(np.sum(a * a) for a in t))
    out = []
    for e in eps:
        f1 = oc.nl_tendency(port, xb, [a + e * b for a, b in zip(xb, dx)])
        fd = [(a - b) / e for a, b in zip(f1, f0)]
        num = np.sqrt(sum(np.sum((a - b) ** 2) for a, b in zip(fd, t)))
        out.append(num / max(nt, np.sqrt(sum(np.sum(a * a) for a in fd)), 1e-30))
    return out


def test_tl_tendency_is_the_derivative_of_the_nonlinear_tendency(oc):
    """check_tangent's finite-difference criterion (tangent_linear.cpp:832-880;
    the U-shaped curve of test_tl_ad.cpp:420-460) at the tendency level:
    truncation error O(e) for large e, rounding O(1/e) for small e, and a
    small interior minimum."""
    import tlad_cases as tc
    s = tc.tl_setup(oc)
    p = oc.Model(s, "port")
    xb = tc.base_state(oc, p)
    dx = tc.perturbation(oc, p, 41)
    eps = [10.0 ** -k for k in range(1, 11)]
    errs = fd_curve(oc, s, p, xb, dx, eps)
    k = int(np.argmin(errs))
    assert 0 < k < len(eps) - 1 and errs[0] > errs[k] and errs[-1] > errs[k], errs
    assert errs[k] < 1e-6, errs


def test_restart_port_matches_golden_and_reads_back(oc, tmp_path):
    """.vibebin restart (io::write_restart, field_io.cpp:207-227): the port
    writes the bytes of the reference-written golden file for the same state,
    and reading it back restores the state, time and step."""
    golden = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_restart.vibebin")
    s = small(oc)
    p = oc.Model(s, "port")
    assert p.rk3_step(1.0, 2) == 0
    path = str(tmp_path / "port.vibebin")
    assert oc.write_restart(p, path, 12.5, 3) == 0
    assert open(path, "rb").read() == open(golden, "rb").read()
    q = oc.Model(s, "port")
    assert oc.read_restart(q, golden) == (0, 12.5, 3)
    for sp in range(12):
        assert np.array_equal(q.get(sp), p.get(sp))


@need_ref
def test_restart_port_is_bit_exact_to_reference(oc, tmp_path):
    s = small(oc, advection=5, weno_scalars=1, moist=1, qv_surface=0.01)
    p, r = oc.Model(s, "port"), oc.Model(s, "ref")
    assert p.rk3_step(1.0, 2) == 0 and r.rk3_step(1.0, 2) == 0
    a, b = str(tmp_path / "a.vibebin"), str(tmp_path / "b.vibebin")
    assert oc.write_restart(p, a, 7.0, 11) == 0 and oc.write_restart(r, b, 7.0, 11) == 0
    assert open(a, "rb").read() == open(b, "rb").read()
    q = oc.Model(s, "ref")
    assert oc.read_restart(q, a) == (0, 7.0, 11)
    for sp in range(12):
        assert np.array_equal(q.get(sp), r.get(sp))


@need_ref
@pytest.mark.parametrize("case", [0, 3])
def test_energy_budget_port_is_bit_exact_to_reference(oc, case):
    """dyn::energy_budget (diagnostics.cpp:255-277) with terrain and moisture."""
    kw = dict(REF_CASES[case], terrain_kind=1, hill_h=300.0, hill_a=1500.0, hill_xc=2500.0, hill_yc=2000.0,
              moist=1, qv_surface=0.01)
    s = small(oc, **kw)
    p, r = oc.Model(s, "port"), oc.Model(s, "ref")
    assert p.rk3_step(1.0, 2) == 0 and r.rk3_step(1.0, 2) == 0
    assert oc.energy_budget(p) == oc.energy_budget(r)


# ---- Kessler warm rain (src/physics/microphysics_kessler.cpp) ----
def _kessler_runs(oc, kind):
    import kessler_cases as kc
    out = []
    for c in kc.cases():
        for dt in kc.DTS:
            for offset in (1,):
                k = oc.Kessler.defaults(exner_offset=offset)
                out.append(oc.kessler_column(k, dt, c["z"], c["p"], c["rho"], c["theta"], c["qv"], c["qc"], c["qr"],
                                             kind=kind))
    return out


@need_ref
def test_kessler_column_port_is_bit_exact_to_reference(oc):
    """The restated column step against KesslerMicrophysics::step_column of
    the compiled reference: saturation adjustment, autoconversion and
    accretion, sedimentation, rain evaporation, positivity."""
    for a, b in zip(_kessler_runs(oc, "port"), _kessler_runs(oc, "ref")):
        for x, y in zip(a[:4], b[:4]):
            assert np.array_equal(x, y)
        assert a[4] == b[4]


def test_kessler_column_port_matches_golden(oc):
    path = os.path.join(GOLDEN, "ref_kessler.npz")
    if not os.path.exists(path):
        pytest.skip("golden fixture ref_kessler.npz missing")
    g = np.load(path)
    runs = _kessler_runs(oc, "port")
    assert int(g["nruns"]) == len(runs)
    for r, run in enumerate(runs):
        for f, name in enumerate(("theta", "qv", "qc", "qr")):
            assert np.array_equal(run[f], g["run%d_%s" % (r, name)]), (r, name)
        assert run[4] == float(g["run%d_precip" % r])
    # every process acted somewhere in the cases
    import kessler_cases as kc
    cs = kc.cases()
    assert np.any(runs[0][2] > 0)                         # condensation (case 0, no cloud before)
    assert np.all(runs[2][2] <= cs[1]["qc"])              # cloud evaporates or converts in subsaturated air
    assert runs[4][4] > 0.0                                # rain reaches the ground
    assert np.any(runs[4][1] > cs[2]["qv"])                # rain evaporation moistens the dry layer


def test_kessler_coupling_in_rk3_step(oc):
    """vo_rk3_step with the scheme coupled: a moist case condenses (qc
    appears), with physics off it does not; the tendency of a state without
    water is zero."""
    s = small(oc, moist=1, qv_surface=0.018, qv_decay_height=2500.0)
    k = oc.Kessler.defaults(exner_offset=0)
    a, b = oc.Model(s, "port"), oc.Model(s, "port")
    oc.set_physics_kessler(a, k)
    assert a.rk3_step(1.0, 2) == 0 and b.rk3_step(1.0, 2) == 0
    qc_a, qc_b = oc.interior(s, 7, a.get(7)), oc.interior(s, 7, b.get(7))
    assert qc_a.max() > 0.0 and qc_b.max() == 0.0
    dry = oc.Model(small(oc, qv_surface=0.0), "port")
    for t in oc.kessler_tendency(dry, k, 1.0):
        assert not np.any(t)


# ---- C-ABI edge cases (NULL arguments, empty and negative grids, a grid
# without interior points, one-row systems) -----------------------------------
def test_oracle_c_abi_edge_cases(oc):
    import cabi_edge_cases as ce
    out = ce.run_cases(ce.oracle_table(oc.PORT_SO))
    assert out[0] == 0 and out[1][0] == 1.5  # one row: d / b
    assert out[2] == 1 and out[3][0] == -7.0  # zero one-row pivot: singular, x untouched
    assert out[4] == 2 and out[5][0] == -7.0  # n = 0: bad argument
    assert out[6] == 0 and list(out[7]) == [0.5, 0.75, -0.625]  # a, c NULL: diagonal
    assert out[8] == -7.0  # WENO5 with a NULL output writes nothing
    assert out[9] == out[10] == out[11] == 0.0  # bilinear: NULL f, nz <= 0
    assert all(np.all(a == 7.0) for a in out[-4:])  # flux: dqdt untouched


@need_ref
def test_c_abi_edge_cases_port_is_bit_exact_to_reference(oc):
    import cabi_edge_cases as ce
    ce.compare(ce.run_cases(ce.oracle_table(oc.PORT_SO)), ce.run_cases(ce.reference_table(oc.REF_SO)))
