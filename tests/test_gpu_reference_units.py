"""The reference's own unit-test assertions for this path, re-expressed
against the GPU library: tests/unit/test_time.cpp:116-183 (Helmholtz
manufactured solution, Krylov convergence, residual definition) and
tests/unit/test_dynamics.cpp:115-172 (advection of a constant field, linearity
of the advection operator, advective CFL by hand). The reference's grid for
them: dx = dy = 2 km, z_top = 20 km, zeta stretched from a first layer of
weight 1 by 1.08."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def zeta(nz, first=1.0, stretch=1.08):
    dz = first * stretch ** np.arange(nz)
    return np.concatenate([[0.0], np.cumsum(dz) / dz.sum()])


def cell(nx, ny, nz):
    return np.zeros((nz + 8) * (ny + 8) * (nx + 8))


def interior(a, nx, ny, nz):
    return a.reshape(nz + 8, ny + 8, nx + 8)[4:4 + nz, 4:4 + ny, 4:4 + nx]


def solver(vg, kind, nx, ny, nz, max_iter=300, tol=1e-10):
    return vg.Helmholtz(kind, nx, ny, nz, 2000.0, 2000.0, 20000.0, np.diff(zeta(nz)), np.zeros(nx * ny), max_iter,
                        tol)


def test_vertical_tridiagonal_recovers_manufactured_solution(vg, oc):
    """test_time.cpp:116-150: a = 1, b = 0.01, x = sin(pi (k+1)/(nz+1)),
    f = (2a/dz^2 + b) x - a/dz^2 (x(k-1) + x(k+1)) with clamped neighbours;
    the reference asserts recovery to 1e-8. The vertical solver's matrix
    (helmholtz.cpp:251-258) keeps the full diagonal 2a/dz^2 + b at the ground
    and lid levels and drops the neighbour beyond them (a zero value there),
    while that f takes the clamped neighbour, so no exact solve of the
    solver's system meets it at those levels: the compiled reference misses
    by 5.4e-5 at k = 0 (its C Thomas solve is also wrong, c_kernels.c:18-60),
    the oracle and this library by 4.2e-5. Two levels in from each end the
    manufactured solution is recovered to 1e-8, and the GPU solve is the
    oracle's bit for bit."""
    nx, ny, nz = 4, 4, 16
    a, b, f, xt = cell(nx, ny, nz), cell(nx, ny, nz), cell(nx, ny, nz), cell(nx, ny, nz)
    interior(a, nx, ny, nz)[...] = 1.0
    interior(b, nx, ny, nz)[...] = 0.01
    x_true = np.sin(np.pi * np.arange(1, nz + 1) / (nz + 1))
    interior(xt, nx, ny, nz)[...] = x_true[:, None, None]
    dz = np.diff(zeta(nz)) * 20000.0
    lo, hi = np.concatenate([[x_true[0]], x_true[:-1]]), np.concatenate([x_true[1:], [x_true[-1]]])
    fk = (2.0 / dz ** 2 + 0.01) * x_true - (lo + hi) / dz ** 2
    interior(f, nx, ny, nz)[...] = fk[:, None, None]
    with solver(vg, vg.HZ_VERTICAL_TRIDIAGONAL, nx, ny, nz) as h:
        assert h.name() == "vertical_tridiagonal"
        h.set_coefficients(a, b)
        rc, x = h.solve(a, b, f)
        assert rc == 0 and h.iterations() >= 1
    err = np.abs(interior(x, nx, ny, nz)[:, 0, 0] - x_true)
    assert err[2:-2].max() < 1e-8, err
    s = oc.defaults().copy(nx=nx, ny=ny, nz=nz, dx=2000.0, dy=2000.0, z_top=20000.0, zeta_first=1.0,
                           zeta_stretch=1.08, terrain_kind=0)
    xp, _, _, _ = oc.Model(s, "port").helmholtz_solve(0, 300, 1e-10, a, b, f)
    assert np.array_equal(x, xp)


def test_krylov_converges_on_smooth_rhs(vg):
    """test_time.cpp:152-170: Jacobi-BiCGSTAB on a = b = 1, f = sin(0.4 i)
    cos(0.3 j): finite solution, residual below 1."""
    nx, ny, nz = 8, 8, 8
    a, b, f = cell(nx, ny, nz), cell(nx, ny, nz), cell(nx, ny, nz)
    interior(a, nx, ny, nz)[...] = 1.0
    interior(b, nx, ny, nz)[...] = 1.0
    j, i = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    interior(f, nx, ny, nz)[...] = (np.sin(0.4 * i) * np.cos(0.3 * j))[None]
    with solver(vg, vg.HZ_KRYLOV_JACOBI, nx, ny, nz) as h:
        h.set_coefficients(a, b)
        _, x = h.solve(a, b, f)
        assert np.all(np.isfinite(x)) and h.residual() < 1.0


def test_residual_matches_definition(vg):
    """test_time.cpp:172-183: a = b = f = 1, x = 0 on 4 x 4 x 4: ||f - A x|| = sqrt(64)."""
    nx = ny = nz = 4
    a, b, f, x = cell(nx, ny, nz), cell(nx, ny, nz), cell(nx, ny, nz), cell(nx, ny, nz)
    for arr in (a, b, f):
        interior(arr, nx, ny, nz)[...] = 1.0
    with solver(vg, vg.HZ_KRYLOV_JACOBI, nx, ny, nz) as h:
        h.set_coefficients(a, b)
        assert abs(h.residual_l2(f, x) - 8.0) <= 1e-9


def advection_model(vg, scheme):
    """The reference composition (all flags 0) on the unit tests' grid, with
    the given scheme for the non-conservative scalar advection."""
    s = vg.Setup.defaults(nx=8, ny=8, nz=16, dx=2000.0, dy=2000.0, z_top=20000.0, zeta_first=1.0,
                          zeta_stretch=1.08, ref_kind=0, theta0=300.0, bubble_amplitude=0.0, qv_surface=0.0,
                          u_background=0.0, shear_u=0.0, advection=scheme, weno_scalars=0, weno_advective=0,
                          pgf_perturbation=0, split_fast=0, acoustic_mode=0, coriolis=0, divergence_damping=0.0)
    return s, vg.Model(s, vg.FP64)


def theta_tendency(vg, s, m, theta, u, v, w):
    st = m.state()
    for sp, val in ((0, u), (1, v), (2, w)):
        vg.interior(s, sp, st[sp])[...] = val
    vg.interior(s, 3, st[3])[...] = 1.0
    vg.interior(s, 4, st[4])[...] = theta
    m.set_state(st)
    return vg.interior(s, 4, m.slow_tendency()[4])


def test_advection_of_constant_field_is_zero(vg):
    """test_dynamics.cpp:115-130: u = 10, v = -5, w = 0.5, theta = 300: the
    theta tendency vanishes at interior points (1e-10)."""
    s, m = advection_model(vg, 2)
    with m:
        d = theta_tendency(vg, s, m, 300.0, 10.0, -5.0, 0.5)
        assert np.abs(d[1:-1, 1:-1, 1:-1]).max() <= 1e-10


def test_advection_is_linear(vg):
    """test_dynamics.cpp:132-157, 4th order: the tendency of 2 q1 - 3 q2 is
    2 d1 - 3 d2 at interior points (1e-9), u = 8, v = 3, w = 0."""
    s, m = advection_model(vg, 4)
    k, j, i = np.meshgrid(np.arange(s.nz), np.arange(s.ny), np.arange(s.nx), indexing="ij")
    q1 = np.sin(0.3 * i)
    q2 = np.cos(0.2 * j + k)
    with m:
        d1 = theta_tendency(vg, s, m, q1, 8.0, 3.0, 0.0)
        d2 = theta_tendency(vg, s, m, q2, 8.0, 3.0, 0.0)
        dc = theta_tendency(vg, s, m, 2.0 * q1 - 3.0 * q2, 8.0, 3.0, 0.0)
        assert np.abs((dc - (2.0 * d1 - 3.0 * d2))[1:-1, 1:-1, 1:-1]).max() <= 1e-9
        assert np.abs(d1).max() > 1e-3  # the operator acts


def test_advection_cfl_matches_hand_calculation(vg):
    """test_dynamics.cpp:159-170: at rest the advective CFL is 0; u = 100 m/s,
    dt = 10 s, dx = 2 km gives 0.5."""
    s, m = advection_model(vg, 2)
    with m:
        st = m.state()
        for sp in (0, 1, 2):
            st[sp][...] = 0.0
        m.set_state(st)
        assert abs(m.cfl(10.0, 1.0)[0]) <= 1e-12
        vg.interior(s, 0, st[0])[...] = 100.0
        m.set_state(st)
        assert abs(m.cfl(10.0, 1.0)[0] - 0.5) <= 1e-9
