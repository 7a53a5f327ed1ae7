"""GPU C-ABI kernels (include/vibe_c_kernels.h) against the reference's own
known-answer tests (tests/unit/test_common.cpp:163-266,
tests/unit/test_time.cpp:53-100, tests/unit/test_gpu_precision.cpp) and
against the oracle on seeded inputs."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


# ---- known answers from the reference's tests --------------------------------
def test_thomas_residual_diag_1_m4_1(vg):
    """test_common.cpp:163-175: diag(1,-4,1), d = 1, residual <= 1e-10 (the
    reference's own c_kernels.c fails this with 9e-2)."""
    n = 24
    a = np.ones(n - 1)
    c = np.ones(n - 1)
    b = np.full(n, -4.0)
    d = np.ones(n)
    rc, x = vg.tridiagonal_solve(a, b, c, d)
    assert rc == 0
    lhs = -4.0 * x
    lhs[1:] += x[:-1]
    lhs[:-1] += x[1:]
    assert np.abs(lhs - 1.0).max() <= 1e-10


def test_thomas_singular_and_bad_args(vg):
    """test_common.cpp:177-186."""
    lib = vg.lib
    b = np.zeros(2)
    d = np.ones(2)
    x = np.zeros(2)
    ws = np.zeros(2)
    assert lib.vibe_tridiagonal_solve_f64(None, b.ctypes.data, None, d.ctypes.data, 2, x.ctypes.data,
                                          ws.ctypes.data) == 1
    assert lib.vibe_tridiagonal_solve_f64(None, None, None, None, 2, x.ctypes.data, ws.ctypes.data) == 2
    assert lib.vibe_tridiagonal_solve_f64(None, b.ctypes.data, None, d.ctypes.data, 0, x.ctypes.data,
                                          ws.ctypes.data) == 2


def test_thomas_mms_and_variable_coefficients(vg, oc):
    """test_time.cpp:53-88 pattern; variable coefficients vs the oracle."""
    n = 24
    j = np.arange(n)
    b = 4.0 + 0.1 * j
    d = np.sin(0.3 * j)
    a = np.full(n - 1, -1.0)
    c = np.full(n - 1, -1.2)
    rc, x = vg.tridiagonal_solve(a, b, c, d)
    assert rc == 0
    xo = np.zeros(n)
    ws = np.zeros(n)
    L = oc.port_lib()
    assert L.vo_tridiagonal_solve(a.ctypes.data, b.ctypes.data, c.ctypes.data, d.ctypes.data, n, xo.ctypes.data,
                                  ws.ctypes.data) == 0
    assert np.abs(x - xo).max() <= 1e-12 * np.abs(xo).max()


def test_thomas_batched_matches_oracle(vg, oc):
    rng = np.random.default_rng(7)
    n_sys, n = 1000, 60
    b = 4.0 + rng.random((n_sys, n))
    a = -rng.random((n_sys, n - 1))
    c = -rng.random((n_sys, n - 1))
    d = rng.standard_normal((n_sys, n))
    rc, x = vg.tridiagonal_solve_batched(a, b, c, d)
    assert rc == 0
    L = oc.port_lib()
    for s in (0, 17, 999):
        xo = np.zeros(n)
        ws = np.zeros(n)
        aa, bb, cc, dd = (np.ascontiguousarray(v[s]) for v in (a, b, c, d))
        L.vo_tridiagonal_solve(aa.ctypes.data, bb.ctypes.data, cc.ctypes.data, dd.ctypes.data, n, xo.ctypes.data,
                               ws.ctypes.data)
        assert np.abs(x[s] - xo).max() <= 1e-12 * np.abs(xo).max()


@pytest.mark.parametrize("n,n_sys", [(129, 1), (200, 5), (225, 4), (1000, 37), (4097, 3)])
def test_thomas_tall_systems_warp_cooperative(vg, oc, n, n_sys):
    """n > 128: one warp per system (chunked Thomas per lane + the 2x2
    block-tridiagonal interface system). Agrees with the oracle's sequential
    sweep to rounding (1e-12 of the solution's scale) on diagonally dominant
    systems, including a one-row last chunk (n = 225: 28 chunks of 8 rows and
    one of 1)."""
    rng = np.random.default_rng(n)
    b = 4.0 + rng.random((n_sys, n))
    a = -rng.random((n_sys, n - 1))
    c = -rng.random((n_sys, n - 1))
    d = rng.standard_normal((n_sys, n))
    rc, x = vg.tridiagonal_solve_batched(a, b, c, d)
    assert rc == 0
    L = oc.port_lib()
    for s in range(n_sys):
        xo = np.zeros(n)
        ws = np.zeros(n)
        aa, bb, cc, dd = (np.ascontiguousarray(v[s]) for v in (a, b, c, d))
        L.vo_tridiagonal_solve(aa.ctypes.data, bb.ctypes.data, cc.ctypes.data, dd.ctypes.data, n, xo.ctypes.data,
                               ws.ctypes.data)
        assert np.abs(x[s] - xo).max() <= 1e-12 * np.abs(xo).max()
    # the single-system entry point takes the same path; NULL a / c read as 0
    rc1, x1 = vg.tridiagonal_solve(None, b[0], c[0], d[0])
    assert rc1 == 0
    A = np.diag(b[0]) + np.diag(c[0], 1)
    assert np.abs(x1 - np.linalg.solve(A, d[0])).max() <= 1e-12 * np.abs(x1).max()
    # an exact zero pivot is reported
    bz = b.copy()
    bz[0, 0] = 0.0
    az = a.copy()
    az[0, :] = 0.0
    rcz, _ = vg.tridiagonal_solve_batched(az, bz, c, d)
    assert rcz == 1


def _residual(a, b, c, d, x):
    """max |Ax - d| / max(|A||x| + |d|) of one tridiagonal system."""
    r = b * x - d
    r[1:] += a * x[:-1]
    r[:-1] += c * x[1:]
    scale = np.abs(b * x) + np.abs(d)
    scale[1:] += np.abs(a * x[:-1])
    scale[:-1] += np.abs(c * x[1:])
    return float(np.abs(r).max() / scale.max())


def _oracle_solve(oc, a, b, c, d):
    n = b.size
    xo, ws = np.zeros(n), np.zeros(n)
    aa, bb, cc, dd = (np.ascontiguousarray(v) for v in (a, b, c, d))
    rc = oc.port_lib().vo_tridiagonal_solve(aa.ctypes.data, bb.ctypes.data, cc.ctypes.data, dd.ctypes.data, n,
                                            xo.ctypes.data, ws.ctypes.data)
    return rc, xo


@pytest.mark.parametrize("n", [300, 1000])
def test_thomas_tall_zero_chunk_pivot_falls_back_to_the_sweep(vg, oc, n):
    """A nonsingular system whose diagonal is 0 at the first row of a warp
    chunk (rows per chunk m = ceil(n/32)): the chunked elimination has a zero
    pivot there, the single sweep does not. The reference's contract
    (c_kernels.c:26,34,40) reports singular only on a zero sweep pivot, so
    the solver must solve it, as the oracle's sweep does."""
    m = (n + 31) // 32
    rng = np.random.default_rng(n + 5)
    n_sys = 6
    b = 4.0 + rng.random((n_sys, n))
    a = -rng.random((n_sys, n - 1))
    c = -rng.random((n_sys, n - 1))
    d = rng.standard_normal((n_sys, n))
    for s in range(n_sys):  # a zero at the start of chunk s+1 (every system a different chunk)
        b[s, (s + 1) * m] = 0.0
    rc, x = vg.tridiagonal_solve_batched(a, b, c, d)
    assert rc == 0
    for s in range(n_sys):
        rco, xo = _oracle_solve(oc, a[s], b[s], c[s], d[s])
        assert rco == 0
        assert np.abs(x[s] - xo).max() <= 1e-12 * np.abs(xo).max()
        assert _residual(a[s], b[s], c[s], d[s], x[s]) <= 1e-13


def test_thomas_tall_non_dominant_diagonals(vg, oc):
    """Diagonals of either sign and no dominance (|b| ~ |a| + |c|): every
    system is solved to the sweep's accuracy (residual 1e-10 of the row
    scale, the sweep's own residual within a factor 100), and the return code
    is the sweep's."""
    rng = np.random.default_rng(11)
    n, n_sys = 513, 40
    b = rng.uniform(-2.0, 2.0, (n_sys, n))
    a = rng.uniform(-1.0, 1.0, (n_sys, n - 1))
    c = rng.uniform(-1.0, 1.0, (n_sys, n - 1))
    d = rng.standard_normal((n_sys, n))
    _, x = vg.tridiagonal_solve_batched(a, b, c, d)
    for s in range(n_sys):
        rco, xo = _oracle_solve(oc, a[s], b[s], c[s], d[s])
        assert rco == 0
        r_gpu, r_seq = _residual(a[s], b[s], c[s], d[s], x[s]), _residual(a[s], b[s], c[s], d[s], xo)
        assert r_gpu <= max(1e-10, 100.0 * r_seq), (s, r_gpu, r_seq)
        rc1, x1 = vg.tridiagonal_solve(a[s], b[s], c[s], d[s])
        assert rc1 == rco


def test_host_entry_points_reentrant_and_allocation_free(vg, oc):
    """c_kernels.h:17-18: reentrant, OpenMP-thread-safe, no allocation per
    call. Eight host threads call vibe_tridiagonal_solve_f64 and
    vibe_neumaier_sum_f64 concurrently on their own inputs (ctypes releases
    the interpreter lock during the call); every result matches the oracle.
    After each thread's first calls, further calls of the same sizes make no
    allocation (vibe_c_allocations() stays put). Prints the latency of one
    n = 80 solve."""
    import threading
    import time
    lib = vg.lib
    lib.vibe_c_allocations.restype = ctypes.c_ulonglong
    lib.vibe_neumaier_sum_f64.restype = ctypes.c_double
    lib.vibe_neumaier_sum_f64.argtypes = [ctypes.c_void_p, ctypes.c_size_t]
    L = oc.port_lib()
    nthreads, calls, n = 8, 40, 80
    cases = []
    for t in range(nthreads):
        rng = np.random.default_rng(100 + t)
        sys_ = []
        for q in range(calls):
            b = 4.0 + rng.random(n)
            a, c = -rng.random(n - 1), -rng.random(n - 1)
            d = rng.standard_normal(n)
            xs = rng.standard_normal(5000) * 10.0 ** rng.integers(-8, 8, 5000)
            _, xo = _oracle_solve(oc, a, b, c, d)
            so = L.vo_neumaier_sum(xs.ctypes.data, xs.size)
            sys_.append((a, b, c, d, xo, xs, so))
        cases.append(sys_)
    errors = []
    warm, go, done = threading.Barrier(nthreads + 1), threading.Barrier(nthreads + 1), threading.Barrier(nthreads + 1)

    def worker(t):
        try:
            x, ws = np.zeros(n), np.zeros(n)

            def run_all():
                for a, b, c, d, xo, xs, so in cases[t]:
                    rc = lib.vibe_tridiagonal_solve_f64(a.ctypes.data, b.ctypes.data, c.ctypes.data, d.ctypes.data,
                                                        n, x.ctypes.data, ws.ctypes.data)
                    if rc != 0 or np.abs(x - xo).max() > 1e-12 * np.abs(xo).max():
                        errors.append(("thomas", t, rc))
                    sv = lib.vibe_neumaier_sum_f64(xs.ctypes.data, xs.size)
                    if abs(sv - so) > 1e-13 * np.abs(xs).sum():
                        errors.append(("neumaier", t, sv, so))
            run_all()
            warm.wait()
            go.wait()
            run_all()
            done.wait()
        except Exception as e:  # noqa: BLE001 - reported below
            errors.append(("exception", t, repr(e)))
            for bar in (warm, go, done):
                bar.abort()

    threads = [threading.Thread(target=worker, args=(t,)) for t in range(nthreads)]
    for th in threads:
        th.start()
    warm.wait()
    before = lib.vibe_c_allocations()
    go.wait()
    done.wait()
    after = lib.vibe_c_allocations()
    for th in threads:
        th.join()
    assert not errors, errors[:5]
    assert after == before, (before, after)
    a, b, c, d, xo, _, _ = cases[0][0]
    x, ws = np.zeros(n), np.zeros(n)
    for _ in range(20):
        lib.vibe_tridiagonal_solve_f64(a.ctypes.data, b.ctypes.data, c.ctypes.data, d.ctypes.data, n, x.ctypes.data,
                                       ws.ctypes.data)
    t0 = time.perf_counter()
    for _ in range(500):
        lib.vibe_tridiagonal_solve_f64(a.ctypes.data, b.ctypes.data, c.ctypes.data, d.ctypes.data, n, x.ctypes.data,
                                       ws.ctypes.data)
    print("host vibe_tridiagonal_solve_f64, n = 80: %.1f us per call" % ((time.perf_counter() - t0) / 500 * 1e6))


def test_dev_entry_points_share_no_scratch_across_streams(vg, oc):
    """The _dev forms take their scratch from the calling thread's buffer and
    order a call on one stream after the previous call on another: solves
    queued back to back on two streams, the second needing a larger scratch
    than the first (the buffer is replaced only after its last user), with a
    Neumaier sum after each, all come out right."""
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    vp, i = ctypes.c_void_p, ctypes.c_int
    f = vg.lib.vibe_tridiagonal_solve_batched_f64_dev
    f.restype, f.argtypes = i, [vp, vp, vp, vp, i, i, vp, vp, vp]
    g = vg.lib.vibe_neumaier_sum_f64_dev
    g.restype, g.argtypes = i, [vp, ctypes.c_size_t, vp, vp]
    s1, s2 = torch.cuda.Stream(dev), torch.cuda.Stream(dev)
    outs = []
    for q, (n, n_sys, st) in enumerate(((60, 2000, s1), (300, 2000, s2), (60, 20000, s1))):
        rng = np.random.default_rng(q)
        arrs = [4.0 + rng.random((n_sys, n)), -rng.random((n_sys, n - 1)), -rng.random((n_sys, n - 1)),
                rng.standard_normal((n_sys, n))]
        b, a, c, d = (torch.tensor(v, device=dev) for v in arrs)
        x = torch.zeros((n_sys, n), dtype=torch.float64, device=dev)
        assert f(a.data_ptr(), b.data_ptr(), c.data_ptr(), d.data_ptr(), n, n_sys, x.data_ptr(), None,
                 st.cuda_stream) == 0
        xs = torch.tensor(rng.standard_normal(100000), device=dev)
        out = torch.zeros(1, dtype=torch.float64, device=dev)
        assert g(xs.data_ptr(), xs.numel(), out.data_ptr(), s1.cuda_stream) == 0
        outs.append((arrs, x, xs, out))
    torch.cuda.synchronize(dev)
    for arrs, x, xs, out in outs:
        b, a, c, d = arrs
        xg = x.cpu().numpy()
        for s in (0, b.shape[0] - 1):
            _, xo = _oracle_solve(oc, a[s], b[s], c[s], d[s])
            assert np.abs(xg[s] - xo).max() <= 1e-12 * np.abs(xo).max()
        assert abs(float(out.item()) - float(np.sum(xs.cpu().numpy()))) <= 1e-10 * float(xs.abs().sum())


def test_weno5_known_answers(vg, oc):
    """test_common.cpp:188-205: exact on constants, bounded on monotone data."""
    ql, qr = vg.weno5_reconstruct(3.5, 3.5, 3.5, 3.5, 3.5)
    assert abs(ql - 3.5) <= 1e-12 and abs(qr - 3.5) <= 1e-12
    ql, qr = vg.weno5_reconstruct(0.2, -0.4, 1.1, 0.9, 2.3)
    assert -0.4 <= ql <= 2.3 and -0.4 <= qr <= 2.3
    L = oc.port_lib()
    a, b = ctypes.c_double(), ctypes.c_double()
    L.vo_weno5_reconstruct(0.2, -0.4, 1.1, 0.9, 2.3, ctypes.byref(a), ctypes.byref(b))
    assert abs(ql - a.value) <= 1e-14 and abs(qr - b.value) <= 1e-14


def test_bilinear_known_answers(vg):
    """test_common.cpp:207-226."""
    halo, nx, ny, nz = 2, 5, 4, 2
    nsx, nsy = nx + 2 * halo, ny + 2 * halo
    f = np.zeros((nz + 2 * halo, nsy, nsx))
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                f[k + halo, j + halo, i + halo] = 10.0 * i + j + 100.0 * k
    assert abs(vg.bilinear(f, halo, nsx, nsy, nz, 2.0, 1.0, 1) - 121.0) <= 1e-12
    assert abs(vg.bilinear(f, halo, nsx, nsy, nz, 1.5, 1.0, 0) - 16.0) <= 1e-12
    assert abs(vg.bilinear(f, halo, nsx, nsy, nz, -50.0, -50.0, 0) - 0.0) <= 1e-12


def test_cfl_scan_known_answers(vg):
    """test_common.cpp:228-242: linear in dt, hand value 0.02, min dz 1000."""
    nx, ny, nz = 4, 3, 3
    u = np.full(nx * ny * nz, 20.0)
    v = np.zeros_like(u)
    w = np.zeros_like(u)
    dzeta = np.array([0.05, 0.10, 0.20])
    c1, mw, mdz = vg.cfl_scan(u, v, w, dzeta, None, nx, ny, nz, 1000.0, 1000.0, 20000.0, 1.0)
    c2, _, _ = vg.cfl_scan(u, v, w, dzeta, None, nx, ny, nz, 1000.0, 1000.0, 20000.0, 2.0)
    assert abs(c2 - 2.0 * c1) <= 1e-12
    assert abs(mw - 20.0) <= 1e-12
    assert abs(mdz - 0.05 * 20000.0) <= 1e-9
    assert abs(c1 - 20.0 / 1000.0) <= 1e-12


def test_cfl_scan_matches_oracle_with_terrain(vg, oc):
    rng = np.random.default_rng(3)
    nx, ny, nz = 37, 23, 19
    n = nx * ny * nz
    u, v, w = (rng.standard_normal(n) * s for s in (15.0, 10.0, 2.0))
    dzeta = rng.random(nz) * 0.1 + 1e-3
    zs = rng.random(nx * ny) * 500.0
    r, mw, mdz = vg.cfl_scan(u, v, w, dzeta, zs, nx, ny, nz, 1000.0, 800.0, 20000.0, 6.0)
    L = oc.port_lib()
    a, b = ctypes.c_double(), ctypes.c_double()
    ro = L.vo_cfl_scan(u.ctypes.data, v.ctypes.data, w.ctypes.data, dzeta.ctypes.data, zs.ctypes.data, nx, ny, nz,
                       1000.0, 800.0, 20000.0, 6.0, ctypes.byref(a), ctypes.byref(b))
    assert r == ro and mw == a.value and mdz == b.value  # max/min are exact


def test_neumaier_cancellation(vg):
    """test_common.cpp:244-254: [1e16, 1 x 9998, -1e16] sums to 9998."""
    n = 10000
    x = np.ones(n)
    x[0] = 1e16
    x[-1] = -1e16
    assert abs(vg.neumaier_sum(x) - (n - 2)) <= 1e-6
    assert abs(vg.neumaier_sum(np.ones(1_000_000)) - 1e6) <= 1e-3  # test_gpu_precision.cpp reduce on 1e6 ones


def test_neumaier_matches_oracle(vg, oc):
    rng = np.random.default_rng(11)
    x = rng.standard_normal(3_000_017) * 10.0 ** rng.integers(-8, 8, 3_000_017)
    L = oc.port_lib()
    ref = L.vo_neumaier_sum(x.ctypes.data, x.size)
    got = vg.neumaier_sum(x)
    assert abs(got - ref) <= 1e-12 * np.abs(x).sum()
    assert vg.neumaier_sum(np.zeros(0)) == 0.0


def test_flux_advection_constant_is_zero(vg):
    """test_common.cpp:256-266."""
    nx, ny, nz = 6, 5, 4
    n = nx * ny * nz
    q, rho, u, v, w = (np.full(n, val) for val in (3.0, 1.2, 7.0, -3.0, 0.5))
    dzeta = np.array([0.05, 0.08, 0.12, 0.2])
    dq = vg.advect_scalar_flux(q, rho, u, v, w, dzeta, None, nx, ny, nz, 1000.0, 1000.0, 20000.0)
    assert np.abs(dq).max() <= 1e-10


def test_flux_advection_matches_oracle(vg, oc):
    rng = np.random.default_rng(5)
    nx, ny, nz = 33, 17, 9
    n = nx * ny * nz
    q = rng.random(n)
    rho = 1.0 + 0.1 * rng.random(n)
    u, v, w = (rng.standard_normal(n) for _ in range(3))
    dzeta = rng.random(nz) * 0.1 + 0.01
    zs = rng.random(nx * ny) * 300.0
    dq = vg.advect_scalar_flux(q, rho, u, v, w, dzeta, zs, nx, ny, nz, 900.0, 1100.0, 15000.0)
    out = np.zeros(n)
    oc.port_lib().vo_advect_scalar_flux(q.ctypes.data, rho.ctypes.data, u.ctypes.data, v.ctypes.data, w.ctypes.data,
                                        dzeta.ctypes.data, zs.ctypes.data, nx, ny, nz, 900.0, 1100.0, 15000.0,
                                        out.ctypes.data)
    assert np.abs(dq - out).max() <= 1e-12 * np.abs(out).max()


# ---- FP32 twins (the *_f32 names of c_kernels.h:15-16) -----------------------
_F = ctypes.c_float
_fp = ctypes.POINTER(ctypes.c_float)


def f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _sig(vg, name, res, args):
    fn = getattr(vg.lib, name)
    fn.restype = res
    fn.argtypes = args
    return fn


def test_f32_thomas(vg):
    """diag(1,-4,1) known answer and variable coefficients at float precision;
    singular and bad-argument codes as the FP64 form."""
    fn = _sig(vg, "vibe_tridiagonal_solve_f32", ctypes.c_int, [ctypes.c_void_p] * 4 + [ctypes.c_int] +
              [ctypes.c_void_p] * 2)
    n = 24
    j = np.arange(n)
    for a, b, c, d in ((np.ones(n - 1), np.full(n, -4.0), np.ones(n - 1), np.ones(n)),
                       (np.full(n - 1, -1.0), 4.0 + 0.1 * j, np.full(n - 1, -1.2), np.sin(0.3 * j))):
        a32, b32, c32, d32 = f32(a), f32(b), f32(c), f32(d)
        x, ws = np.zeros(n, np.float32), np.zeros(n, np.float32)
        assert fn(a32.ctypes.data, b32.ctypes.data, c32.ctypes.data, d32.ctypes.data, n, x.ctypes.data,
                  ws.ctypes.data) == 0
        A = np.diag(b) + np.diag(a, -1) + np.diag(c, 1)
        ref = np.linalg.solve(A, d)
        assert np.abs(x - ref).max() <= 1e-5 * np.abs(ref).max()
    z, one, x, ws = np.zeros(2, np.float32), np.ones(2, np.float32), np.zeros(2, np.float32), np.zeros(2, np.float32)
    assert fn(None, z.ctypes.data, None, one.ctypes.data, 2, x.ctypes.data, ws.ctypes.data) == 1
    assert fn(None, None, None, None, 2, x.ctypes.data, ws.ctypes.data) == 2


def test_f32_weno_bilinear_cfl_neumaier_flux(vg, oc):
    """Each twin against the FP64 entry point on the same (float-representable)
    inputs: relative differences at float rounding."""
    weno = _sig(vg, "vibe_weno5_reconstruct_f32", None, [_F] * 5 + [_fp, _fp])
    rng = np.random.default_rng(9)
    for _ in range(20):
        q = f32(rng.standard_normal(5)).astype(np.float64)
        l32, r32 = _F(), _F()
        weno(*[float(v) for v in q], ctypes.byref(l32), ctypes.byref(r32))
        l64, r64 = vg.weno5_reconstruct(*q)
        assert abs(l32.value - l64) <= 2e-5 * max(1.0, abs(l64)) and abs(r32.value - r64) <= 2e-5 * max(1.0, abs(r64))

    bil = _sig(vg, "vibe_bilinear_f32", _F, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                               ctypes.c_int, _F, _F, ctypes.c_int])
    halo, nx, ny, nz = 2, 7, 5, 3
    nsx, nsy = nx + 2 * halo, ny + 2 * halo
    f = f32(rng.standard_normal(nsx * nsy * (nz + 2 * halo)))
    for xi, yj, k in ((2.25, 1.5, 1), (-3.0, 9.0, 0), (5.75, 3.125, 2)):
        got = bil(f.ctypes.data, halo, nsx, nsy, nz, xi, yj, k)
        ref = vg.bilinear(f.astype(np.float64), halo, nsx, nsy, nz, xi, yj, k)
        assert abs(got - ref) <= 1e-5 * max(1.0, abs(ref))

    cfl = _sig(vg, "vibe_cfl_scan_f32", _F, [ctypes.c_void_p] * 5 + [ctypes.c_int] * 3 + [_F] * 4 + [_fp, _fp])
    nx, ny, nz = 37, 23, 19
    n = nx * ny * nz
    u, v, w = (f32(rng.standard_normal(n) * s) for s in (15.0, 10.0, 2.0))
    dzeta, zs = f32(rng.random(nz) * 0.1 + 1e-3), f32(rng.random(nx * ny) * 500.0)
    mw, mdz = _F(), _F()
    got = cfl(u.ctypes.data, v.ctypes.data, w.ctypes.data, dzeta.ctypes.data, zs.ctypes.data, nx, ny, nz, 1000.0,
              800.0, 20000.0, 6.0, ctypes.byref(mw), ctypes.byref(mdz))
    r, m64, d64 = vg.cfl_scan(*(a.astype(np.float64) for a in (u, v, w, dzeta, zs)), nx, ny, nz, 1000.0, 800.0,
                              20000.0, 6.0)
    assert abs(got - r) <= 1e-5 * r and abs(mw.value - m64) <= 1e-5 * m64 and abs(mdz.value - d64) <= 1e-5 * d64

    neu = _sig(vg, "vibe_neumaier_sum_f32", _F, [ctypes.c_void_p, ctypes.c_size_t])
    x = np.ones(10000, np.float32)
    x[0], x[-1] = 1e8, -1e8
    assert neu(x.ctypes.data, x.size) == 9998.0  # compensation recovers what a plain float sum loses
    y = f32(rng.standard_normal(1_000_003))
    assert abs(neu(y.ctypes.data, y.size) - y.astype(np.float64).sum()) <= 1e-6 * np.abs(y).sum()

    flux = _sig(vg, "vibe_advect_scalar_flux_f32", None, [ctypes.c_void_p] * 7 + [ctypes.c_int] * 3 + [_F] * 3 +
                [ctypes.c_void_p])
    nx, ny, nz = 33, 17, 9
    n = nx * ny * nz
    q, rho = f32(rng.random(n)), f32(1.0 + 0.1 * rng.random(n))
    u, v, w = (f32(rng.standard_normal(n)) for _ in range(3))
    dzeta, zs = f32(rng.random(nz) * 0.1 + 0.01), f32(rng.random(nx * ny) * 300.0)
    out = np.zeros(n, np.float32)
    flux(*(a.ctypes.data for a in (q, rho, u, v, w, dzeta, zs)), nx, ny, nz, 900.0, 1100.0, 15000.0, out.ctypes.data)
    ref = vg.advect_scalar_flux(*(a.astype(np.float64) for a in (q, rho, u, v, w, dzeta, zs)), nx, ny, nz, 900.0,
                                1100.0, 15000.0)
    assert np.abs(out - ref).max() <= 1e-4 * np.abs(ref).max()


# ---- TL / AD of the flux advection ------------------------------------------
def _adv_case(seed, nx=23, ny=17, nz=9, dtype=np.float64):
    rng = np.random.default_rng(seed)
    n = nx * ny * nz
    x = {"q": 0.5 + rng.random(n), "rho": 1.0 + 0.1 * rng.random(n), "u": rng.standard_normal(n),
         "v": rng.standard_normal(n), "w": 0.3 * rng.standard_normal(n)}
    d = {k: rng.standard_normal(n) * (0.1 if k == "rho" else 1.0) for k in x}
    dzeta = rng.random(nz) * 0.1 + 0.01
    zs = rng.random(nx * ny) * 300.0
    cast = lambda a: np.ascontiguousarray(a, dtype=dtype)
    return ({k: cast(a) for k, a in x.items()}, {k: cast(a) for k, a in d.items()}, cast(dzeta), cast(zs),
            (nx, ny, nz))


ADV = ("q", "rho", "u", "v", "w")
GEO = (900.0, 1100.0, 15000.0)


def _tl(vg, x, d, dzeta, zs, dims, f32=False):
    nx, ny, nz = dims
    out = np.zeros(nx * ny * nz, dtype=np.float32 if f32 else np.float64)
    fn = vg.lib.vibe_advect_scalar_flux_tl_f32 if f32 else vg.lib.vibe_advect_scalar_flux_tl_f64
    fn.restype = ctypes.c_int
    F = ctypes.c_float if f32 else ctypes.c_double
    fn.argtypes = [ctypes.c_void_p] * 12 + [ctypes.c_int] * 3 + [F] * 3 + [ctypes.c_void_p]
    rc = fn(*[x[k].ctypes.data for k in ADV], *[d[k].ctypes.data for k in ADV], dzeta.ctypes.data, zs.ctypes.data,
            nx, ny, nz, *GEO, out.ctypes.data)
    assert rc == 0
    return out


def _ad(vg, x, bd, dzeta, zs, dims, acc=None, f32=False):
    nx, ny, nz = dims
    n = nx * ny * nz
    dt = np.float32 if f32 else np.float64
    outs = {k: (acc[k].copy() if acc else np.zeros(n, dtype=dt)) for k in ADV}
    fn = vg.lib.vibe_advect_scalar_flux_ad_f32 if f32 else vg.lib.vibe_advect_scalar_flux_ad_f64
    fn.restype = ctypes.c_int
    F = ctypes.c_float if f32 else ctypes.c_double
    fn.argtypes = [ctypes.c_void_p] * 8 + [ctypes.c_int] * 3 + [F] * 3 + [ctypes.c_void_p] * 5
    rc = fn(*[x[k].ctypes.data for k in ADV], bd.ctypes.data, dzeta.ctypes.data, zs.ctypes.data, nx, ny, nz, *GEO,
            *[outs[k].ctypes.data for k in ADV])
    assert rc == 0
    return outs


def test_flux_advection_tl_matches_finite_differences(vg):
    """Central differences of the FP64 forward kernel (which matches the
    oracle) converge to the TL: error O(eps^2) down to rounding."""
    x, d, dzeta, zs, dims = _adv_case(1)
    nx, ny, nz = dims
    fwd = lambda xx: vg.advect_scalar_flux(*[xx[k] for k in ADV], dzeta, zs, nx, ny, nz, *GEO)
    tl = _tl(vg, x, d, dzeta, zs, dims)
    errs = []
    for eps in (1e-2, 1e-3, 1e-4):
        xp = {k: x[k] + eps * d[k] for k in ADV}
        xm = {k: x[k] - eps * d[k] for k in ADV}
        fd = (fwd(xp) - fwd(xm)) / (2 * eps)
        errs.append(np.abs(fd - tl).max() / np.abs(tl).max())
    # second order (x100 per decade of eps) until rounding takes over
    assert errs[1] <= 0.02 * errs[0] or errs[1] < 1e-9, errs
    assert min(errs) < 1e-7, errs


@pytest.mark.parametrize("dims", [(23, 17, 9), (1, 5, 4), (2, 1, 3)])
def test_flux_advection_adjoint_dot_product(vg, dims):
    """<TL dx, y> = <dx, AD y> over all five inputs (1e-12 in FP64), on
    regular, one-column-wide and two-wide periodic grids; AD accumulates."""
    x, d, dzeta, zs, dims = _adv_case(2, *dims)
    rng = np.random.default_rng(3)
    y = rng.standard_normal(x["q"].size)
    lhs = float(np.dot(_tl(vg, x, d, dzeta, zs, dims), y))
    bar = _ad(vg, x, y, dzeta, zs, dims)
    rhs = float(sum(np.dot(d[k], bar[k]) for k in ADV))
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), abs(rhs)), (lhs, rhs)
    twice = _ad(vg, x, y, dzeta, zs, dims, acc=bar)
    for k in ADV:
        assert np.allclose(twice[k], 2 * bar[k], rtol=1e-14, atol=0)


def test_flux_advection_adjoint_dot_product_f32(vg):
    x, d, dzeta, zs, dims = _adv_case(4, dtype=np.float32)
    y = np.random.default_rng(5).standard_normal(x["q"].size).astype(np.float32)
    lhs = float(np.dot(_tl(vg, x, d, dzeta, zs, dims, f32=True).astype(np.float64), y))
    bar = _ad(vg, x, y, dzeta, zs, dims, f32=True)
    rhs = float(sum(np.dot(d[k].astype(np.float64), bar[k]) for k in ADV))
    assert abs(lhs - rhs) <= 1e-5 * max(abs(lhs), abs(rhs)), (lhs, rhs)
