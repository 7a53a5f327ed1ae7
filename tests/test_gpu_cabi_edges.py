"""Edge cases of the GPU C-ABI kernels (include/vibe_c_kernels.h) against the
oracle: NULL arguments, empty and negative grids, a grid without interior
points, one-row and diagonal systems (tests/cabi_edge_cases.py, whose oracle
results match the compiled reference's c_kernels.c bit for bit), the
device-pointer forms on empty and negative grids, and a batch with a singular
system, whose x stays as it was."""
import ctypes

import numpy as np
import pytest

import cabi_edge_cases as ce

pytestmark = pytest.mark.gpu

_vp, _I, _D = ctypes.c_void_p, ctypes.c_int, ctypes.c_double


def test_host_forms_match_the_oracle(vg, oc):
    want = ce.run_cases(ce.oracle_table(oc.PORT_SO))
    # FP64: the same values (the bilinear weights to rounding of a contracted multiply-add)
    ce.compare(ce.run_cases(ce.gpu_table(vg.lib._name)), want, rtol=1e-14)
    # FP32 twins: the same cases on float inputs
    ce.compare(ce.run_cases(ce.gpu_table(vg.lib._name, f32=True)), want, rtol=1e-5)


def test_device_forms_on_empty_and_negative_grids(vg):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    lib = ctypes.CDLL(vg.lib._name)
    cfl = lib.vibe_cfl_scan_f64_dev
    cfl.restype, cfl.argtypes = _I, [_vp] * 5 + [_I, _I, _I, _D, _D, _D, _D, _vp, _vp]
    flux = lib.vibe_advect_scalar_flux_f64_dev
    flux.restype, flux.argtypes = _I, [_vp] * 7 + [_I, _I, _I, _D, _D, _D, _vp, _vp]
    neu = lib.vibe_neumaier_sum_f64_dev
    neu.restype, neu.argtypes = _I, [_vp, ctypes.c_size_t, _vp, _vp]
    weno = lib.vibe_weno5_reconstruct_batched_f64_dev
    weno.restype, weno.argtypes = _I, [_vp, ctypes.c_size_t, _vp, _vp, _vp]
    thomas = lib.vibe_tridiagonal_solve_batched_f64_dev
    thomas.restype, thomas.argtypes = _I, [_vp] * 4 + [_I, _I, _vp, _vp, _vp]
    st = torch.cuda.current_stream(dev).cuda_stream
    one = torch.ones(8, dtype=torch.float64, device=dev)
    p = one.data_ptr()
    out3 = torch.full((3,), -7.0, dtype=torch.float64, device=dev)
    assert cfl(p, p, p, p, None, 0, 3, 2, 1e3, 1e3, 2e4, 5.0, out3.data_ptr(), st) == 0
    torch.cuda.synchronize(dev)
    assert out3.tolist() == [0.0, 0.0, 0.0]  # no cells: (0, 0, 0) as the host form
    assert cfl(p, p, p, p, None, -1, 3, 2, 1e3, 1e3, 2e4, 5.0, out3.data_ptr(), st) == 2
    dq = torch.full((8,), 7.0, dtype=torch.float64, device=dev)
    assert flux(p, p, p, p, p, p, None, 0, 2, 2, 1e3, 1e3, 2e4, dq.data_ptr(), st) == 0
    assert flux(p, p, p, p, p, p, None, -2, -3, 1, 1e3, 1e3, 2e4, dq.data_ptr(), st) == 2
    s = torch.full((1,), -7.0, dtype=torch.float64, device=dev)
    assert neu(p, 0, s.data_ptr(), st) == 0
    assert weno(p, 0, p, p, st) == 0
    assert thomas(p, p, p, p, 4, 0, p, None, st) == 0
    assert thomas(p, p, p, p, 0, 1, p, None, st) == 2
    torch.cuda.synchronize(dev)
    assert s.item() == 0.0 and bool((dq == 7.0).all()) and bool((one == 1.0).all())


@pytest.mark.parametrize("n", [1, 5, 200])
def test_batch_with_a_singular_system_leaves_its_x(vg, oc, n):
    """Systems 0 and 2 solve; system 1 has a zero pivot (b[0] = 0, or a zero
    pivot after elimination): the call returns VIBE_C_ERR_SINGULAR, x of the
    solved systems is the oracle's and system 1's x is as it was."""
    rng = np.random.default_rng(n)
    n_sys = 3
    b = 4.0 + rng.random((n_sys, n))
    a, c = -rng.random((n_sys, max(n - 1, 1))), -rng.random((n_sys, max(n - 1, 1)))
    d = rng.standard_normal((n_sys, n))
    if n == 1:
        b[1, 0] = 0.0
    else:  # row 1 of system 1: b[1] - a[0] c[0] / b[0] = 2 - 4 (1 / 2) = 0, exactly
        b[1, 0], c[1, 0], a[1, 0], b[1, 1] = 2.0, 1.0, 4.0, 2.0
    a, c = a[:, :n - 1].copy(), c[:, :n - 1].copy()
    x = np.full((n_sys, n), -7.0)
    lib = vg.lib
    rc = lib.vibe_tridiagonal_solve_batched_f64(a.ctypes.data, b.ctypes.data, c.ctypes.data, d.ctypes.data, n, n_sys,
                                                x.ctypes.data)
    assert rc == 1
    assert np.all(x[1] == -7.0)
    L = oc.port_lib()
    for s in (0, 2):
        xo, ws = np.zeros(n), np.zeros(n)
        assert L.vo_tridiagonal_solve(a[s].ctypes.data if n > 1 else None, b[s].ctypes.data,
                                      c[s].ctypes.data if n > 1 else None, d[s].ctypes.data, n, xo.ctypes.data,
                                      ws.ctypes.data) == 0
        assert np.abs(x[s] - xo).max() <= 1e-12 * np.abs(xo).max()
