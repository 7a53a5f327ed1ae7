"""The allocation-free batched Thomas solve,
vibe_tridiagonal_solve_batched_f64_dev_noalloc.

Some callers of this library cannot allocate device memory: a host model
whose own allocator has reserved the device memory and forbids any other
allocation, or a time-critical step loop in which cudaMalloc/cudaFree would
synchronise the device. This entry point serves them from a fixed device
array. The tests check that it returns the same solutions as the allocating
entry point, on two calls in a row with different systems (the array keeps
the previous call's contents), and that it refuses a request larger than the
array. Device buffers here come from torch, as a caller's own allocator
would provide them.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LIMIT = 1 << 18  # doubles in the fixed workspace (n * n_sys)


def _bind(vg):
    vp, i = ctypes.c_void_p, ctypes.c_int
    for name in ("vibe_tridiagonal_solve_batched_f64_dev_noalloc", "vibe_tridiagonal_solve_batched_f64_dev"):
        f = getattr(vg.lib, name)
        f.restype = i
        f.argtypes = [vp, vp, vp, vp, i, i, vp, vp, vp]
    return (vg.lib.vibe_tridiagonal_solve_batched_f64_dev_noalloc, vg.lib.vibe_tridiagonal_solve_batched_f64_dev)


def test_noalloc_matches_allocating_entry_point_on_two_calls(vg):
    torch = pytest.importorskip("torch")
    noalloc, alloc = _bind(vg)
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev).cuda_stream
    for n, n_sys, seed in ((80, 3000, 1), (57, 4111, 2)):
        assert n * n_sys <= LIMIT
        rng = np.random.default_rng(seed)
        b = torch.tensor(4.0 + rng.random((n_sys, n)), device=dev)
        a = torch.tensor(-rng.random((n_sys, n - 1)), device=dev)
        c = torch.tensor(-rng.random((n_sys, n - 1)), device=dev)
        d = torch.tensor(rng.standard_normal((n_sys, n)), device=dev)
        x_ref = torch.full((n_sys, n), float("nan"), dtype=torch.float64, device=dev)
        x_na = torch.full((n_sys, n), float("nan"), dtype=torch.float64, device=dev)
        st_ref = torch.full((n_sys,), -1, dtype=torch.int32, device=dev)
        st_na = torch.full((n_sys,), -1, dtype=torch.int32, device=dev)
        args = [t.data_ptr() for t in (a, b, c, d)]
        assert alloc(*args, n, n_sys, x_ref.data_ptr(), st_ref.data_ptr(), stream) == 0
        assert noalloc(*args, n, n_sys, x_na.data_ptr(), st_na.data_ptr(), stream) == 0
        torch.cuda.synchronize(dev)
        assert int(st_ref.abs().sum()) == 0 and int(st_na.abs().sum()) == 0
        scale = float(x_ref.abs().max())
        assert float((x_na - x_ref).abs().max()) <= 1e-12 * scale


def test_noalloc_rejects_requests_beyond_its_workspace(vg):
    torch = pytest.importorskip("torch")
    noalloc, _ = _bind(vg)
    dev = torch.device("cuda", 0)
    buf = torch.zeros(16, dtype=torch.float64, device=dev)
    p = buf.data_ptr()
    n, n_sys = 80, LIMIT // 80 + 1  # one system too many; rejected before any launch
    rc = noalloc(p, p, p, p, n, n_sys, p, None, torch.cuda.current_stream(dev).cuda_stream)
    assert rc == 2
    assert b"exceeds the fixed workspace" in vg.lib.vibe_c_last_error()


def test_noalloc_tall_systems_and_null_status(vg):
    """n > 128: this form runs the one-thread sweep where the allocating form
    runs the warp-per-system solver, so the two agree to rounding; a call
    without a status array (status = NULL) solves the same."""
    torch = pytest.importorskip("torch")
    noalloc, alloc = _bind(vg)
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev).cuda_stream
    n, n_sys = 300, 800
    assert n * n_sys <= LIMIT
    rng = np.random.default_rng(3)
    b = torch.tensor(4.0 + rng.random((n_sys, n)), device=dev)
    a = torch.tensor(-rng.random((n_sys, n - 1)), device=dev)
    c = torch.tensor(-rng.random((n_sys, n - 1)), device=dev)
    d = torch.tensor(rng.standard_normal((n_sys, n)), device=dev)
    args = [t.data_ptr() for t in (a, b, c, d)]
    x_ref = torch.full((n_sys, n), float("nan"), dtype=torch.float64, device=dev)
    x_na = torch.full((n_sys, n), float("nan"), dtype=torch.float64, device=dev)
    x_nul = torch.full((n_sys, n), float("nan"), dtype=torch.float64, device=dev)
    st = torch.full((n_sys,), -1, dtype=torch.int32, device=dev)
    assert alloc(*args, n, n_sys, x_ref.data_ptr(), None, stream) == 0
    assert noalloc(*args, n, n_sys, x_na.data_ptr(), st.data_ptr(), stream) == 0
    assert noalloc(*args, n, n_sys, x_nul.data_ptr(), None, stream) == 0
    torch.cuda.synchronize(dev)
    assert int(st.abs().sum()) == 0
    scale = float(x_ref.abs().max())
    assert float((x_na - x_ref).abs().max()) <= 1e-12 * scale
    assert torch.equal(x_na, x_nul)
