"""Nest transfers on the GPU (include/vibe_nest.h) against the oracle's
restatement of grid::Nest (src/grid/nest.cpp:34-124): bit for bit."""
import numpy as np
import pytest

import nest_cases as nc

pytestmark = pytest.mark.gpu


def placement(vg, pl):
    q = vg.NestPlacement()
    for k, v in pl.items():
        setattr(q, k, v)
    return q


@pytest.mark.parametrize("case", range(len(nc.CASES)))
def test_nest_transfers_bit_exact(vg, oc, case):
    pdims, cdims, pl = nc.CASES[case]
    q = placement(vg, pl)
    assert np.array_equal(vg.davies_profile(pl["boundary_zone"]), oc.davies_profile(pl["boundary_zone"]))
    parent = nc.fields(oc, pdims, 1)
    res = {}
    for side in ("gpu", "port"):
        child = nc.fields(oc, cdims, 2)
        inner = nc.fields(oc, cdims, 3)
        par = [p.copy() for p in parent]
        if side == "gpu":
            vg.nest_interpolate_from_parent(q, nc.STAGGERS, pdims, parent, cdims, child)
            interp = [c.copy() for c in child]
            vg.nest_apply_lateral_boundary(q, nc.STAGGERS, cdims, inner, interp)
            vg.nest_restrict_to_parent(q, nc.STAGGERS, cdims, inner, pdims, par)
        else:
            oc.nest_interpolate_from_parent(pl, nc.STAGGERS, pdims, parent, cdims, child)
            interp = [c.copy() for c in child]
            oc.nest_apply_lateral_boundary(pl, nc.STAGGERS, cdims, inner, interp)
            oc.nest_restrict_to_parent(pl, nc.STAGGERS, cdims, inner, pdims, par)
        res[side] = (interp, inner, par)
    for a, b in zip(res["gpu"], res["port"]):
        for x, y in zip(a, b):
            assert np.array_equal(x, y)


def test_nest_device_form_many_fields(vg, oc):
    """The _dev form on device arrays, 20 fields in one call (two launches
    of up to 16 fields each)."""
    torch = pytest.importorskip("torch")
    import ctypes
    pdims, cdims, pl = nc.CASES[0]
    q = placement(vg, pl)
    st = [nc.STAGGERS[v % 7] for v in range(20)]
    rng = np.random.default_rng(5)
    parent = [rng.standard_normal(oc.fieldt_size(*pdims, s)) for s in st]
    child = [rng.standard_normal(oc.fieldt_size(*cdims, s)) for s in st]
    dp = [torch.tensor(a, device="cuda") for a in parent]
    dc = [torch.tensor(a, device="cuda") for a in child]
    sta = np.ascontiguousarray(st, dtype=np.int32)
    ptrs = lambda ts: (ctypes.c_void_p * len(ts))(*[t.data_ptr() for t in ts])
    rc = vg.lib.vibe_nest_interpolate_from_parent_dev(ctypes.byref(q), 20, sta.ctypes.data, *pdims, ptrs(dp), *cdims,
                                                      ptrs(dc), torch.cuda.current_stream().cuda_stream)
    assert rc == 0
    torch.cuda.synchronize()
    oc.nest_interpolate_from_parent(pl, st, pdims, parent, cdims, child)
    for a, b in zip(dc, child):
        assert np.array_equal(a.cpu().numpy(), b)


def test_nest_rejects_bad_placements(vg, oc):
    pdims, cdims, pl = nc.CASES[0]
    parent = nc.fields(oc, pdims, 1)
    child = nc.fields(oc, cdims, 2)
    for bad in (dict(pl, ratio=1), dict(pl, boundary_zone=0), dict(pl, i0=pdims[0])):
        with pytest.raises(RuntimeError):
            vg.nest_restrict_to_parent(placement(vg, bad), nc.STAGGERS, cdims, child, pdims, [p.copy() for p in parent])
