"""Edge cases of the C-ABI kernels, run through any library that exports them:
NULL arguments, empty and negative grids, a grid without interior points,
one-row and diagonal systems (c_kernels.c:18-60 Thomas, 64-104 WENO5,
108-144 bilinear, 148-186 CFL scan, 190-205 Neumaier, 209-260 flux
advection). The oracle, the compiled reference and the GPU library each get a
binding table (`oracle_table`, `reference_table`, `gpu_table`, each from the
library's path through a handle of its own, so the argument types it sets
touch no other test's bindings) and `run_cases` makes the same calls on
each, so their results can be compared one for one."""
import ctypes

import numpy as np

_vp, _I, _D = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
_F = ctypes.c_float
_SIGS = {  # (restype, argtypes) for the FP64 names
    "thomas": (_I, [_vp] * 4 + [_I, _vp, _vp]),
    "weno": (None, [_D] * 5 + [_vp, _vp]),
    "bilinear": (_D, [_vp, _I, _I, _I, _I, _D, _D, _I]),
    "cfl": (_D, [_vp] * 5 + [_I, _I, _I, _D, _D, _D, _D, _vp, _vp]),
    "neumaier": (_D, [_vp, ctypes.c_size_t]),
    "flux": (None, [_vp] * 7 + [_I, _I, _I, _D, _D, _D, _vp]),
}
_REF_NAMES = {"thomas": "vibe_tridiagonal_solve_f64", "weno": "vibe_weno5_reconstruct_f64",
              "bilinear": "vibe_bilinear_f64", "cfl": "vibe_cfl_scan_f64", "neumaier": "vibe_neumaier_sum_f64",
              "flux": "vibe_advect_scalar_flux_f64"}
_ORACLE_NAMES = {"thomas": "vo_tridiagonal_solve", "weno": "vo_weno5_reconstruct", "bilinear": "vo_bilinear",
                 "cfl": "vo_cfl_scan", "neumaier": "vo_neumaier_sum", "flux": "vo_advect_scalar_flux"}


def _table(path, names, dtype=np.float64):
    lib = ctypes.CDLL(path)
    t = {"dtype": dtype}
    for key, name in names.items():
        f = getattr(lib, name)
        res, args = _SIGS[key]
        if dtype == np.float32:  # the FP32 twins take and return float where the FP64 forms use double
            res = _F if res is _D else res
            args = [_F if a is _D else a for a in args]
        f.restype, f.argtypes = res, args
        t[key] = f
    return t


def oracle_table(path):
    return _table(path, _ORACLE_NAMES)


def reference_table(path):
    return _table(path, _REF_NAMES)


def gpu_table(path, f32=False):
    if not f32:
        return _table(path, _REF_NAMES)
    return _table(path, {k: v.replace("_f64", "_f32") for k, v in _REF_NAMES.items()}, np.float32)


def _p(a):
    return None if a is None else a.ctypes.data


def run_cases(t):
    """Every case's outputs, in a fixed order: return codes, scalars and the
    arrays a call writes (or leaves alone)."""
    dt = t["dtype"]
    arr = lambda v: np.ascontiguousarray(v, dtype=dt)  # noqa: E731
    out = []
    # Thomas: one row, a zero one-row pivot, n = 0, a diagonal system (a, c NULL)
    for b, d in (([2.0], [3.0]), ([0.0], [1.0])):
        b, d, x, ws = arr(b), arr(d), arr([-7.0]), arr([0.0])
        out += [t["thomas"](None, _p(b), None, _p(d), 1, _p(x), _p(ws)), x.copy()]
    b, d, x, ws = arr([1.0]), arr([1.0]), arr([-7.0]), arr([0.0])
    out += [t["thomas"](None, _p(b), None, _p(d), 0, _p(x), _p(ws)), x.copy()]
    b, d, x, ws = arr([2.0, 4.0, -8.0]), arr([1.0, 3.0, 5.0]), arr([0.0] * 3), arr([0.0] * 3)
    out += [t["thomas"](None, _p(b), None, _p(d), 3, _p(x), _p(ws)), x.copy()]
    # WENO5 with a NULL output: no write, no fault
    q = ctypes.c_double(-7.0) if dt == np.float64 else ctypes.c_float(-7.0)
    t["weno"](1.0, 2.0, 3.0, 4.0, 5.0, ctypes.addressof(q), None)
    out.append(q.value)
    # bilinear: NULL field, nz <= 0, a grid without interior points in x
    # (nsx = 2 halo) and one interior row in y, points far outside
    f = arr(np.arange(2 * 3 * 4, dtype=np.float64) * 0.5 - 3.0)  # halo 1, nsx 2, nsy 3, nz 2: 4 planes
    out.append(t["bilinear"](None, 1, 2, 3, 2, 0.5, 0.5, 0))
    out.append(t["bilinear"](_p(f), 1, 2, 3, 0, 0.5, 0.5, 0))
    out.append(t["bilinear"](_p(f), 1, 2, 3, -2, 0.5, 0.5, 0))
    for xi, yj, k in ((-1.5, -2.25, -1), (0.25, 0.75, 0), (3.7, 9.0, 1), (-0.5, 0.5, 7)):
        out.append(t["bilinear"](_p(f), 1, 2, 3, 2, xi, yj, k))
    g = arr(np.sin(np.arange(7 * 6 * 5, dtype=np.float64)))  # halo 2, 3 x 2 interior points, nz 1
    for xi, yj, k in ((-3.0, 5.5, 0), (1.25, 0.5, 0), (2.99, -0.01, 3)):
        out.append(t["bilinear"](_p(g), 2, 7, 6, 1, xi, yj, k))
    # CFL scan: NULL wind (outputs untouched), empty and negative grids
    u = arr(np.linspace(-3.0, 4.0, 8))
    dz = arr([0.1, 0.2])
    for dims, wind in (((2, 2, 2), None), ((0, 3, 2), u), ((-1, -1, 1), u), ((2, 2, 0), u), ((2, -2, 2), u)):
        mw, md = arr([-7.0]), arr([-7.0])
        r = t["cfl"](_p(wind), _p(u), _p(u), _p(dz), None, *dims, 1000.0, 1000.0, 20000.0, 5.0, _p(mw), _p(md))
        out += [r, mw.copy(), md.copy()]
    # Neumaier: NULL, n = 0
    out += [t["neumaier"](None, 5), t["neumaier"](_p(u), 0)]
    # flux advection: NULL q, empty and negative grids leave dqdt alone
    for dims, qq in (((2, 2, 2), None), ((0, 2, 2), u), ((-2, -3, 1), u), ((2, 2, -1), u)):
        dq = arr([7.0] * 8)
        t["flux"](_p(qq), _p(u), _p(u), _p(u), _p(u), _p(dz), None, *dims, 1000.0, 1000.0, 20000.0, _p(dq))
        out.append(dq.copy())
    return out


def compare(a, b, rtol=0.0):
    """Case by case: equal (bit for bit with rtol 0), NaN where the other is NaN."""
    assert len(a) == len(b)
    for n, (x, y) in enumerate(zip(a, b)):
        x, y = np.asarray(x, dtype=np.float64), np.asarray(y, dtype=np.float64)
        assert x.shape == y.shape, n
        same = (x == y) | (np.isnan(x) & np.isnan(y)) | (np.abs(x - y) <= rtol * np.abs(y))
        assert np.all(same), (n, x, y)
