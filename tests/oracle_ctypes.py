"""ctypes view of the CPU oracle (oracle/vibe_oracle.h) for the tests.

Two interchangeable back ends share one interface:
  * ``port``: oracle/liboracle.so, the plain-C restatement of the reference
    step (builds anywhere);
  * ``ref``: oracle/_ref/libvibe_ref.so, the reference's own sources compiled
    unchanged plus a thin driver (only where the reference tree was present
    at build time).
This module is test infrastructure: nothing on the product path imports it.
"""
import ctypes
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
PORT_SO = os.path.join(ORACLE_DIR, "liboracle.so")
REF_SO = os.path.join(ORACLE_DIR, "_ref", "libvibe_ref.so")

SPECIES = ["u", "v", "w", "rho", "theta", "pi", "qv", "qc", "qr", "qi", "qs", "qg"]
NSPECIES = 12
HALO = 4
REFFIELDS = ["theta0", "pi0", "rho0", "p0", "qv0"]

_D, _I = ctypes.c_double, ctypes.c_int


class Setup(ctypes.Structure):
    """Mirror of ``vo_setup`` (same field order)."""

    _fields_ = [
        ("nx", _I), ("ny", _I), ("nz", _I),
        ("dx", _D), ("dy", _D), ("z_top", _D),
        ("zeta_first", _D), ("zeta_stretch", _D),
        ("terrain_kind", _I), ("hill_h", _D), ("hill_a", _D), ("hill_xc", _D), ("hill_yc", _D),
        ("ref_kind", _I), ("theta0", _D), ("p_surf", _D), ("bv_n", _D), ("profile_dz", _D),
        ("bubble_amplitude", _D), ("bubble_radius_x", _D), ("bubble_radius_z", _D),
        ("bubble_xc", _D), ("bubble_yc", _D), ("bubble_zc", _D),
        ("qv_surface", _D), ("qv_decay_height", _D),
        ("u_background", _D), ("shear_u", _D),
        ("advection", _I), ("weno_scalars", _I), ("moist", _I),
        ("coriolis", _I), ("latitude", _D),
        ("sponge_alpha", _D), ("sponge_start_fraction", _D),
        ("divergence_damping", _D), ("divergence_order", _I),
        ("pgf_perturbation", _I), ("acoustic_mode", _I), ("hevi_beta", _D),
        ("split_fast", _I), ("weno_advective", _I), ("w_rigid", _I),
    ]

    def copy(self, **kw):
        s = Setup()
        ctypes.pointer(s)[0] = self
        for k, v in kw.items():
            setattr(s, k, v)
        return s


def storage_shape(setup, species):
    """(nsz, nsy, nsx) of a species' halo'd storage (field.hpp:40-53)."""
    h2 = 2 * HALO
    return (setup.nz + h2 + (species == 2), setup.ny + h2 + (species == 1),
            setup.nx + h2 + (species == 0))


def interior(setup, species, arr):
    """View of the interior points incl. the extra face (State::pack order)."""
    a = arr.reshape(storage_shape(setup, species))
    nx, ny, nz = setup.nx, setup.ny, setup.nz
    return a[HALO:HALO + nz + (species == 2), HALO:HALO + ny + (species == 1),
             HALO:HALO + nx + (species == 0)]


_libs = {}


def _load(kind):
    if kind in _libs:
        return _libs[kind]
    path = PORT_SO if kind == "port" else REF_SO
    lib = ctypes.CDLL(path)
    p = "vo_" if kind == "port" else "vref_"
    vp = ctypes.c_void_p
    dp = ctypes.POINTER(ctypes.c_double)
    sig = {
        "create": (vp, [ctypes.POINTER(Setup)]),
        "destroy": (None, [vp]),
        "storage_size": (ctypes.c_size_t, [vp, _I]),
        "get_field": (None, [vp, _I, vp]),
        "set_field": (None, [vp, _I, vp]),
        "get_reffield": (None, [vp, _I, vp]),
        "get_zeta": (None, [vp, vp]),
        "get_terrain": (None, [vp, vp]),
        "get_sponge": (None, [vp, vp]),
        "rk3_step": (_I, [vp, _D, _I]),
        "slow_tendency": (None, [vp, ctypes.POINTER(dp)]),
        "acoustic_substep": (None, [vp, _D]),
        "hevi_substep": (None, [vp, _D]),
        "sponge": (None, [vp, _D]),
        "helmholtz_solve": (_I, [vp, _I, _I, _D, _I, vp, vp, vp, vp, ctypes.POINTER(_I), dp]),
        "multigrid_restrict": (None, [vp, vp, vp]),
        "multigrid_prolong": (None, [vp, vp, vp]),
        "si_step": (_I, [vp, _D, _I, _I, _D, ctypes.POINTER(_I), dp, vp, vp, vp]),
        "write_restart": (_I, [vp, ctypes.c_char_p, _D, _I]),
        "read_restart": (_I, [vp, ctypes.c_char_p, dp, ctypes.POINTER(_I)]),
        "energy_budget": (None, [vp, dp]),
    }
    if kind == "port":
        sig["helmholtz_apply"] = (None, [vp, vp, vp, vp, vp])
        sig["helmholtz_residual_l2"] = (_D, [vp, vp, vp, vp, vp])
    else:
        sig["helmholtz_apply_norm"] = (None, [vp, vp, vp, vp, vp, dp])
    fns = {}
    for name, (res, args) in sig.items():
        f = getattr(lib, p + name)
        f.restype = res
        f.argtypes = args
        fns[name] = f
    if kind == "port":
        lib.vo_setup_defaults.argtypes = [ctypes.POINTER(Setup)]
        lib.vo_setup_defaults.restype = None
        lib.vo_tridiagonal_solve.restype = _I
        lib.vo_tridiagonal_solve.argtypes = [vp, vp, vp, vp, _I, vp, vp]
        lib.vo_weno5_reconstruct.restype = None
        lib.vo_weno5_reconstruct.argtypes = [_D, _D, _D, _D, _D, dp, dp]
        lib.vo_bilinear.restype = _D
        lib.vo_bilinear.argtypes = [vp, _I, _I, _I, _I, _D, _D, _I]
        lib.vo_cfl_scan.restype = _D
        lib.vo_cfl_scan.argtypes = [vp, vp, vp, vp, vp, _I, _I, _I, _D, _D, _D, _D, dp, dp]
        lib.vo_neumaier_sum.restype = _D
        lib.vo_neumaier_sum.argtypes = [vp, ctypes.c_size_t]
        lib.vo_advect_scalar_flux.restype = None
        lib.vo_advect_scalar_flux.argtypes = [vp] * 7 + [_I, _I, _I, _D, _D, _D, vp]
    _libs[kind] = (lib, fns)
    return _libs[kind]


def port_lib():
    return _load("port")[0]


def ref_available():
    return os.path.exists(REF_SO)


def defaults():
    """Config-1 warm bubble (64x64x40, dx=dy=dz=250 m, theta0=300 K)."""
    s = Setup()
    port_lib().vo_setup_defaults(ctypes.byref(s))
    return s


class Model:
    """One oracle model instance (``kind`` = 'port' or 'ref')."""

    def __init__(self, setup, kind="port"):
        self.kind = kind
        self.setup = setup.copy()
        self._lib, self._f = _load(kind)
        self.h = self._f["create"](ctypes.byref(self.setup))

    def close(self):
        if self.h:
            self._f["destroy"](self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def size(self, sp):
        return int(self._f["storage_size"](self.h, sp))

    def get(self, sp):
        a = np.empty(self.size(sp))
        self._f["get_field"](self.h, sp, a.ctypes.data)
        return a

    def set(self, sp, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64).ravel()
        assert a.size == self.size(sp)
        self._f["set_field"](self.h, sp, a.ctypes.data)

    def state(self):
        return [self.get(sp) for sp in range(NSPECIES)]

    def set_state(self, st):
        for sp, a in enumerate(st):
            self.set(sp, a)

    def reffield(self, which):
        a = np.empty(self.size(3))
        self._f["get_reffield"](self.h, which, a.ctypes.data)
        return a

    def zeta(self):
        a = np.empty(self.setup.nz + 1)
        self._f["get_zeta"](self.h, a.ctypes.data)
        return a

    def terrain(self):
        a = np.empty(self.setup.nx * self.setup.ny)
        self._f["get_terrain"](self.h, a.ctypes.data)
        return a

    def sponge_profile(self):
        a = np.empty(self.setup.nz)
        self._f["get_sponge"](self.h, a.ctypes.data)
        return a

    def rk3_step(self, dt, n_sub):
        return int(self._f["rk3_step"](self.h, dt, n_sub))

    def slow_tendency(self):
        outs = [np.empty(self.size(sp)) for sp in range(NSPECIES)]
        ptrs = (ctypes.POINTER(ctypes.c_double) * NSPECIES)(
            *[o.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) for o in outs])
        self._f["slow_tendency"](self.h, ptrs)
        return outs

    def acoustic_substep(self, dtau):
        self._f["acoustic_substep"](self.h, dtau)

    def hevi_substep(self, dtau):
        self._f["hevi_substep"](self.h, dtau)

    def sponge(self, dt):
        self._f["sponge"](self.h, dt)

    # ---- Helmholtz family and the semi-implicit step ----
    def _cell(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64).ravel()
        assert a.size == self.size(3)
        return a

    def helmholtz_apply(self, a, b, x):
        a, b, x = self._cell(a), self._cell(b), self._cell(x)
        y = np.zeros(self.size(3))
        self._f["helmholtz_apply"](self.h, a.ctypes.data, b.ctypes.data, x.ctypes.data, y.ctypes.data)
        return y

    def helmholtz_residual_l2(self, a, b, f, x):
        a, b, f, x = self._cell(a), self._cell(b), self._cell(f), self._cell(x)
        if self.kind == "port":
            return float(self._f["helmholtz_residual_l2"](self.h, a.ctypes.data, b.ctypes.data, f.ctypes.data,
                                                          x.ctypes.data))
        out = ctypes.c_double()
        self._f["helmholtz_apply_norm"](self.h, a.ctypes.data, b.ctypes.data, f.ctypes.data, x.ctypes.data,
                                        ctypes.byref(out))
        return out.value

    def helmholtz_solve(self, kind, max_iter, tol, a, b, f, refine=1):
        """Returns (x, iterations, residual, rc)."""
        a, b, f = self._cell(a), self._cell(b), self._cell(f)
        x = np.zeros(self.size(3))
        it, res = _I(), _D()
        rc = self._f["helmholtz_solve"](self.h, kind, max_iter, tol, refine, a.ctypes.data, b.ctypes.data,
                                        f.ctypes.data, x.ctypes.data, ctypes.byref(it), ctypes.byref(res))
        return x, it.value, res.value, int(rc)

    def multigrid_restrict(self, fine):
        fine = self._cell(fine)
        out = np.zeros(self.size(3))
        self._f["multigrid_restrict"](self.h, fine.ctypes.data, out.ctypes.data)
        return out

    def multigrid_prolong(self, coarse):
        coarse = self._cell(coarse)
        out = np.zeros(self.size(3))
        self._f["multigrid_prolong"](self.h, coarse.ctypes.data, out.ctypes.data)
        return out

    def si_step(self, dt, kind=1, max_iter=200, tol=1e-8):
        """One O-SI step. Returns (rc, iterations, residual, pi_new, rhs, a_coef)."""
        outs = [np.zeros(self.size(3)) for _ in range(3)]
        it, res = _I(), _D()
        rc = self._f["si_step"](self.h, dt, kind, max_iter, tol, ctypes.byref(it), ctypes.byref(res),
                                *[o.ctypes.data for o in outs])
        return int(rc), it.value, res.value, outs[0], outs[1], outs[2]


# ---- nest transfers (port: vo_*, reference-linked: vref_*) ----
class NestPlacement(ctypes.Structure):
    _fields_ = [("i0", _I), ("j0", _I), ("k0", _I), ("iext", _I), ("jext", _I), ("ratio", _I),
                ("boundary_zone", _I)]


def _nest_fns(kind):
    lib = _load(kind)[0]
    p = "vo_" if kind == "port" else "vref_"
    vp = ctypes.c_void_p
    f = {}
    for name, args in (("nest_interpolate_from_parent", [vp, _I, vp, _I, _I, _I, vp, _I, _I, _I, vp]),
                       ("nest_restrict_to_parent", [vp, _I, vp, _I, _I, _I, vp, _I, _I, _I, vp]),
                       ("nest_apply_lateral_boundary", [vp, _I, vp, _I, _I, _I, vp, vp]),
                       ("davies_profile", [_I, _D, vp])):
        fn = getattr(lib, p + name)
        fn.restype = None
        fn.argtypes = args
        f[name] = fn
    return f


def _arr(arrs):
    return (ctypes.c_void_p * len(arrs))(*[a.ctypes.data for a in arrs])


def _pl(pl):
    q = NestPlacement()
    for name, _ in NestPlacement._fields_:
        setattr(q, name, int(pl.get(name, 0)))
    return q


def davies_profile(n_zone, alpha_max=1.0, kind="port"):
    out = np.zeros(n_zone)
    _nest_fns(kind)["davies_profile"](n_zone, alpha_max, out.ctypes.data)
    return out


def nest_interpolate_from_parent(pl, staggers, pdims, parent, cdims, child, kind="port"):
    st = np.ascontiguousarray(staggers, dtype=np.int32)
    q = _pl(pl)
    _nest_fns(kind)["nest_interpolate_from_parent"](ctypes.byref(q), len(st), st.ctypes.data, *pdims, _arr(parent),
                                                    *cdims, _arr(child))
    return child


def nest_restrict_to_parent(pl, staggers, cdims, child, pdims, parent, kind="port"):
    st = np.ascontiguousarray(staggers, dtype=np.int32)
    q = _pl(pl)
    _nest_fns(kind)["nest_restrict_to_parent"](ctypes.byref(q), len(st), st.ctypes.data, *cdims, _arr(child),
                                               *pdims, _arr(parent))
    return parent


def nest_apply_lateral_boundary(pl, staggers, cdims, child, parent_interp, kind="port"):
    st = np.ascontiguousarray(staggers, dtype=np.int32)
    q = _pl(pl)
    _nest_fns(kind)["nest_apply_lateral_boundary"](ctypes.byref(q), len(st), st.ctypes.data, *cdims, _arr(child),
                                                   _arr(parent_interp))
    return child


def fieldt_size(nx, ny, nz, stagger):
    return (nx + 2 * HALO + (stagger == 1)) * (ny + 2 * HALO + (stagger == 2)) * (nz + 2 * HALO + (stagger == 3))


# ---- TL/AD (port: vo_*, reference-linked: vref_*) ----
def _tlad_fns(kind):
    lib = _load(kind)[0]
    p = "vo_" if kind == "port" else "vref_"
    vp = ctypes.c_void_p
    f = {}
    names = [("tl_step", [vp, vp, vp, _D, vp]), ("ad_step", [vp, vp, vp, _D, vp])]
    if kind == "port":
        names += [("tl_tendency", [vp, vp, vp, vp]), ("ad_tendency", [vp, vp, vp, vp]),
                  ("nl_step", [vp, vp, vp, _D, vp]), ("nl_tendency", [vp, vp, vp, vp])]
    else:
        names += [("tl_propagate", [vp, vp, vp, _D, _I, vp]), ("ad_propagate", [vp, vp, vp, _D, _I, vp])]
    for name, args in names:
        fn = getattr(lib, p + name)
        fn.restype = None
        fn.argtypes = args
        f[name] = fn
    return f


def _arr12(arrs):
    return (ctypes.c_void_p * 12)(*[a.ctypes.data for a in arrs])


def _tl_call(model, name, *args):
    return _tlad_fns(model.kind)[name](model.h, *args)


def tl_tendency(model, xb, dx):
    d = [np.zeros(model.size(sp)) for sp in range(12)]
    _tl_call(model, "tl_tendency", _arr12(xb), _arr12(dx), _arr12(d))
    return d


def ad_tendency(model, xb, bar_d):
    bx = [np.zeros(model.size(sp)) for sp in range(12)]
    _tl_call(model, "ad_tendency", _arr12(xb), _arr12(bar_d), _arr12(bx))
    return bx


def tl_step(model, xb, dx, dt):
    out = [np.zeros(model.size(sp)) for sp in range(12)]
    _tl_call(model, "tl_step", _arr12(xb), _arr12(dx), dt, _arr12(out))
    return out


def nl_tendency(model, xb, x):
    d = [np.zeros(model.size(sp)) for sp in range(12)]
    _tl_call(model, "nl_tendency", _arr12(xb), _arr12(x), _arr12(d))
    return d


def nl_step(model, xb, x, dt):
    out = [np.zeros(model.size(sp)) for sp in range(12)]
    _tl_call(model, "nl_step", _arr12(xb), _arr12(x), dt, _arr12(out))
    return out


def ad_step(model, xb, bar_out, dt):
    out = [np.zeros(model.size(sp)) for sp in range(12)]
    _tl_call(model, "ad_step", _arr12(xb), _arr12(bar_out), dt, _arr12(out))
    return out


def tl_propagate(model, xb, dx0, dt, n):
    """Port: n frozen-base TL steps; reference: TangentLinearModel::propagate."""
    if model.kind == "ref":
        out = [np.zeros(model.size(sp)) for sp in range(12)]
        _tl_call(model, "tl_propagate", _arr12(xb), _arr12(dx0), dt, n, _arr12(out))
        return out
    cur = [a.copy() for a in dx0]
    for _ in range(n):
        cur = tl_step(model, xb, cur, dt)
    return cur


def ad_propagate(model, xb, dy, dt, n):
    """Port: n frozen-base AD steps; reference: propagate_with_trajectory over
    the trajectory record_trajectory stores."""
    if model.kind == "ref":
        out = [np.zeros(model.size(sp)) for sp in range(12)]
        _tl_call(model, "ad_propagate", _arr12(xb), _arr12(dy), dt, n, _arr12(out))
        return out
    cur = [a.copy() for a in dy]
    for _ in range(n):
        cur = ad_step(model, xb, cur, dt)
    return cur


def cfl(model, dt, dtau):
    """(cfl_number, max_sound_speed, acoustic_cfl) of the model's state."""
    lib = _load(model.kind)[0]
    f = getattr(lib, ("vo_" if model.kind == "port" else "vref_") + "cfl")
    f.restype = None
    f.argtypes = [ctypes.c_void_p, _D, _D, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    out = [ctypes.c_double() for _ in range(3)]
    f(model.h, dt, dtau, *[ctypes.byref(o) for o in out])
    return tuple(o.value for o in out)


def max_stable_dt(model):
    lib = _load(model.kind)[0]
    f = getattr(lib, ("vo_" if model.kind == "port" else "vref_") + "max_stable_dt")
    f.restype = _D
    f.argtypes = [ctypes.c_void_p]
    return f(model.h)


# ---- .vibebin restart files (io::write_restart / read_restart) ----
def write_restart(model, path, time=0.0, step=0):
    return model._f["write_restart"](model.h, os.fsencode(path), time, step)


def read_restart(model, path):
    t, n = ctypes.c_double(), ctypes.c_int()
    rc = model._f["read_restart"](model.h, os.fsencode(path), ctypes.byref(t), ctypes.byref(n))
    return rc, t.value, n.value


def energy_budget(model):
    """{kinetic, internal, potential, latent, total, mass} (dyn::energy_budget)."""
    out = (ctypes.c_double * 6)()
    model._f["energy_budget"](model.h, out)
    return dict(zip(("kinetic", "internal", "potential", "latent", "total", "mass"), out))


# ---- Kessler warm rain (KesslerMicrophysics::step_column, PhysicsDriver's microphysics step) ----
class Kessler(ctypes.Structure):
    """Mirror of vo_kessler (PhysicsOptions' Kessler fields)."""
    _fields_ = [("qc0", _D), ("k1", _D), ("k2", _D), ("evap_coef", _D), ("rain_a", _D), ("rain_b", _D),
                ("positive_definite", _I), ("exner_offset", _I)]

    @classmethod
    def defaults(cls, **kw):
        k = cls()
        lib = port_lib()
        lib.vo_kessler_defaults.argtypes = [ctypes.POINTER(Kessler)]
        lib.vo_kessler_defaults.restype = None
        lib.vo_kessler_defaults(ctypes.byref(k))
        for name, v in kw.items():
            setattr(k, name, v)
        return k


def kessler_column(k, dt, z, p, rho, theta, qv, qc, qr, kind="port"):
    """One column step; returns (theta, qv, qc, qr, precipitation rate)."""
    lib = _load(kind)[0]
    f = getattr(lib, "vo_kessler_column" if kind == "port" else "vref_kessler_column")
    vp = ctypes.c_void_p
    f.argtypes = [ctypes.POINTER(Kessler), _I, _D] + [vp] * 7
    f.restype = _D
    arrs = [np.ascontiguousarray(a, dtype=np.float64).copy() for a in (z, p, rho, theta, qv, qc, qr)]
    pr = f(ctypes.byref(k), len(arrs[0]), dt, *[a.ctypes.data for a in arrs])
    return arrs[3], arrs[4], arrs[5], arrs[6], pr


def kessler_tendency(model, k, dt):
    """PhysicsTendency of the microphysics step: [theta, qv, qc, qr] rates (cell FieldT storage)."""
    lib = model._lib
    dp = ctypes.POINTER(ctypes.c_double)
    lib.vo_kessler_tendency.argtypes = [ctypes.c_void_p, ctypes.POINTER(Kessler), _D, ctypes.POINTER(dp)]
    lib.vo_kessler_tendency.restype = None
    outs = [np.zeros(model.size(3)) for _ in range(4)]
    arr = (dp * 4)(*[o.ctypes.data_as(dp) for o in outs])
    lib.vo_kessler_tendency(model.h, ctypes.byref(k), dt, arr)
    return outs


def set_physics_kessler(model, k):
    lib = model._lib
    lib.vo_set_physics_kessler.argtypes = [ctypes.c_void_p, ctypes.POINTER(Kessler)]
    lib.vo_set_physics_kessler.restype = None
    lib.vo_set_physics_kessler(model.h, ctypes.byref(k) if k is not None else None)
