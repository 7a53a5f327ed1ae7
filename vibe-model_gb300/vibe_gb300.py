"""Python host binding of libvibe_gb300.so (include/vibe_gb300.h,
include/vibe_c_kernels.h).

Mirrors the reference's stepper interface for this path:
``Model`` ~ RungeKutta3Integrator + the State it advances
(include/vibe/time/runge_kutta.hpp:46-80, include/vibe/dyn/state.hpp:98-166),
``Model.step(dt, n_sub)`` ~ ``Integrator::step(State&, StepContext)``
(include/vibe/time/integrator.hpp:65), fields exchanged in the reference's
halo'd FieldT storage layout. Failures raise, as the reference's
NumericalError / VIBE_CHECK do. Importing this module fails loudly when the
CUDA library has not been built: there is no CPU path.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libvibe_gb300.so")

SPECIES = ["u", "v", "w", "rho", "theta", "pi", "qv", "qc", "qr", "qi", "qs", "qg"]
NSPECIES = 12
HALO = 4
FP64, MIXED, FP64_EXACT = 0, 1, 2
_D, _I = ctypes.c_double, ctypes.c_int

if not os.path.exists(LIB_PATH):
    raise ImportError("libvibe_gb300.so is not built (run vibe-model_gb300/build.py); "
                      "the dynamics step has no CPU implementation")
lib = ctypes.CDLL(LIB_PATH)


class Setup(ctypes.Structure):
    """Mirror of ``vibe_gb300_setup``."""

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

    @classmethod
    def defaults(cls, **kw):
        s = cls()
        lib.vibe_gb300_setup_defaults(ctypes.byref(s))
        for k, v in kw.items():
            if not hasattr(s, k):
                raise AttributeError(k)
            setattr(s, k, v)
        return s

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


_vp = ctypes.c_void_p
_dp = ctypes.POINTER(ctypes.c_double)
_sigs = {
    "vibe_gb300_setup_defaults": (None, [ctypes.POINTER(Setup)]),
    "vibe_gb300_model_create": (_I, [ctypes.POINTER(Setup), _I, ctypes.POINTER(_vp)]),
    "vibe_gb300_model_destroy": (None, [_vp]),
    "vibe_gb300_storage_size": (ctypes.c_size_t, [_vp, _I]),
    "vibe_gb300_get_field": (_I, [_vp, _I, _vp]),
    "vibe_gb300_set_field": (_I, [_vp, _I, _vp]),
    "vibe_gb300_get_reffield": (_I, [_vp, _I, _vp]),
    "vibe_gb300_get_zeta": (_I, [_vp, _vp]),
    "vibe_gb300_get_terrain": (_I, [_vp, _vp]),
    "vibe_gb300_get_sponge": (_I, [_vp, _vp]),
    "vibe_gb300_step": (_I, [_vp, _D, _I, _I]),
    "vibe_gb300_step_async": (_I, [_vp, _D, _I, _I]),
    "vibe_gb300_sync": (_I, [_vp]),
    "vibe_gb300_slow_tendency": (_I, [_vp, ctypes.POINTER(_dp)]),
    "vibe_gb300_acoustic_substep": (_I, [_vp, _D]),
    "vibe_gb300_acoustic_tl": (_I, [_vp, _D, _I, ctypes.POINTER(_dp), ctypes.POINTER(_dp)]),
    "vibe_gb300_acoustic_ad": (_I, [_vp, _D, _I, ctypes.POINTER(_dp), ctypes.POINTER(_dp)]),
    "vibe_gb300_hevi_tl": (_I, [_vp, _D, _I, ctypes.POINTER(_dp), ctypes.POINTER(_dp)]),
    "vibe_gb300_acoustic_tl_f32": (_I, [_vp, _D, _I, ctypes.POINTER(_dp), ctypes.POINTER(_dp)]),
    "vibe_gb300_acoustic_ad_f32": (_I, [_vp, _D, _I, ctypes.POINTER(_dp), ctypes.POINTER(_dp)]),
    "vibe_gb300_hevi_tl_f32": (_I, [_vp, _D, _I, ctypes.POINTER(_dp), ctypes.POINTER(_dp)]),
    "vibe_gb300_hevi_ad_f32": (_I, [_vp, _D, _I, ctypes.POINTER(_dp), ctypes.POINTER(_dp)]),
    "vibe_gb300_hevi_ad": (_I, [_vp, _D, _I, ctypes.POINTER(_dp), ctypes.POINTER(_dp)]),
    "vibe_gb300_hevi_substep": (_I, [_vp, _D]),
    "vibe_gb300_tendency_tl": (_I, [_vp, ctypes.POINTER(_dp), ctypes.POINTER(_dp)]),
    "vibe_gb300_tendency_ad": (_I, [_vp, ctypes.POINTER(_dp), ctypes.POINTER(_dp)]),
    "vibe_gb300_step_tl": (_I, [_vp, _D, _I, ctypes.POINTER(_dp), ctypes.POINTER(_dp)]),
    "vibe_gb300_step_ad": (_I, [_vp, _D, _I, ctypes.POINTER(_dp), ctypes.POINTER(_dp)]),
    "vibe_gb300_window_plan": (_I, [ctypes.c_size_t, ctypes.c_size_t, _I, _I, ctypes.POINTER(_I)]),
    "vibe_gb300_sponge": (_I, [_vp, _D]),
    "vibe_gb300_snapshot": (_I, [_vp, _I]),
    "vibe_gb300_step_io": (_I, [_vp, ctypes.POINTER(_dp), _I, ctypes.POINTER(_dp), _I, _D, _I]),
    "vibe_gb300_io_join": (_I, [_vp]),
    "vibe_gb300_energy_budget": (_I, [_vp, _dp]),
    "vibe_gb300_write_restart": (_I, [_vp, ctypes.c_char_p, _D, _I]),
    "vibe_gb300_read_restart": (_I, [_vp, ctypes.c_char_p, ctypes.POINTER(_D), ctypes.POINTER(_I)]),
    "vibe_gb300_device_field": (_I, [_vp, _I, ctypes.POINTER(_dp), ctypes.POINTER(_I)]),
    "vibe_gb300_set_state": (_I, [_vp, ctypes.POINTER(_dp), _I]),
    "vibe_gb300_get_state": (_I, [_vp, ctypes.POINTER(_dp), _I]),
    "vibe_gb300_set_kernel_timing": (_I, [_vp, _I]),
    "vibe_gb300_kernel_times": (_I, [_vp, _dp, ctypes.POINTER(ctypes.c_long), _I]),
    "vibe_gb300_stream": (_vp, [_vp]),
    "vibe_gb300_launches_per_step": (_I, [_vp, _I]),
    "vibe_gb300_last_error": (ctypes.c_char_p, []),
    "vibe_gb300_si_step": (_I, [_vp, _D, _I, _I, _D, ctypes.POINTER(_I), _dp, _vp]),
    "vibe_gb300_si_stats": (_I, [_vp, ctypes.POINTER(_I), _dp, _dp]),
    "vibe_gb300_set_graph": (_I, [_vp, _I]),
    "vibe_gb300_cfl": (_I, [_vp, _D, _D, _dp, _dp, _dp]),
    "vibe_gb300_max_stable_dt": (_I, [_vp, _dp]),
    # C-ABI kernels (include/vibe_c_kernels.h)
    "vibe_tridiagonal_solve_f64": (_I, [_vp, _vp, _vp, _vp, _I, _vp, _vp]),
    "vibe_tridiagonal_solve_batched_f64": (_I, [_vp, _vp, _vp, _vp, _I, _I, _vp]),
    "vibe_weno5_reconstruct_f64": (None, [_D, _D, _D, _D, _D, _dp, _dp]),
    "vibe_bilinear_f64": (_D, [_vp, _I, _I, _I, _I, _D, _D, _I]),
    "vibe_cfl_scan_f64": (_D, [_vp, _vp, _vp, _vp, _vp, _I, _I, _I, _D, _D, _D, _D, _dp, _dp]),
    "vibe_neumaier_sum_f64": (_D, [_vp, ctypes.c_size_t]),
    "vibe_advect_scalar_flux_f64": (None, [_vp] * 7 + [_I, _I, _I, _D, _D, _D, _vp]),
    "vibe_c_last_error": (ctypes.c_char_p, []),
}
for _name, (_res, _args) in _sigs.items():
    _f = getattr(lib, _name)
    _f.restype = _res
    _f.argtypes = _args

ERRORS = {-1: "bad argument", -2: "device error", -3: "non-finite state", -4: "singular tridiagonal",
          -5: "unsupported"}


class VibeError(RuntimeError):
    """Raised for any non-zero status (the reference throws NumericalError)."""

    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (ERRORS.get(code, "error"), code, msg))
        self.code = code


def _check(rc):
    if rc != 0:
        raise VibeError(rc, lib.vibe_gb300_last_error().decode())
    return rc


def storage_shape(setup, species):
    """(nsz, nsy, nsx) of a species' FieldT storage (field.hpp:40-53)."""
    h2 = 2 * HALO
    return (setup.nz + h2 + (species == 2), setup.ny + h2 + (species == 1),
            setup.nx + h2 + (species == 0))


def interior(setup, species, arr):
    """Interior points incl. the extra face of a storage array."""
    a = np.asarray(arr).reshape(storage_shape(setup, species))
    return a[HALO:HALO + setup.nz + (species == 2), HALO:HALO + setup.ny + (species == 1),
             HALO:HALO + setup.nx + (species == 0)]


class Tuning(ctypes.Structure):
    """Mirror of vibe_gb300_tuning."""
    _fields_ = [("stage_levels", _I), ("column_kernel", _I), ("ms_per_step", _D), ("default_ms_per_step", _D),
                ("candidates", _I)]


lib.vibe_gb300_autotune.restype = _I
lib.vibe_gb300_autotune.argtypes = [_vp, _D, _I, ctypes.POINTER(Tuning)]
lib.vibe_gb300_set_tuning.restype = _I
lib.vibe_gb300_set_tuning.argtypes = [_vp, ctypes.POINTER(Tuning)]


class Kessler(ctypes.Structure):
    """Mirror of vibe_gb300_kessler (PhysicsOptions' Kessler fields)."""
    _fields_ = [("qc0", _D), ("k1", _D), ("k2", _D), ("evap_coef", _D), ("rain_a", _D), ("rain_b", _D),
                ("positive_definite", _I), ("exner_offset", _I)]

    @classmethod
    def defaults(cls, **kw):
        k = cls()
        lib.vibe_gb300_kessler_defaults(ctypes.byref(k))
        for name, v in kw.items():
            if not hasattr(k, name):
                raise AttributeError(name)
            setattr(k, name, v)
        return k


lib.vibe_gb300_kessler_defaults.restype = None
lib.vibe_gb300_kessler_defaults.argtypes = [ctypes.POINTER(Kessler)]
lib.vibe_gb300_set_physics.restype = _I
lib.vibe_gb300_set_physics.argtypes = [_vp, _vp, _vp]
lib.vibe_gb300_physics_tendency.restype = _I
lib.vibe_gb300_physics_tendency.argtypes = [_vp, _D, ctypes.POINTER(ctypes.POINTER(_D))]
PHYSICS_FIELDS = (0, 1, 4, 6, 7, 8, 9, 10, 11)  # u, v, theta, qv..qg


class Model:
    """A device-resident state plus its RK3 integrator."""

    def __init__(self, setup, precision=FP64):
        self.setup = setup
        self.precision = precision
        h = _vp()
        _check(lib.vibe_gb300_model_create(ctypes.byref(setup), precision, ctypes.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib.vibe_gb300_model_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def size(self, sp):
        return int(lib.vibe_gb300_storage_size(self.h, sp))

    def get(self, sp):
        a = np.empty(self.size(sp))
        _check(lib.vibe_gb300_get_field(self.h, sp, a.ctypes.data))
        return a

    def set(self, sp, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64).ravel()
        if a.size != self.size(sp):
            raise ValueError("species %d expects %d values, got %d" % (sp, self.size(sp), a.size))
        _check(lib.vibe_gb300_set_field(self.h, sp, a.ctypes.data))

    def state(self):
        return [self.get(sp) for sp in range(NSPECIES)]

    def set_state(self, st):
        for sp, a in enumerate(st):
            self.set(sp, a)

    def reffield(self, which):
        a = np.empty(self.size(3))
        _check(lib.vibe_gb300_get_reffield(self.h, which, a.ctypes.data))
        return a

    def zeta(self):
        a = np.empty(self.setup.nz + 1)
        _check(lib.vibe_gb300_get_zeta(self.h, a.ctypes.data))
        return a

    def terrain(self):
        a = np.empty(self.setup.nx * self.setup.ny)
        _check(lib.vibe_gb300_get_terrain(self.h, a.ctypes.data))
        return a

    def sponge_profile(self):
        a = np.empty(self.setup.nz)
        _check(lib.vibe_gb300_get_sponge(self.h, a.ctypes.data))
        return a

    def step(self, dt, n_sub, n_steps=1):
        return _check(lib.vibe_gb300_step(self.h, dt, n_sub, n_steps))

    def step_async(self, dt, n_sub, n_steps=1):
        return _check(lib.vibe_gb300_step_async(self.h, dt, n_sub, n_steps))

    def sync(self):
        return _check(lib.vibe_gb300_sync(self.h))

    def slow_tendency(self):
        outs = [np.empty(self.size(sp)) for sp in range(NSPECIES)]
        ptrs = (_dp * NSPECIES)(*[o.ctypes.data_as(_dp) for o in outs])
        _check(lib.vibe_gb300_slow_tendency(self.h, ptrs))
        return outs

    def acoustic_substep(self, dtau):
        _check(lib.vibe_gb300_acoustic_substep(self.h, dtau))

    def hevi_substep(self, dtau):
        _check(lib.vibe_gb300_hevi_substep(self.h, dtau))

    ACOUSTIC_FIELDS = (0, 1, 2, 3, 5)  # species of u, v, w, rho, pi

    def _acoustic_linear(self, fn, dtau, n_sub, fields):
        ins = [np.ascontiguousarray(fields[f], dtype=np.float64) for f in range(5)]
        for f, a in enumerate(ins):
            sp = self.ACOUSTIC_FIELDS[f]
            if a.size != self.size(sp):
                raise ValueError("%s has %d points, expected %d" % (SPECIES[sp], a.size, self.size(sp)))
        outs = [np.empty_like(a) for a in ins]
        pin = (_dp * 5)(*[a.ctypes.data_as(_dp) for a in ins])
        pout = (_dp * 5)(*[o.ctypes.data_as(_dp) for o in outs])
        _check(fn(self.h, dtau, n_sub, pin, pout))
        return outs

    def acoustic_tl(self, dtau, n_sub, fields):
        """Tangent-linear of n_sub explicit forward-backward substeps on the
        perturbations [u, v, w, rho, pi] (FieldT storage)."""
        return self._acoustic_linear(lib.vibe_gb300_acoustic_tl, dtau, n_sub, fields)

    def acoustic_ad(self, dtau, n_sub, fields):
        """Adjoint of acoustic_tl: <acoustic_tl(x), y> = <x, acoustic_ad(y)>."""
        return self._acoustic_linear(lib.vibe_gb300_acoustic_ad, dtau, n_sub, fields)

    def acoustic_tl_f32(self, dtau, n_sub, fields):
        """FP32 tangent-linear of the mixed model's forward-backward substep."""
        return self._acoustic_linear(lib.vibe_gb300_acoustic_tl_f32, dtau, n_sub, fields)

    def acoustic_ad_f32(self, dtau, n_sub, fields):
        """Adjoint of acoustic_tl_f32."""
        return self._acoustic_linear(lib.vibe_gb300_acoustic_ad_f32, dtau, n_sub, fields)

    def hevi_tl_f32(self, dtau, n_sub, fields):
        """FP32 tangent-linear of the mixed model's HEVI substep."""
        return self._acoustic_linear(lib.vibe_gb300_hevi_tl_f32, dtau, n_sub, fields)

    def hevi_ad_f32(self, dtau, n_sub, fields):
        """Adjoint of hevi_tl_f32."""
        return self._acoustic_linear(lib.vibe_gb300_hevi_ad_f32, dtau, n_sub, fields)

    def hevi_tl(self, dtau, n_sub, fields):
        """Tangent-linear of n_sub consistent HEVI substeps on [u, v, w, rho, pi]."""
        return self._acoustic_linear(lib.vibe_gb300_hevi_tl, dtau, n_sub, fields)

    def hevi_ad(self, dtau, n_sub, fields):
        """Adjoint of hevi_tl."""
        return self._acoustic_linear(lib.vibe_gb300_hevi_ad, dtau, n_sub, fields)

    def _own_linear(self, fn, args, states):
        ins = [np.ascontiguousarray(a, dtype=np.float64) for a in states]
        assert len(ins) == NSPECIES
        outs = [np.zeros(a.size) for a in ins]
        pin = (_dp * NSPECIES)(*[a.ctypes.data_as(_dp) for a in ins])
        pout = (_dp * NSPECIES)(*[a.ctypes.data_as(_dp) for a in outs])
        _check(fn(self.h, *args, pin, pout))
        return outs

    def tendency_tl(self, dx):
        """Tangent-linear of the slow tendency about the current state: 12
        FieldT perturbations in, the tendency's perturbation out."""
        return self._own_linear(lib.vibe_gb300_tendency_tl, (), dx)

    def tendency_ad(self, bar_r):
        """Adjoint of tendency_tl."""
        return self._own_linear(lib.vibe_gb300_tendency_ad, (), bar_r)

    def step_tl(self, dt, n_sub, dx):
        """Tangent-linear of one model step (slow tendency, acoustic substeps,
        sponge) about the current state, which it leaves as it is."""
        return self._own_linear(lib.vibe_gb300_step_tl, (dt, n_sub), dx)

    def step_ad(self, dt, n_sub, dy):
        """Adjoint of step_tl."""
        return self._own_linear(lib.vibe_gb300_step_ad, (dt, n_sub), dy)

    def autotune(self, dt, n_sub):
        """Pick the fastest launch shapes for this grid (mixed path); the
        candidates compute the same update up to FP32 rounding."""
        t = Tuning()
        _check(lib.vibe_gb300_autotune(self.h, dt, n_sub, ctypes.byref(t)))
        return {name: getattr(t, name) for name, _ in Tuning._fields_}

    def set_physics_kessler(self, kessler=None):
        """Couple the built-in Kessler warm-rain package into every RK stage
        (None: no physics). The options are kept alive by the model."""
        if kessler is None:
            _check(lib.vibe_gb300_set_physics(self.h, None, None))
            self._kessler = None
            return
        self._kessler = Kessler()
        ctypes.memmove(ctypes.addressof(self._kessler), ctypes.addressof(kessler), ctypes.sizeof(Kessler))
        fn = ctypes.cast(lib.vibe_gb300_physics_kessler, _vp)
        _check(lib.vibe_gb300_set_physics(self.h, fn, ctypes.addressof(self._kessler)))

    def physics_tendency(self, dt):
        """The installed package's tendency of the current state: dict species -> FieldT array."""
        outs = [np.zeros(self.size(sp)) for sp in PHYSICS_FIELDS]
        dp = ctypes.POINTER(_D)
        arr = (dp * 9)(*[o.ctypes.data_as(dp) for o in outs])
        _check(lib.vibe_gb300_physics_tendency(self.h, dt, arr))
        return dict(zip(PHYSICS_FIELDS, outs))

    def set_tuning(self, stage_levels=0, column_kernel=-1):
        """Pin launch shapes for this grid (0 / -1: the built-in choice)."""
        t = Tuning(stage_levels=stage_levels, column_kernel=column_kernel)
        _check(lib.vibe_gb300_set_tuning(self.h, ctypes.byref(t)))

    def step_io(self, in_ptrs, out_ptrs, dt, n_sub):
        """One asynchronous, pipelined step from host input to host output
        (lists of host addresses, None skips a species); finish with sync()."""
        a = (_dp * len(in_ptrs))(*[ctypes.cast(p, _dp) if p else None for p in in_ptrs])
        b = (_dp * len(out_ptrs))(*[ctypes.cast(p, _dp) if p else None for p in out_ptrs])
        _check(lib.vibe_gb300_step_io(self.h, a, len(in_ptrs), b, len(out_ptrs), dt, n_sub))

    def io_join(self):
        _check(lib.vibe_gb300_io_join(self.h))

    def energy_budget(self):
        """{kinetic, internal, potential, latent, total, mass} of the state (FP64)."""
        out = (_D * 6)()
        _check(lib.vibe_gb300_energy_budget(self.h, out))
        return dict(zip(("kinetic", "internal", "potential", "latent", "total", "mass"), out))

    def write_restart(self, path, time=0.0, step=0):
        """.vibebin restart file of the state (the reference's format)."""
        _check(lib.vibe_gb300_write_restart(self.h, os.fsencode(path), time, step))

    def read_restart(self, path):
        """Load a .vibebin restart file; returns (time, step)."""
        t, n = _D(), _I()
        _check(lib.vibe_gb300_read_restart(self.h, os.fsencode(path), ctypes.byref(t), ctypes.byref(n)))
        return t.value, n.value

    def save_snapshot(self):
        """Device copy of the current state (asynchronous)."""
        _check(lib.vibe_gb300_snapshot(self.h, 0))

    def restore_snapshot(self):
        _check(lib.vibe_gb300_snapshot(self.h, 1))

    def sponge(self, dt):
        _check(lib.vibe_gb300_sponge(self.h, dt))

    def set_state_ptrs(self, ptrs):
        """Asynchronous bulk upload from host addresses (ints; None skips)."""
        arr = (_dp * len(ptrs))(*[ctypes.cast(p, _dp) if p else None for p in ptrs])
        _check(lib.vibe_gb300_set_state(self.h, arr, len(ptrs)))

    def get_state_ptrs(self, ptrs):
        arr = (_dp * len(ptrs))(*[ctypes.cast(p, _dp) if p else None for p in ptrs])
        _check(lib.vibe_gb300_get_state(self.h, arr, len(ptrs)))

    def set_kernel_timing(self, on):
        _check(lib.vibe_gb300_set_kernel_timing(self.h, 1 if on else 0))

    def kernel_times(self):
        """{class: (total_ms, n_spans)} for 0 stage, 1 substep, 2 finish."""
        ms = (ctypes.c_double * 4)()
        n = (ctypes.c_long * 4)()
        _check(lib.vibe_gb300_kernel_times(self.h, ms, n, 4))
        return {c: (ms[c], n[c]) for c in range(4)}

    def stream(self):
        return lib.vibe_gb300_stream(self.h)

    def launches_per_step(self, n_sub):
        return int(lib.vibe_gb300_launches_per_step(self.h, n_sub))

    def si_step(self, dt, kind=1, max_iter=200, tol=1e-8, want_pi=False):
        """One semi-implicit step (SemiImplicitIntegrator::step). Returns
        (iterations, residual, pi_new or None); pi_new in FieldT storage."""
        it, res = ctypes.c_int(), ctypes.c_double()
        pin = np.full(self.size(3), np.nan) if want_pi else None
        _check(lib.vibe_gb300_si_step(self.h, dt, kind, max_iter, tol, ctypes.byref(it), ctypes.byref(res),
                                      None if pin is None else pin.ctypes.data))
        return it.value, res.value, pin

    def cfl(self, dt, dtau):
        """(cfl_number(s, dt), max_sound_speed(s), acoustic_cfl(s, dtau))."""
        out = [ctypes.c_double() for _ in range(3)]
        _check(lib.vibe_gb300_cfl(self.h, dt, dtau, *[ctypes.byref(o) for o in out]))
        return tuple(o.value for o in out)

    def max_stable_dt(self):
        out = ctypes.c_double()
        _check(lib.vibe_gb300_max_stable_dt(self.h, ctypes.byref(out)))
        return out.value

    def set_graph(self, on):
        _check(lib.vibe_gb300_set_graph(self.h, 1 if on else 0))

    def si_stats(self):
        """(iterations, residual, solve_ms) of the last semi-implicit step."""
        it, res, ms = ctypes.c_int(), ctypes.c_double(), ctypes.c_double()
        _check(lib.vibe_gb300_si_stats(self.h, ctypes.byref(it), ctypes.byref(res), ctypes.byref(ms)))
        return it.value, res.value, ms.value


# ---- C-ABI kernels (names as in the reference's c_kernels.h) ----------------
def _ptr(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64).ctypes.data


def tridiagonal_solve(a, b, c, d):
    """vibe_tridiagonal_solve_f64: returns (rc, x)."""
    b = np.ascontiguousarray(b, dtype=np.float64)
    n = b.size
    keep = [np.ascontiguousarray(v, dtype=np.float64) if v is not None else None for v in (a, c, d)]
    x = np.zeros(n)
    ws = np.zeros(max(n, 1))
    rc = lib.vibe_tridiagonal_solve_f64(_ptr(keep[0]), b.ctypes.data, _ptr(keep[1]), keep[2].ctypes.data, n,
                                        x.ctypes.data, ws.ctypes.data)
    return rc, x


def tridiagonal_solve_batched(a, b, c, d):
    """n_sys systems as rows of b, d (n_sys, n) and a, c (n_sys, n-1)."""
    b = np.ascontiguousarray(b, dtype=np.float64)
    n_sys, n = b.shape
    a = np.ascontiguousarray(a, dtype=np.float64)
    c = np.ascontiguousarray(c, dtype=np.float64)
    d = np.ascontiguousarray(d, dtype=np.float64)
    x = np.zeros_like(b)
    rc = lib.vibe_tridiagonal_solve_batched_f64(a.ctypes.data, b.ctypes.data, c.ctypes.data, d.ctypes.data, n, n_sys,
                                                x.ctypes.data)
    return rc, x


def weno5_reconstruct(qm2, qm1, q0, q1, q2):
    ql, qr = ctypes.c_double(), ctypes.c_double()
    lib.vibe_weno5_reconstruct_f64(qm2, qm1, q0, q1, q2, ctypes.byref(ql), ctypes.byref(qr))
    return ql.value, qr.value


def bilinear(f, halo, nsx, nsy, nz, xi, yj, k):
    f = np.ascontiguousarray(f, dtype=np.float64)
    return lib.vibe_bilinear_f64(f.ctypes.data, halo, nsx, nsy, nz, xi, yj, k)


def cfl_scan(u, v, w, dzeta, zs, nx, ny, nz, dx, dy, z_top, dt):
    keep = [np.ascontiguousarray(a, dtype=np.float64) if a is not None else None for a in (u, v, w, dzeta, zs)]
    mw, mdz = ctypes.c_double(), ctypes.c_double()
    r = lib.vibe_cfl_scan_f64(*[_ptr(k) for k in keep], nx, ny, nz, dx, dy, z_top, dt, ctypes.byref(mw),
                              ctypes.byref(mdz))
    return r, mw.value, mdz.value


def neumaier_sum(x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    return lib.vibe_neumaier_sum_f64(x.ctypes.data, x.size)


def advect_scalar_flux(q, rho, u, v, w, dzeta, zs, nx, ny, nz, dx, dy, z_top):
    keep = [np.ascontiguousarray(a, dtype=np.float64) if a is not None else None for a in (q, rho, u, v, w, dzeta, zs)]
    out = np.full(nx * ny * nz, np.nan)
    lib.vibe_advect_scalar_flux_f64(*[_ptr(k) for k in keep], nx, ny, nz, dx, dy, z_top, out.ctypes.data)
    return out


# ---- Helmholtz solvers (include/vibe_helmholtz.h) ---------------------------
HZ_VERTICAL_TRIDIAGONAL, HZ_KRYLOV_MULTIGRID, HZ_KRYLOV_JACOBI, HZ_MG_BICGSTAB_FP64, HZ_MG_BICGSTAB_MIXED = range(5)
_vp = ctypes.c_void_p
for _name, _res, _args in (
        ("vibe_helmholtz_create", _I, [_I, _I, _I, _I, _D, _D, _D, _vp, _vp, _I, _D, ctypes.POINTER(_vp)]),
        ("vibe_helmholtz_destroy", None, [_vp]),
        ("vibe_helmholtz_set_coefficients", _I, [_vp, _vp, _vp]),
        ("vibe_helmholtz_solve", _I, [_vp, _vp, _vp, _vp, _vp]),
        ("vibe_helmholtz_set_coefficients_dev", _I, [_vp, _vp, _vp, _vp]),
        ("vibe_helmholtz_solve_dev", _I, [_vp, _vp, _vp, _vp]),
        ("vibe_helmholtz_apply_dev", _I, [_vp, _vp, _vp, _vp]),
        ("vibe_helmholtz_iterations", _I, [_vp]),
        ("vibe_helmholtz_residual", _D, [_vp]),
        ("vibe_helmholtz_name", ctypes.c_char_p, [_vp]),
        ("vibe_helmholtz_set_iterative_refinement", _I, [_vp, _I, _I]),
        ("vibe_helmholtz_levels", _I, [_vp]),
        ("vibe_helmholtz_residual_l2", _D, [_vp, _vp, _vp]),
        ("vibe_helmholtz_last_error", ctypes.c_char_p, [])):
    _f = getattr(lib, _name)
    _f.restype = _res
    _f.argtypes = _args


class HelmholtzError(RuntimeError):
    def __init__(self, rc):
        super().__init__("helmholtz rc=%d: %s" % (rc, lib.vibe_helmholtz_last_error().decode()))
        self.rc = rc


class Helmholtz:
    """~ timeint::HelmholtzSolver from make_helmholtz_solver (helmholtz.hpp:63-98).
    Fields are host arrays in FieldT cell storage (halo 4); the *_dev
    methods take device addresses of nx*ny*nz doubles (i fastest)."""

    def __init__(self, kind, nx, ny, nz, dx, dy, z_top, dzeta, zs=None, max_iter=200, tol=1e-8):
        self.kind, self.shape = kind, (nz, ny, nx)
        self.h = _vp()
        dz = np.ascontiguousarray(dzeta, dtype=np.float64)
        zz = None if zs is None else np.ascontiguousarray(zs, dtype=np.float64)
        rc = lib.vibe_helmholtz_create(kind, nx, ny, nz, dx, dy, z_top, dz.ctypes.data,
                                       None if zz is None else zz.ctypes.data, max_iter, tol, ctypes.byref(self.h))
        if rc:
            raise HelmholtzError(rc)

    def close(self):
        if self.h:
            lib.vibe_helmholtz_destroy(self.h)
            self.h = _vp()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_coefficients(self, a, b):
        a, b = (np.ascontiguousarray(v, dtype=np.float64) for v in (a, b))
        rc = lib.vibe_helmholtz_set_coefficients(self.h, a.ctypes.data, b.ctypes.data)
        if rc:
            raise HelmholtzError(rc)

    def solve(self, a, b, f):
        """Returns (rc, x): rc 0 or 1 (singular column), x in FieldT storage."""
        f = np.ascontiguousarray(f, dtype=np.float64)
        x = np.full(f.size, np.nan)
        keep = [None if v is None else np.ascontiguousarray(v, dtype=np.float64) for v in (a, b)]
        rc = lib.vibe_helmholtz_solve(self.h, *[None if v is None else v.ctypes.data for v in keep], f.ctypes.data,
                                      x.ctypes.data)
        if rc not in (0, 1):
            raise HelmholtzError(rc)
        return rc, x

    def set_coefficients_dev(self, a_ptr, b_ptr, stream=0):
        rc = lib.vibe_helmholtz_set_coefficients_dev(self.h, a_ptr, b_ptr, stream)
        if rc:
            raise HelmholtzError(rc)

    def solve_dev(self, f_ptr, x_ptr, stream=0):
        rc = lib.vibe_helmholtz_solve_dev(self.h, f_ptr, x_ptr, stream)
        if rc not in (0, 1):
            raise HelmholtzError(rc)
        return rc

    def apply_dev(self, x_ptr, y_ptr, stream=0):
        rc = lib.vibe_helmholtz_apply_dev(self.h, x_ptr, y_ptr, stream)
        if rc:
            raise HelmholtzError(rc)

    def iterations(self):
        return int(lib.vibe_helmholtz_iterations(self.h))

    def residual(self):
        return float(lib.vibe_helmholtz_residual(self.h))

    def name(self):
        return lib.vibe_helmholtz_name(self.h).decode()

    def levels(self):
        return int(lib.vibe_helmholtz_levels(self.h))

    def set_iterative_refinement(self, on, precision=3):
        lib.vibe_helmholtz_set_iterative_refinement(self.h, 1 if on else 0, precision)

    def residual_l2(self, f, x):
        f, x = (np.ascontiguousarray(v, dtype=np.float64) for v in (f, x))
        return float(lib.vibe_helmholtz_residual_l2(self.h, f.ctypes.data, x.ctypes.data))


# ---- nest transfers (include/vibe_nest.h) -----------------------------------
class NestPlacement(ctypes.Structure):
    """Mirror of vibe_nest_placement (NestPlacement, nest.hpp:41-48)."""
    _fields_ = [("i0", _I), ("j0", _I), ("k0", _I), ("iext", _I), ("jext", _I), ("ratio", _I),
                ("boundary_zone", _I), ("two_way", _I)]


for _name, _args in (("vibe_nest_interpolate_from_parent", [_vp, _I, _vp, _I, _I, _I, _vp, _I, _I, _I, _vp]),
                     ("vibe_nest_restrict_to_parent", [_vp, _I, _vp, _I, _I, _I, _vp, _I, _I, _I, _vp]),
                     ("vibe_nest_apply_lateral_boundary", [_vp, _I, _vp, _I, _I, _I, _vp, _vp]),
                     ("vibe_nest_interpolate_from_parent_dev", [_vp, _I, _vp, _I, _I, _I, _vp, _I, _I, _I, _vp, _vp]),
                     ("vibe_nest_restrict_to_parent_dev", [_vp, _I, _vp, _I, _I, _I, _vp, _I, _I, _I, _vp, _vp]),
                     ("vibe_nest_apply_lateral_boundary_dev", [_vp, _I, _vp, _I, _I, _I, _vp, _vp, _vp]),
                     ("vibe_davies_profile", [_I, _D, _vp])):
    _f = getattr(lib, _name)
    _f.restype = _I
    _f.argtypes = _args


def _ptr_array(arrs):
    return (_vp * len(arrs))(*[a.ctypes.data for a in arrs])


def davies_profile(n_zone, alpha_max=1.0):
    out = np.zeros(n_zone)
    rc = lib.vibe_davies_profile(n_zone, alpha_max, out.ctypes.data)
    if rc:
        raise VibeError(-1)
    return out


def nest_interpolate_from_parent(pl, staggers, pdims, parent, cdims, child):
    """child (list of FieldT arrays) updated in place and returned."""
    st = np.ascontiguousarray(staggers, dtype=np.int32)
    parent = [np.ascontiguousarray(a, dtype=np.float64) for a in parent]
    rc = lib.vibe_nest_interpolate_from_parent(ctypes.byref(pl), len(st), st.ctypes.data, *pdims,
                                               _ptr_array(parent), *cdims, _ptr_array(child))
    if rc:
        raise RuntimeError("nest interpolate rc=%d" % rc)
    return child


def nest_restrict_to_parent(pl, staggers, cdims, child, pdims, parent):
    st = np.ascontiguousarray(staggers, dtype=np.int32)
    child = [np.ascontiguousarray(a, dtype=np.float64) for a in child]
    rc = lib.vibe_nest_restrict_to_parent(ctypes.byref(pl), len(st), st.ctypes.data, *cdims, _ptr_array(child),
                                          *pdims, _ptr_array(parent))
    if rc:
        raise RuntimeError("nest restrict rc=%d" % rc)
    return parent


def nest_apply_lateral_boundary(pl, staggers, cdims, child, parent_interp):
    st = np.ascontiguousarray(staggers, dtype=np.int32)
    parent_interp = [np.ascontiguousarray(a, dtype=np.float64) for a in parent_interp]
    rc = lib.vibe_nest_apply_lateral_boundary(ctypes.byref(pl), len(st), st.ctypes.data, *cdims, _ptr_array(child),
                                              _ptr_array(parent_interp))
    if rc:
        raise RuntimeError("nest lateral rc=%d" % rc)
    return child


# ---- tangent-linear / adjoint (include/vibe_tlad.h) -------------------------
for _name, _args in (("vibe_tlad_create", [_I, _I, _I, _D, _D, _D, _vp, _vp, _I, ctypes.POINTER(_vp)]),
                     ("vibe_tlad_set_base", [_vp, _vp]),
                     ("vibe_tl_tendency", [_vp, _vp, _vp]),
                     ("vibe_ad_tendency", [_vp, _vp, _vp]),
                     ("vibe_tl_step", [_vp, _D, _vp, _vp]),
                     ("vibe_tl_propagate", [_vp, _D, _I, _vp, _vp]),
                     ("vibe_ad_step", [_vp, _D, _vp, _vp]),
                     ("vibe_ad_propagate", [_vp, _D, _I, _vp, _vp]),
                     ("vibe_nl_propagate", [_vp, _D, _I, _vp, _vp]),
                     ("vibe_nl_tendency", [_vp, _vp, _vp])):
    _f = getattr(lib, _name)
    _f.restype = _I
    _f.argtypes = _args
lib.vibe_tlad_destroy.restype = None
lib.vibe_tlad_destroy.argtypes = [_vp]
lib.vibe_tlad_last_error.restype = ctypes.c_char_p
lib.vibe_tlad_last_error.argtypes = []


class TLAD:
    """~ da::TangentLinearModel + da::AdjointModel (tangent_linear.hpp:80-150).
    States: lists of 12 FieldT storage arrays (species order)."""

    def __init__(self, nx, ny, nz, dx, dy, z_top, dzeta, zs=None, precision=0):
        self.h = _vp()
        self.sizes = None
        dz = np.ascontiguousarray(dzeta, dtype=np.float64)
        zz = None if zs is None else np.ascontiguousarray(zs, dtype=np.float64)
        rc = lib.vibe_tlad_create(nx, ny, nz, dx, dy, z_top, dz.ctypes.data, None if zz is None else zz.ctypes.data,
                                  precision, ctypes.byref(self.h))
        self._rc(rc)

    @staticmethod
    def _rc(rc):
        if rc:
            raise RuntimeError("tlad rc=%d: %s" % (rc, lib.vibe_tlad_last_error().decode()))

    def close(self):
        if self.h:
            lib.vibe_tlad_destroy(self.h)
            self.h = _vp()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @staticmethod
    def _arr(states):
        return (_vp * 12)(*[s.ctypes.data for s in states])

    def _prep(self, states):
        return [np.ascontiguousarray(s, dtype=np.float64) for s in states]

    def set_base(self, xb):
        xb = self._prep(xb)
        self.sizes = [a.size for a in xb]
        self._rc(lib.vibe_tlad_set_base(self.h, self._arr(xb)))

    def _out(self):
        return [np.zeros(n) for n in self.sizes]

    def tl_tendency(self, dx):
        dx, d = self._prep(dx), self._out()
        self._rc(lib.vibe_tl_tendency(self.h, self._arr(dx), self._arr(d)))
        return d

    def ad_tendency(self, bar_d, bar_dx=None):
        bar_d = self._prep(bar_d)
        out = self._out() if bar_dx is None else [a.copy() for a in self._prep(bar_dx)]
        self._rc(lib.vibe_ad_tendency(self.h, self._arr(bar_d), self._arr(out)))
        return out

    def tl_propagate(self, dt, n, dx0):
        dx0, out = self._prep(dx0), self._out()
        self._rc(lib.vibe_tl_propagate(self.h, dt, n, self._arr(dx0), self._arr(out)))
        return out

    def ad_propagate(self, dt, n, dy):
        dy, out = self._prep(dy), self._out()
        self._rc(lib.vibe_ad_propagate(self.h, dt, n, self._arr(dy), self._arr(out)))
        return out

    def nl_tendency(self, x):
        x, d = self._prep(x), self._out()
        self._rc(lib.vibe_nl_tendency(self.h, self._arr(x), self._arr(d)))
        return d

    def nl_propagate(self, dt, n, x0):
        """The nonlinear collocated RK3 whose TL this is (FD checks)."""
        x0, out = self._prep(x0), self._out()
        self._rc(lib.vibe_nl_propagate(self.h, dt, n, self._arr(x0), self._arr(out)))
        return out

    def tl_step(self, dt, dx):
        return self.tl_propagate(dt, 1, dx)

    def ad_step(self, dt, dy):
        return self.ad_propagate(dt, 1, dy)


# ---- groups of models advanced together (include/vibe_gb300.h) --------------
for _name, _res, _args in (("vibe_gb300_group_create", _I, [ctypes.POINTER(_vp), _I, ctypes.POINTER(_vp)]),
                           ("vibe_gb300_group_destroy", None, [_vp]),
                           ("vibe_gb300_group_step", _I, [_vp, _D, _I, _I]),
                           ("vibe_gb300_group_launches_per_step", _I, [_vp]),
                           ("vibe_gb300_group_stream", _vp, [_vp])):
    _f = getattr(lib, _name)
    _f.restype = _res
    _f.argtypes = _args


class Group:
    """Several mixed-precision models stepped with one launch per kernel for
    all of them (the batched ensemble / nest step)."""

    def __init__(self, models):
        self.models = list(models)
        arr = (_vp * len(self.models))(*[m.h for m in self.models])
        self.h = _vp()
        _check(lib.vibe_gb300_group_create(arr, len(self.models), ctypes.byref(self.h)))

    def step(self, dt, n_sub, n_steps=1):
        _check(lib.vibe_gb300_group_step(self.h, dt, n_sub, n_steps))

    def launches_per_step(self):
        return int(lib.vibe_gb300_group_launches_per_step(self.h))

    def stream(self):
        return lib.vibe_gb300_group_stream(self.h)

    def close(self):
        if self.h:
            lib.vibe_gb300_group_destroy(self.h)
            self.h = _vp()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


# ---- nested sets: parents with two-way nests (include/vibe_gb300.h) ---------
for _name, _res, _args in (("vibe_gb300_nested_create", _I, [ctypes.POINTER(_vp), _I, ctypes.POINTER(_vp), _I,
                                                              ctypes.POINTER(_I), ctypes.POINTER(NestPlacement),
                                                              ctypes.POINTER(NestPlacement), ctypes.POINTER(_vp)]),
                           ("vibe_gb300_nested_destroy", None, [_vp]),
                           ("vibe_gb300_nested_step", _I, [_vp, _D, _I, _I]),
                           ("vibe_gb300_nested_launch", _I, [_vp, _D, _I, _I]),
                           ("vibe_gb300_nested_wait", _I, [_vp]),
                           ("vibe_gb300_nested_launches_per_step", _I, [_vp]),
                           ("vibe_gb300_nested_stream", _vp, [_vp])):
    _f = getattr(lib, _name)
    _f.restype = _res
    _f.argtypes = _args


class Nested:
    """Parents stepped with dt and their two-way nests with ratio sub-steps
    of dt/ratio, coupled by interpolation, Davies relaxation and
    restriction. interp_pl / restrict_pl: one NestPlacement per nest, the
    first with its offset in nest points, the second in parent points."""

    def __init__(self, parents, children, parent_of, interp_pl, restrict_pl):
        self.parents, self.children = list(parents), list(children)
        pa = (_vp * len(self.parents))(*[m.h for m in self.parents])
        ch = (_vp * len(self.children))(*[m.h for m in self.children])
        po = (_I * len(self.children))(*parent_of)
        ip = (NestPlacement * len(self.children))(*interp_pl)
        rp = (NestPlacement * len(self.children))(*restrict_pl)
        self.h = _vp()
        _check(lib.vibe_gb300_nested_create(pa, len(self.parents), ch, len(self.children), po, ip, rp,
                                            ctypes.byref(self.h)))

    def step(self, dt, n_sub, n_steps=1):
        _check(lib.vibe_gb300_nested_step(self.h, dt, n_sub, n_steps))

    def step_async(self, dt, n_sub, n_steps=1):
        _check(lib.vibe_gb300_nested_launch(self.h, dt, n_sub, n_steps))

    def wait(self):
        _check(lib.vibe_gb300_nested_wait(self.h))

    def launches_per_step(self):
        return int(lib.vibe_gb300_nested_launches_per_step(self.h))

    def stream(self):
        return lib.vibe_gb300_nested_stream(self.h)

    def close(self):
        if self.h:
            lib.vibe_gb300_nested_destroy(self.h)
            self.h = _vp()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


# ---- assimilation windows: TL/AD about the model trajectory (vibe_gb300.h) --
for _name, _res, _args in (("vibe_gb300_window_create", _I, [_vp, _vp, _D, _I, _I, _I, _I, ctypes.POINTER(_vp)]),
                           ("vibe_gb300_window_destroy", None, [_vp]),
                           ("vibe_gb300_window_tl", _I, [_vp, _vp, _vp]),
                           ("vibe_gb300_window_ad", _I, [_vp, _vp, _vp]),
                           ("vibe_gb300_window_stats", _I, [_vp, ctypes.POINTER(_D), ctypes.POINTER(ctypes.c_size_t),
                                                            ctypes.POINTER(ctypes.c_size_t)])):
    _f = getattr(lib, _name)
    _f.restype = _res
    _f.argtypes = _args


def window_plan(free_bytes, state_bytes, n_steps, seg_states):
    """The window's automatic checkpoint spacing (every = 0) for a given free
    device memory: 1 (store every step) or ceil(sqrt(n_steps / seg_states));
    raises VibeError when the checkpoints do not fit."""
    every = _I()
    _check(lib.vibe_gb300_window_plan(free_bytes, state_bytes, n_steps, seg_states, ctypes.byref(every)))
    return every.value


class Window:
    """TL/AD linearised about the trajectory of a Model over n_steps steps of
    dt, checkpointed every `every` steps and recomputed in the adjoint sweep.
    tlad = a TLAD object (the reference's collocated TL/AD, tl_substeps steps
    per model step) or None (the TL/AD of the model's own step).
    Perturbations are lists of 12 FieldT arrays."""

    def __init__(self, model, tlad, dt, n_sub, n_steps, every=10, tl_substeps=1):
        self.model, self.tlad = model, tlad
        self.h = _vp()
        _check(lib.vibe_gb300_window_create(model.h, tlad.h if tlad is not None else None, dt, n_sub, n_steps,
                                            every, tl_substeps, ctypes.byref(self.h)))

    def _io(self, states):
        ins = [np.ascontiguousarray(a, dtype=np.float64) for a in states]
        outs = [np.zeros(a.size) for a in ins]
        return ins, outs

    def tl(self, dx0):
        ins, outs = self._io(dx0)
        _check(lib.vibe_gb300_window_tl(self.h, TLAD._arr(ins), TLAD._arr(outs)))
        return outs

    def ad(self, dy):
        ins, outs = self._io(dy)
        _check(lib.vibe_gb300_window_ad(self.h, TLAD._arr(ins), TLAD._arr(outs)))
        return outs

    def stats(self):
        """(device ms of the last sweep, checkpoint bytes, segment bytes)"""
        ms, ck, sg = _D(), ctypes.c_size_t(), ctypes.c_size_t()
        _check(lib.vibe_gb300_window_stats(self.h, ctypes.byref(ms), ctypes.byref(ck), ctypes.byref(sg)))
        return ms.value, ck.value, sg.value

    def close(self):
        if self.h:
            lib.vibe_gb300_window_destroy(self.h)
            self.h = _vp()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
