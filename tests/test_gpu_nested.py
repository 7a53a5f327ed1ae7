"""Nested sets (vibe_gb300_nested_*): one parent step with dt, the nest's
r = 3 sub-steps of dt/3 with the parent interpolated into a boundary buffer
(Nest::interpolate_from_parent, src/grid/nest.cpp:58-84), Davies relaxation
after every sub-step (apply_lateral_boundary, nest.cpp:107-124) and two-way
restriction at the end (restrict_to_parent, nest.cpp:86-105).

Two checks:
  * the nested object matches the same sequence composed by hand from single
    models and the oracle's transfers on host copies of the state to FP32
    rounding (the transfers are bit-exact; grouped and single steps agree to
    rounding, 1e-6 of each field's scale);
  * the whole composition run on the oracle (FP64 steps, FP64 transfers)
    agrees with the mixed GPU path to 5e-5 of each field's scale: four
    mixed steps (one parent step, three nest steps) each within 1e-5 of
    the FP64 step, plus the transfers, which are linear in the state.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STAGGERS = [1, 2, 3, 0, 0, 0, 0]  # u v w rho theta pi qv
DT, NSUB, R = 6.0, 6, 3
TOL_NEST = 5e-5


def setups(vg):
    common = dict(nz=14, z_top=6000.0, zeta_first=1.0, zeta_stretch=1.05, ref_kind=1, acoustic_mode=2,
                  u_background=8.0, shear_u=0.001, bubble_zc=1500.0, bubble_radius_z=1000.0, qv_surface=0.0)
    parent = vg.Setup.defaults(nx=24, ny=20, dx=1500.0, dy=1500.0, bubble_xc=16000.0, bubble_yc=13000.0,
                               bubble_radius_x=4500.0, bubble_amplitude=2.0, **common)
    child = vg.Setup.defaults(nx=31, ny=25, dx=500.0, dy=500.0, bubble_xc=6500.0, bubble_yc=5500.0,
                              bubble_radius_x=3000.0, bubble_amplitude=1.5, **common)
    interp = dict(i0=18, j0=15, iext=10, jext=8, ratio=R, boundary_zone=5, two_way=1)
    restrict = dict(i0=6, j0=5, iext=10, jext=8, ratio=R, boundary_zone=5, two_way=1)
    return parent, child, interp, restrict


def second_nest(vg):
    """A second, differently shaped nest of the same parent (west edge, partly
    outside it: the interpolation clamps to the parent's edge cells)."""
    common = dict(nz=14, z_top=6000.0, zeta_first=1.0, zeta_stretch=1.05, ref_kind=1, acoustic_mode=2,
                  u_background=8.0, shear_u=0.001, bubble_zc=1500.0, bubble_radius_z=1000.0, qv_surface=0.0,
                  bubble_amplitude=0.0)
    child = vg.Setup.defaults(nx=13, ny=40, dx=500.0, dy=500.0, **common)
    interp = dict(i0=-3, j0=6, iext=4, jext=13, ratio=R, boundary_zone=4, two_way=1)
    restrict = dict(i0=0, j0=2, iext=4, jext=13, ratio=R, boundary_zone=4, two_way=1)
    return child, interp, restrict


def placement(cls, d):
    q = cls()
    for name, _ in cls._fields_:
        if name in d:
            setattr(q, name, int(d[name]))
    return q


def dims(s):
    return (s.nx, s.ny, s.nz)


def oracle_setup(oc, s):
    t = oc.Setup()
    for name, _ in oc.Setup._fields_:
        setattr(t, name, getattr(s, name))
    return t


def compose(oc, parents, ps, nests, step):
    """One parent step of the nested sequence on models with get/set.
    nests: (child model, child setup, parent index, interp, restrict);
    step(model, dt) advances one model by one step."""
    for p in parents:
        step(p, DT)
    bufs = []
    for c, cs, pi, interp, _ in nests:
        buf = [np.zeros(oc.fieldt_size(*dims(cs), st)) for st in STAGGERS]
        oc.nest_interpolate_from_parent(interp, STAGGERS, dims(ps), [parents[pi].get(q) for q in range(7)],
                                        dims(cs), buf)
        bufs.append(buf)
    for _ in range(R):
        for (c, cs, pi, interp, _), buf in zip(nests, bufs):
            step(c, DT / R)
            st = [c.get(q) for q in range(7)]
            oc.nest_apply_lateral_boundary(interp, STAGGERS, dims(cs), st, buf)
            for q in range(7):
                c.set(q, st[q])
    for c, cs, pi, _, restrict in nests:
        pst = [parents[pi].get(q) for q in range(7)]
        oc.nest_restrict_to_parent(restrict, STAGGERS, dims(cs), [c.get(q) for q in range(7)], dims(ps), pst)
        for q in range(7):
            parents[pi].set(q, pst[q])


def test_nested_step_equals_composition(vg, oc):
    """Two members, each a parent with two nests of different shapes."""
    ps, cs, interp, restrict = setups(vg)
    cs2, interp2, restrict2 = second_nest(vg)
    shapes = [(cs, 0, interp, restrict), (cs2, 0, interp2, restrict2), (cs, 1, interp, restrict),
              (cs2, 1, interp2, restrict2)]
    models = []

    def build():
        pa = [vg.Model(ps, vg.MIXED) for _ in range(2)]
        th = pa[1].get(4)
        pa[1].set(4, th + 0.01 * np.random.default_rng(3).standard_normal(th.size) * (th != 0.0))
        ch = [vg.Model(s, vg.MIXED) for s, _, _, _ in shapes]
        models.extend(pa + ch)
        return pa, ch

    try:
        a_p, a_c = build()
        b_p, b_c = build()
        with vg.Nested(a_p, a_c, [pi for _, pi, _, _ in shapes],
                       [placement(vg.NestPlacement, i) for _, _, i, _ in shapes],
                       [placement(vg.NestPlacement, r) for _, _, _, r in shapes]) as n:
            n.step(DT, NSUB, 1)
            n.step_async(DT, NSUB, 1)
            n.wait()
            # interpolation, R relaxations (each with its frame's working
            # copy), restriction + the parent box's working copy
            per_nest = 1 + R + 2
            # per stage 1 stage + NSUB column launches; the fix-up after
            # stages 1 and 2; stage 3's is in the finish
            group = 3 * (1 + NSUB) + 2 + 1
            assert n.launches_per_step() == group + R * group + len(shapes) * per_nest
        nests = [(c, s, pi, i, r) for c, (s, pi, i, r) in zip(b_c, shapes)]
        for _ in range(2):
            compose(oc, b_p, ps, nests, lambda m, dt: m.step(dt, NSUB, 1))
        from test_gpu_group import assert_rounding_close
        for x, y, s in zip(a_p + a_c, b_p + b_c, [ps, ps] + [sh[0] for sh in shapes]):
            assert_rounding_close(vg, s, [x.get(q) for q in range(7)], [y.get(q) for q in range(7)],
                                  what="nested vs composition")
    finally:
        for m in models:
            m.close()


def rel_err(vg, s, q, got, ref, vscale):
    g, r = vg.interior(s, q, got), vg.interior(s, q, ref)
    scale = vscale if q < 3 else float(np.abs(r).max())
    if scale == 0.0:  # a species that is zero everywhere (dry qv) must stay zero
        return float(np.abs(g).max())
    return float(np.abs(g - r).max() / scale)


def test_nested_step_tracks_oracle(vg, oc):
    ps, cs, interp, restrict = setups(vg)
    with vg.Model(ps, vg.MIXED) as gp, vg.Model(cs, vg.MIXED) as gc:
        with vg.Nested([gp], [gc], [0], [placement(vg.NestPlacement, interp)],
                       [placement(vg.NestPlacement, restrict)]) as n:
            n.step(DT, NSUB, 1)
        op, ocm = oc.Model(oracle_setup(oc, ps), "port"), oc.Model(oracle_setup(oc, cs), "port")
        compose(oc, [op], ps, [(ocm, cs, 0, interp, restrict)], lambda m, dt: m.rk3_step(dt, NSUB))
        for s, g, o in ((ps, gp, op), (cs, gc, ocm)):
            ref = [o.get(q) for q in range(7)]
            vs = max(float(np.abs(vg.interior(s, q, ref[q])).max()) for q in range(3))
            errs = {vg.SPECIES[q]: rel_err(vg, s, q, g.get(q), ref[q], vs) for q in range(7)}
            assert all(e <= TOL_NEST for e in errs.values()), errs


def test_nested_rejects_bad_sets(vg):
    ps, cs, interp, restrict = setups(vg)
    with vg.Model(ps, vg.MIXED) as p, vg.Model(cs, vg.MIXED) as c:
        bad_ratio = dict(interp, ratio=1)
        with pytest.raises(vg.VibeError):
            vg.Nested([p], [c], [0], [placement(vg.NestPlacement, bad_ratio)],
                      [placement(vg.NestPlacement, restrict)])
        with pytest.raises(vg.VibeError):
            vg.Nested([p], [c], [1], [placement(vg.NestPlacement, interp)],
                      [placement(vg.NestPlacement, restrict)])
