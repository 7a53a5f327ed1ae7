"""Tangent-linear and adjoint of the explicit forward-backward acoustic substep
(vibe_gb300_acoustic_tl / _ad) on the GPU.

The forward substep is RungeKutta3Integrator::acoustic_substep
(runge_kutta.cpp:65-75) with Equations::acoustic_tendencies
(equations.cpp:152-209), pinned against the oracle in test_gpu_step.py. With
the gradient taken of pi itself the substep is linear in (u, v, w, rho, pi):
its tangent-linear is the substep on the perturbation, checked here against
the model's own substep and against finite differences of the substep with
the pi' gradient (where it is affine); the adjoint is checked by the
dot-product test and, on a tiny grid, entry by entry against the transposed
tangent-linear matrix."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = (0, 1, 2, 3, 5)  # u, v, w, rho, pi
SCALE = (1.0, 1.0, 0.5, 1e-3, 1e-4)


def setup(vg, **kw):
    base = dict(nx=18, ny=14, nz=10, dx=250.0, dy=250.0, z_top=3000.0, zeta_first=1.0, zeta_stretch=1.08,
                bubble_xc=2500.0, bubble_yc=2000.0, bubble_zc=1000.0, bubble_radius_x=1500.0,
                bubble_radius_z=1000.0, u_background=5.0, shear_u=0.001, terrain_kind=1, hill_h=300.0,
                hill_a=1000.0, hill_xc=2200.0, hill_yc=1700.0, ref_kind=1)
    base.update(kw)
    return vg.Setup.defaults(**base)


def box(vg, s, sp, a):
    """The staggered box the substep reads and writes: (nx+1, ny+1, nz(+1 for w))."""
    v = np.asarray(a).reshape(vg.storage_shape(s, sp))
    return v[vg.HALO:vg.HALO + s.nz + (sp == 2), vg.HALO:vg.HALO + s.ny + 1, vg.HALO:vg.HALO + s.nx + 1]


def random_fields(vg, m, seed, halo=True):
    rng = np.random.default_rng(seed)
    out = []
    for f, sp in enumerate(FIELDS):
        a = SCALE[f] * rng.standard_normal(m.size(sp))
        if not halo:
            b = np.zeros_like(a)
            box(vg, m.setup, sp, b)[...] = box(vg, m.setup, sp, a)
            a = b
        out.append(a)
    return out


def dot(a, b):
    return float(sum(np.dot(x, y) for x, y in zip(a, b)))


def test_tl_is_the_substep_on_the_perturbation(vg):
    """With pgf_perturbation=0 the model's own substep is linear: running it on
    a state whose acoustic fields are the perturbation gives the TL's bits."""
    s = setup(vg, pgf_perturbation=0)
    with vg.Model(s, vg.FP64) as m:
        dx = random_fields(vg, m, 1)
        got = m.acoustic_tl(0.4, 3, dx)
        st = m.state()
        for f, sp in enumerate(FIELDS):
            st[sp] = dx[f]
        m.set_state(st)
        for _ in range(3):
            m.acoustic_substep(0.4)
        ref = m.state()
        for f, sp in enumerate(FIELDS):
            assert np.array_equal(vg.interior(s, sp, got[f]), vg.interior(s, sp, ref[sp])), vg.SPECIES[sp]


def test_tl_matches_finite_differences_of_the_perturbation_pgf_substep(vg):
    """The reference-semantic substep (pressure gradient of pi - pi0) is affine
    in the state, so (S(x + e dx) - S(x)) / e equals the TL for every e up to
    rounding."""
    s = setup(vg, pgf_perturbation=1)
    with vg.Model(s, vg.FP64) as m:
        x0 = m.state()
        dx = random_fields(vg, m, 2)
        tl = m.acoustic_tl(0.4, 2, dx)
        for e in (1e-2, 1e-4):
            st = [a.copy() for a in x0]
            for f, sp in enumerate(FIELDS):
                st[sp] = st[sp] + e * dx[f]
            m.set_state(st)
            m.acoustic_substep(0.4)
            m.acoustic_substep(0.4)
            s1 = m.state()
            m.set_state(x0)
            m.acoustic_substep(0.4)
            m.acoustic_substep(0.4)
            s0 = m.state()
            for f, sp in enumerate(FIELDS):
                fd = (vg.interior(s, sp, s1[sp]) - vg.interior(s, sp, s0[sp])) / e
                ref = vg.interior(s, sp, tl[f])
                scale = np.abs(ref).max()
                tol = 1e-12 * np.abs(vg.interior(s, sp, x0[sp])).max() / e / scale + 1e-9
                assert np.abs(fd - ref).max() <= tol * scale, (vg.SPECIES[sp], e, np.abs(fd - ref).max() / scale)


@pytest.mark.parametrize("prec", ["FP64", "MIXED"])
def test_dot_product(vg, prec):
    """<TL dx, dy> = <dx, AD dy> over 5 substeps to 1e-12 (FP64 arithmetic for
    either model precision); every point outside the boxes passes through."""
    kw = dict(terrain_kind=0, ref_kind=0, acoustic_mode=2) if prec == "MIXED" else {}
    s = setup(vg, **kw)
    with vg.Model(s, getattr(vg, prec)) as m:
        for seed in (3, 4):
            dx, dy = random_fields(vg, m, seed), random_fields(vg, m, seed + 10)
            tdx = m.acoustic_tl(0.5, 5, dx)
            ady = m.acoustic_ad(0.5, 5, dy)
            lhs, rhs = dot(tdx, dy), dot(dx, ady)
            assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), abs(rhs)), (lhs, rhs)
            for f, sp in enumerate(FIELDS):
                keep = np.ones(m.size(sp), bool)
                box(vg, s, sp, keep)[...] = False
                assert np.array_equal(tdx[f][keep], dx[f][keep])
                assert np.array_equal(ady[f][keep], dy[f][keep])
            # the operator is not the identity
            assert max(np.abs(a - b).max() for a, b in zip(tdx, dx)) > 0.0


def test_adjoint_is_the_transposed_matrix(vg):
    """On a 3 x 2 x 2 grid with terrain: the AD of each unit vector is the
    corresponding row of the TL matrix."""
    s = setup(vg, nx=3, ny=2, nz=2, dx=500.0, dy=500.0, hill_xc=700.0, hill_yc=500.0, hill_a=600.0,
              bubble_xc=700.0, bubble_yc=500.0, bubble_radius_x=600.0)
    with vg.Model(s, vg.FP64) as m:
        pts = []
        for f, sp in enumerate(FIELDS):
            idx = np.arange(m.size(sp))
            pts += [(f, int(e)) for e in box(vg, s, sp, idx).ravel()]
        zero = [np.zeros(m.size(sp)) for sp in FIELDS]

        def unit(p):
            u = [a.copy() for a in zero]
            u[p[0]][p[1]] = 1.0
            return u

        def row(fields):
            return np.array([fields[f][e] for f, e in pts])

        tl = np.array([row(m.acoustic_tl(0.7, 2, unit(p))) for p in pts]).T  # tl[r, c] = d out_r / d in_c
        ad = np.array([row(m.acoustic_ad(0.7, 2, unit(p))) for p in pts]).T
        scale = np.abs(tl).max()
        assert np.abs(ad - tl.T).max() <= 1e-14 * scale, np.abs(ad - tl.T).max() / scale
        assert np.count_nonzero(tl - np.eye(len(pts))) > len(pts)


def test_bad_arguments(vg):
    s = setup(vg)
    with vg.Model(s, vg.FP64) as m:
        f = random_fields(vg, m, 5)
        with pytest.raises(ValueError):
            m.acoustic_tl(0.5, 1, [f[0][:-1]] + f[1:])
        with pytest.raises(RuntimeError):
            m.acoustic_tl(0.5, -1, f)


# ---- the consistent HEVI substep (vibe_gb300_hevi_tl / _ad) ----------------
def test_hevi_tl_is_the_substep_on_the_perturbation(vg):
    """With pgf_perturbation=0 the model's own consistent HEVI substep (column
    solve + u/v update) is linear: on the perturbation it gives the TL's
    bits."""
    s = setup(vg, pgf_perturbation=0, acoustic_mode=2, hevi_beta=0.6)
    with vg.Model(s, vg.FP64) as m:
        dx = random_fields(vg, m, 21)
        got = m.hevi_tl(0.8, 3, dx)
        st = m.state()
        for f, sp in enumerate(FIELDS):
            st[sp] = dx[f]
        m.set_state(st)
        for _ in range(3):
            m.hevi_substep(0.8)
        ref = m.state()
        for f, sp in enumerate(FIELDS):
            assert np.array_equal(vg.interior(s, sp, got[f]), vg.interior(s, sp, ref[sp])), vg.SPECIES[sp]


@pytest.mark.parametrize("prec", ["FP64", "MIXED"])
def test_hevi_dot_product(vg, prec):
    """<TL dx, dy> = <dx, AD dy> over 4 HEVI substeps to 1e-12, with terrain
    (FP64 model) and on the mixed model's flat grid; points outside the boxes
    pass through."""
    kw = dict(terrain_kind=0, ref_kind=0) if prec == "MIXED" else {}
    s = setup(vg, acoustic_mode=2, hevi_beta=0.6, **kw)
    with vg.Model(s, getattr(vg, prec)) as m:
        for seed in (23, 24):
            dx, dy = random_fields(vg, m, seed), random_fields(vg, m, seed + 10)
            tdx = m.hevi_tl(1.5, 4, dx)
            ady = m.hevi_ad(1.5, 4, dy)
            lhs, rhs = dot(tdx, dy), dot(dx, ady)
            assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), abs(rhs)), (lhs, rhs)
            for f, sp in enumerate(FIELDS):
                keep = np.ones(m.size(sp), bool)
                box(vg, s, sp, keep)[...] = False
                assert np.array_equal(tdx[f][keep], dx[f][keep])
                assert np.array_equal(ady[f][keep], dy[f][keep])


def test_hevi_adjoint_is_the_transposed_matrix(vg):
    """3 x 2 x 3 grid with terrain: the HEVI AD of each unit vector is the
    corresponding row of the HEVI TL matrix (to 1e-13 of the largest entry)."""
    s = setup(vg, nx=3, ny=2, nz=3, dx=500.0, dy=500.0, hill_xc=700.0, hill_yc=500.0, hill_a=600.0,
              bubble_xc=700.0, bubble_yc=500.0, bubble_radius_x=600.0, acoustic_mode=2, hevi_beta=0.6)
    with vg.Model(s, vg.FP64) as m:
        pts = []
        for f, sp in enumerate(FIELDS):
            idx = np.arange(m.size(sp))
            pts += [(f, int(e)) for e in box(vg, s, sp, idx).ravel()]
        zero = [np.zeros(m.size(sp)) for sp in FIELDS]

        def unit(p):
            u = [a.copy() for a in zero]
            u[p[0]][p[1]] = 1.0
            return u

        def row(fields):
            return np.array([fields[f][e] for f, e in pts])

        tl = np.array([row(m.hevi_tl(2.0, 2, unit(p))) for p in pts]).T
        ad = np.array([row(m.hevi_ad(2.0, 2, unit(p))) for p in pts]).T
        scale = np.abs(tl).max()
        assert np.abs(ad - tl.T).max() <= 1e-13 * scale, np.abs(ad - tl.T).max() / scale
        assert np.count_nonzero(tl - np.eye(len(pts))) > len(pts)


# ---- the FP32 form on mixed models (vibe_gb300_acoustic_tl_f32 / _ad_f32) ----
def test_fp32_acoustic_tl_ad(vg):
    """The mixed model's own FP32 forward-backward substep as a linear map of
    (u, v, w, rho', pi'): it tracks the FP64 tangent-linear to 1e-5 of each
    field's scale over 4 substeps, and its adjoint passes the dot-product test
    to 1e-5."""
    s = setup(vg, terrain_kind=0, ref_kind=0)
    with vg.Model(s, vg.MIXED) as m:
        dx, dy = random_fields(vg, m, 31), random_fields(vg, m, 32)
        t32 = m.acoustic_tl_f32(0.5, 4, dx)
        t64 = m.acoustic_tl(0.5, 4, dx)
        for f, sp in enumerate(FIELDS):
            g, r = vg.interior(s, sp, t32[f]), vg.interior(s, sp, t64[f])
            assert np.abs(g - r).max() <= 1e-5 * np.abs(r).max(), (vg.SPECIES[sp], np.abs(g - r).max())
        a32 = m.acoustic_ad_f32(0.5, 4, dy)
        lhs, rhs = dot(t32, dy), dot(dx, a32)
        assert abs(lhs - rhs) <= 1e-5 * max(abs(lhs), abs(rhs)), (lhs, rhs)
    with vg.Model(s, vg.FP64) as f64:
        with pytest.raises(vg.VibeError):
            f64.acoustic_tl_f32(0.5, 1, random_fields(vg, f64, 33))


def test_fp32_hevi_tl_ad(vg):
    """The mixed model's own FP32 HEVI substep (TMA column kernel + u/v
    update) as a linear map: it tracks the FP64 HEVI tangent-linear to 1e-5
    of each field's scale over 3 substeps, and its adjoint (the column system
    transposed through its LU factors) passes the dot-product test to 1e-5;
    a step afterwards still matches a model that never ran it (the column
    factors are put back for the step's own dt)."""
    s = setup(vg, terrain_kind=0, ref_kind=0, acoustic_mode=2, hevi_beta=0.6)
    with vg.Model(s, vg.MIXED) as m, vg.Model(s, vg.MIXED) as ref:
        dx, dy = random_fields(vg, m, 41), random_fields(vg, m, 42)
        t32 = m.hevi_tl_f32(1.5, 3, dx)
        t64 = m.hevi_tl(1.5, 3, dx)
        for f, sp in enumerate(FIELDS):
            g, r = vg.interior(s, sp, t32[f]), vg.interior(s, sp, t64[f])
            assert np.abs(g - r).max() <= 1e-5 * np.abs(r).max(), (vg.SPECIES[sp], np.abs(g - r).max())
        a32 = m.hevi_ad_f32(1.5, 3, dy)
        lhs, rhs = dot(t32, dy), dot(dx, a32)
        assert abs(lhs - rhs) <= 1e-5 * max(abs(lhs), abs(rhs)), (lhs, rhs)
        m.step(2.0, 4, 2)
        ref.step(2.0, 4, 2)
        for a, b in zip(m.state(), ref.state()):
            assert np.array_equal(a, b)
