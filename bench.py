#!/usr/bin/env python
"""Throughput of the GB300 dynamics step (cell-updates/s) on the
512 x 512 x 80 single-domain case.

Workload (synthetic, seeded): dx = dy = 1 km; 80 levels stretched from a
50 m first layer over a 20 km top (ratio 1.0341247533415947: with a 50 m
first layer and 20 km depth, geometric stretching over 80 levels ends at
708 m, not 500 m); theta0 = 300 K with N = 0.01 1/s; uniform u = 10 m/s;
theta' ~ U(-0.5, 0.5) K below 1 km plus 20 warm bubbles (1-3 K, radius
1-4 km, centres uniform in x, y and in 1-5 km height); WENO5 scalars,
2nd-order momentum (the reference has no 4th-order momentum advection);
dt = 6 s, 6 acoustic substeps per RK stage with the vertically implicit
substep; pi' pressure gradient and fast terms integrated once.

One step = one SSP-RK3 step: 3 stages + 18 acoustic substeps + sponge.
`value` is the mixed-precision (FP64 state, FP32 compute) path; the plain
FP64 path is measured beside it. Inputs (1.7 GB of FP64 state) are far
larger than the 129 MB L2, so no flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
Under torchrun every rank advances its own replica (an ensemble member):
weak scaling, no collective on the data path.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "vibe-model_gb300")
sys.path.insert(0, PKG)

NX, NY, NZ = 512, 512, 80
DT, NSUB = 6.0, 6
STRETCH = 1.0341247533415947
METRIC = "dyn-step cell-updates/s, mixed vs FP64 on 1 GB300 at stated error vs FP64"
UNIT = "cell-updates/s"
HBM_FALLBACK = 6800.0
RESTART = 20     # timed runs restart from the initial state every RESTART steps
ERR_STEPS = 20   # mixed vs FP64 error after this many steps from the same state


CASE = dict(nz=NZ, dx=1000.0, dy=1000.0, z_top=20000.0, zeta_first=1.0, zeta_stretch=STRETCH,
            ref_kind=1, theta0=300.0, bv_n=0.01, profile_dz=250.0, bubble_amplitude=0.0,
            qv_surface=0.0, u_background=10.0, shear_u=0.0,
            advection=5, weno_scalars=1, weno_advective=1, pgf_perturbation=1, split_fast=1,
            acoustic_mode=2, hevi_beta=0.5, moist=0, coriolis=0)


def case_setup(vg_setup_cls, nx=NX, ny=NY):
    return vg_setup_cls.defaults(nx=nx, ny=ny, **CASE)


# Semi-implicit workload: 256 x 256 x 64, dx = 2 km, 20 km top (uniform
# zeta), Gaussian hill h = 800 m with 10 km half-width, N = 0.01 profile,
# u = 15 m/s, dt = 30 s; the reference's own composition (flags 0).
SI_CASE = dict(nx=256, ny=256, nz=64, dx=2000.0, dy=2000.0, z_top=20000.0, zeta_first=1.0, zeta_stretch=1.0,
               terrain_kind=1, hill_h=800.0, hill_a=10000.0, hill_xc=256000.0, hill_yc=256000.0,
               ref_kind=1, theta0=300.0, bv_n=0.01, profile_dz=250.0, bubble_amplitude=0.0, qv_surface=0.0,
               u_background=15.0, shear_u=0.0, advection=2, weno_scalars=0, weno_advective=0,
               pgf_perturbation=0, split_fast=0, acoustic_mode=0)
SI_DT, SI_TOL = 30.0, 1e-10


def si_leg(vg, steps=3):
    """Helmholtz solve of the semi-implicit step on the 256x256x64 hill case:
    iterations and device time of the mixed solver (FP32 multigrid-BiCGSTAB
    inside FP64 refinement to a relative residual of 1e-10), its error
    against the FP64 solve of the same operator, and what the reference's
    default solver (Jacobi-BiCGSTAB in the refinement wrapper) does on it."""
    s = vg.Setup.defaults(**SI_CASE)
    out = {"workload": "256x256x64 hill (h=800 m, a=10 km), dx=2 km, dt=30 s, N=0.01, u=15 m/s",
           "cells": 256 * 256 * 64, "tol": SI_TOL}
    with vg.Model(s, vg.FP64) as mx, vg.Model(s, vg.FP64) as m64:
        ms, its = [], []
        err_max = err_rms = 0.0
        for step in range(steps + 1):
            it4, res4, x4 = mx.si_step(SI_DT, kind=vg.HZ_MG_BICGSTAB_MIXED, tol=SI_TOL, want_pi=True)
            ms4 = mx.si_stats()[2]
            it3, res3, x3 = m64.si_step(SI_DT, kind=vg.HZ_MG_BICGSTAB_FP64, tol=SI_TOL, want_pi=True)
            ms3 = m64.si_stats()[2]
            if step == 0:
                continue  # first call builds the solvers
            ms.append(ms4)
            its.append(it4)
            d = x4 - x3
            err_max = max(err_max, float(np.abs(d).max() / np.abs(x3).max()))
            err_rms = max(err_rms, float(np.sqrt(np.mean(d * d)) / np.sqrt(np.mean(x3 * x3))))
        out.update({"mixed_solve_ms": float(np.median(ms)), "mixed_iterations": int(np.median(its)),
                    "mixed_residual": res4, "fp64_solve_ms": ms3, "fp64_iterations": it3, "fp64_residual": res3,
                    "mixed_vs_fp64_max_rel_err": err_max, "mixed_vs_fp64_rms_rel_err": err_rms})
    with vg.Model(s, vg.FP64) as mr:
        itr, resr, _ = mr.si_step(SI_DT, kind=vg.HZ_KRYLOV_MULTIGRID)
        out["reference_solver"] = {"kind": "krylov_multigrid (refinement wrapper), max_iter 200, tol 1e-8",
                                   "iterations": itr, "residual": resr if np.isfinite(resr) else str(resr),
                                   "solve_ms": mr.si_stats()[2]}
    return out


# Physics coupling: the single-domain workload with the moisture species
# prognostic (qv from 0.025 at the ground, decaying over 2.5 km: saturated
# near the ground, so the saturation adjustment condenses from the first step)
# and the built-in Kessler warm-rain package at every RK stage (column
# pressure from the total Exner function); mixed path, 10 steps each way.
def physics_leg(vg, torch, steps=10, warmup=3, nx=NX, ny=NY):
    s = vg.Setup.defaults(nx=nx, ny=ny, **dict(CASE, moist=1, qv_surface=0.025, qv_decay_height=2500.0))
    k = vg.Kessler.defaults(exner_offset=0)
    out = {"workload": "%dx%dx%d, moist (qv_surface 0.025, 2.5 km decay), Kessler warm rain at every RK stage, "
                       "mixed path, dt=%g s, %d substeps" % (nx, ny, NZ, DT, NSUB), "steps": steps}
    with vg.Model(s, vg.MIXED) as m:
        m.save_snapshot()
        ext = torch.cuda.ExternalStream(m.stream())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ms = {}
        for phys in (False, True):
            m.set_physics_kessler(k if phys else None)
            m.restore_snapshot()
            m.step(DT, NSUB, warmup)  # eager step + graph capture
            m.restore_snapshot()
            m.sync()
            e0.record(ext)
            m.step_async(DT, NSUB, steps)
            e1.record(ext)
            m.sync()
            ms[phys] = e0.elapsed_time(e1) / steps
        qc = vg.interior(s, 7, m.get(7))
        m.set_physics_kessler(None)
    cells = nx * ny * NZ
    out.update({"ms_per_step_dynamics_only": ms[False], "ms_per_step_with_kessler": ms[True],
                "kessler_ms_per_stage": (ms[True] - ms[False]) / 3.0,
                "value": cells / (ms[True] * 1e-3), "unit": "cell-updates/s", "max_qc_after": float(qc.max())})
    return out


# Batched nests: 8 members, each a 384 x 384 x 60 parent at 3 km with two
# r = 3 two-way nests at 1 km (193 x 193 x 60 and 130 x 241 x 60), Davies
# zone 5 points; 60 levels stretched from a 50 m first layer to the 20 km top
# (ratio 1.0530384502435775); the single-domain base state (theta0 = 300 K,
# N = 0.01 1/s, u = 10 m/s); members differ by seeded theta' ~ N(0, 0.3 K)
# and u' ~ N(0, 0.5 m/s). Parent dt = 18 s, nest dt = 6 s, 6 substeps per stage.
NEST_NZ, NEST_STRETCH, NEST_DT, NEST_MEMBERS = 60, 1.0530384502435775, 18.0, 8
NEST_PARENT = (384, 384, 3000.0)
NEST_CHILDREN = [  # (nx, ny, interp (i0, j0) in nest points, restrict box (i0, j0, iext, jext) in parent points)
    (193, 193, (180, 180), (60, 60, 64, 64)),
    (130, 241, (660, 600), (220, 200, 43, 80)),
]


def nest_leg(vg, torch, warmup, steps=4):
    """One parent step of all 8 members with their nests = one CUDA graph
    (parents of all members in one work-list launch per kernel, nests of all
    members in another, transfers between)."""
    case = dict(CASE, nz=NEST_NZ, zeta_stretch=NEST_STRETCH)
    base = {k: v for k, v in case.items() if k not in ("dx", "dy")}
    ps = vg.Setup.defaults(nx=NEST_PARENT[0], ny=NEST_PARENT[1], dx=NEST_PARENT[2], dy=NEST_PARENT[2], **base)
    cs = [vg.Setup.defaults(nx=nx, ny=ny, dx=1000.0, dy=1000.0, **base) for nx, ny, _, _ in NEST_CHILDREN]
    pl_i, pl_r = [], []
    for nx, ny, (ii, jj), (ri, rj, re, rf) in NEST_CHILDREN:
        a, b = vg.NestPlacement(), vg.NestPlacement()
        a.i0, a.j0, a.ratio, a.boundary_zone, a.two_way = ii, jj, 3, 5, 1
        b.i0, b.j0, b.iext, b.jext, b.ratio, b.boundary_zone, b.two_way = ri, rj, re, rf, 3, 5, 1
        pl_i.append(a)
        pl_r.append(b)
    parents, children, parent_of, ip, rp = [], [], [], [], []
    staggers = [1, 2, 3, 0, 0, 0, 0]
    for mbr in range(NEST_MEMBERS):
        rng = np.random.default_rng(100 + mbr)
        p = vg.Model(ps, vg.MIXED)
        th, u, rho = p.get(4), p.get(0), p.get(3)
        th = th + np.where(th != 0.0, rng.normal(0.0, 0.3, th.size), 0.0)
        u = u + np.where(u != 0.0, rng.normal(0.0, 0.5, u.size), 0.0)
        # pi from the equation of state (dry), as the single-domain set-up
        pi = np.where(rho != 0.0, np.power(np.maximum(rho * 287.05 * th / 100000.0, 0.0), 287.05 / 717.63), 0.0)
        p.set(4, th)
        p.set(0, u)
        p.set(5, pi)
        parents.append(p)
        pst = [p.get(q) for q in range(7)]
        for c, s in enumerate(cs):
            m = vg.Model(s, vg.MIXED)
            cst = [m.get(q) for q in range(7)]
            vg.nest_interpolate_from_parent(pl_i[c], staggers, (ps.nx, ps.ny, ps.nz), pst, (s.nx, s.ny, s.nz),
                                            cst)
            for q in range(7):
                m.set(q, cst[q])
            children.append(m)
            parent_of.append(mbr)
            ip.append(pl_i[c])
            rp.append(pl_r[c])
    cells = NEST_MEMBERS * (ps.nx * ps.ny * NEST_NZ + 3 * sum(s.nx * s.ny * NEST_NZ for s in cs))
    n = vg.Nested(parents, children, parent_of, ip, rp)
    try:
        for m in parents + children:
            m.save_snapshot()
        n.step(NEST_DT, NSUB, warmup)
        for m in parents + children:  # restart from the initial states (the noise grows convectively)
            m.restore_snapshot()
            m.sync()
        ext = torch.cuda.ExternalStream(n.stream())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(ext)
        n.step_async(NEST_DT, NSUB, steps)
        e1.record(ext)
        n.wait()
        ms = e0.elapsed_time(e1)
        launches = n.launches_per_step()
    finally:
        n.close()
        for m in parents + children:
            m.close()
    return {"workload": "8 members x (384x384x60 parent at 3 km + r=3 two-way nests 193x193x60 and 130x241x60 at "
                        "1 km, Davies zone 5), theta'~N(0,0.3 K), u'~N(0,0.5 m/s); parent dt=18 s, nest dt=6 s, "
                        "6 HEVI substeps per stage; one CUDA graph per parent step",
            "cell_updates_per_parent_step": cells, "parent_steps": steps, "ms_per_parent_step": ms / steps,
            "value": cells * steps / (ms * 1e-3), "unit": UNIT, "gpu_launches_per_parent_step": launches,
            "hevi_columns_per_parent_launch": NEST_MEMBERS * ps.nx * ps.ny}


# Assimilation window: 192 x 192 x 50, dx = 3 km, 50 uniform 400 m levels to
# 20 km, the single-domain base state (theta0 = 300 K, N = 0.01 1/s,
# u = 10 m/s) plus seeded theta' ~ N(0, 0.3 K), u' ~ N(0, 0.5 m/s); 120 model
# steps of dt = 15 s (6 HEVI substeps per stage), checkpoints every 10 steps.
# The TL/AD (the reference's collocated RK3 with explicit acoustics) is
# stable only below ~1.4 s on this grid, so it takes 12 steps of 1.25 s per
# model step. TL input dx ~ N(0, 1) scaled: u, v 1 m/s, w 0.1 m/s, theta
# 0.5 K, pi' from a 50 Pa pressure perturbation (pi' = kappa pi0 p'/p0(z)).
WIN = dict(nx=192, ny=192, nz=50, dx=3000.0, dt=15.0, n_steps=120, every=10, tl_sub=12)


def ckernels_leg(vg, torch, reps=10, warmup=3):
    """The C-ABI kernels (include/vibe_c_kernels.h, device-pointer forms) on
    inputs larger than L2, each timed with CUDA events on the calling stream
    over `reps` calls after `warmup`: algorithmic bytes (every input read once,
    every output written once) per call over the call's time."""
    import ctypes
    vp, i32, f64, sz = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_size_t
    lib = ctypes.CDLL(vg.lib._name)  # a handle of its own: its argument types stay here
    sigs = {"vibe_tridiagonal_solve_batched_f64_dev": [vp] * 4 + [i32, i32, vp, vp, vp],
            "vibe_weno5_reconstruct_batched_f64_dev": [vp, sz, vp, vp, vp],
            "vibe_cfl_scan_f64_dev": [vp] * 5 + [i32] * 3 + [f64] * 4 + [vp, vp],
            "vibe_neumaier_sum_f64_dev": [vp, sz, vp, vp],
            "vibe_advect_scalar_flux_f64_dev": [vp] * 7 + [i32] * 3 + [f64] * 3 + [vp, vp]}
    fn = {}
    for name, args in sigs.items():
        f = getattr(lib, name)
        f.restype, f.argtypes = i32, args
        fn[name] = f
    dev = torch.device("cuda", torch.cuda.current_device())
    st = torch.cuda.Stream(dev)
    h = st.cuda_stream
    peak, kind = measured_peak()
    gen = torch.Generator(device=dev).manual_seed(5)
    rnd = lambda *shape: torch.rand(*shape, dtype=torch.float64, device=dev, generator=gen)  # noqa: E731

    def timed(call, nbytes, what):
        for _ in range(warmup):
            assert call() == 0, what
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(dev)
        e0.record(st)
        for _ in range(reps):
            call()
        e1.record(st)
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1) / reps
        gbs = nbytes / (ms * 1e-3) / 1e9
        return {"workload": what, "ms": ms, "bytes": nbytes, "gbs": gbs, "frac": gbs / peak}

    out = {"peak_gbs": peak, "peak_kind": kind, "reps": reps}
    nx, ny, nz = NX, NY, NZ
    with torch.cuda.stream(st):
        for n, n_sys in ((NZ, nx * ny), (200, 65536)):  # a column of the workload; a tall system (warp per system)
            a, c = -rnd(n_sys, n - 1), -rnd(n_sys, n - 1)
            b, d = 4.0 + rnd(n_sys, n), rnd(n_sys, n)
            x = torch.empty_like(b)
            f = fn["vibe_tridiagonal_solve_batched_f64_dev"]
            key = "thomas_batched_n%d" % n
            out[key] = timed(lambda: f(a.data_ptr(), b.data_ptr(), c.data_ptr(), d.data_ptr(), n, n_sys,
                                       x.data_ptr(), None, h),
                             8 * (2 * (n - 1) + 3 * n) * n_sys, "%d systems of %d rows" % (n_sys, n))
            del a, b, c, d, x
        nf = 16 * 1024 * 1024
        q, ql, qr = rnd(5 * nf), torch.empty(nf, dtype=torch.float64, device=dev), \
            torch.empty(nf, dtype=torch.float64, device=dev)
        f = fn["vibe_weno5_reconstruct_batched_f64_dev"]
        out["weno5_batched"] = timed(lambda: f(q.data_ptr(), nf, ql.data_ptr(), qr.data_ptr(), h), 56 * nf,
                                     "%d stencils" % nf)
        del q, ql, qr
        n = nx * ny * nz
        u, v, w = 20.0 * rnd(n) - 10.0, 20.0 * rnd(n) - 10.0, rnd(n) - 0.5
        dz, zs = 0.01 + 0.01 * rnd(nz), 500.0 * rnd(nx * ny)
        o3 = torch.empty(3, dtype=torch.float64, device=dev)
        f = fn["vibe_cfl_scan_f64_dev"]
        out["cfl_scan"] = timed(lambda: f(u.data_ptr(), v.data_ptr(), w.data_ptr(), dz.data_ptr(), zs.data_ptr(),
                                          nx, ny, nz, 1000.0, 1000.0, 20000.0, 6.0, o3.data_ptr(), h),
                                24 * n + 8 * (nx * ny + nz), "%dx%dx%d cells" % (nx, ny, nz))
        qq, rho, dq = rnd(n), 1.0 + rnd(n), torch.empty(n, dtype=torch.float64, device=dev)
        f = fn["vibe_advect_scalar_flux_f64_dev"]
        out["advect_scalar_flux"] = timed(
            lambda: f(qq.data_ptr(), rho.data_ptr(), u.data_ptr(), v.data_ptr(), w.data_ptr(), dz.data_ptr(),
                      zs.data_ptr(), nx, ny, nz, 1000.0, 1000.0, 20000.0, dq.data_ptr(), h),
            48 * n + 8 * (nx * ny + nz), "%dx%dx%d cells" % (nx, ny, nz))
        del u, v, w, qq, rho, dq
        ns = 64 * 1024 * 1024
        xs, s = rnd(ns), torch.empty(1, dtype=torch.float64, device=dev)
        f = fn["vibe_neumaier_sum_f64_dev"]
        out["neumaier_sum"] = timed(lambda: f(xs.data_ptr(), ns, s.data_ptr(), h), 8 * ns, "%d doubles" % ns)
        del xs
    return out


def window_leg(vg, torch):
    case = {k: v for k, v in CASE.items() if k not in ("dx", "dy", "nz", "zeta_stretch", "hevi_beta")}
    s = vg.Setup.defaults(nx=WIN["nx"], ny=WIN["ny"], nz=WIN["nz"], dx=WIN["dx"], dy=WIN["dx"], zeta_stretch=1.0,
                          w_rigid=1, hevi_beta=0.6, **case)
    out = {"workload": "192x192x50 (dx=3 km, 400 m levels), dt=15 s x 120 steps, checkpoints every 10 steps; "
                       "trajectory from the base state plus the single-domain case's seeded perturbations "
                       "(20 bubbles, theta' noise below 1 km), rigid ground and lid, HEVI off-centred (beta 0.6); "
                       "model_step: the TL/AD of the model's own step, one per model step; the rest: the "
                       "reference's collocated TL/AD at 12 x 1.25 s per step",
           "tl_substeps": WIN["tl_sub"], "tl_dt_s": WIN["dt"] / WIN["tl_sub"]}
    kappa = 287.05 / 1004.5

    def model_and_vectors(prec):
        m = vg.Model(s, prec)
        th, pi = perturbed_state(s, m.get(4), m.get(3), m.zeta(), seed=5, nx_full=s.nx, ny_full=s.ny)
        m.set(4, th)
        m.set(5, pi)
        pi0 = vg.interior(s, 5, m.reffield(1))  # reference Exner function and pressure
        vecs = []
        for seed in (11, 12):
            r = np.random.default_rng(seed)
            v = [np.zeros(m.size(sp)) for sp in range(12)]
            for sp, amp in ((0, 1.0), (1, 1.0), (2, 0.1), (4, 0.5)):
                vg.interior(s, sp, v[sp])[...] = amp * r.standard_normal(vg.interior(s, sp, v[sp]).shape)
            p0 = vg.interior(s, 5, m.reffield(3))
            vg.interior(s, 5, v[5])[...] = kappa * pi0 * 50.0 * r.standard_normal(pi0.shape) / p0
            vecs.append(v)
        return m, vecs[0], vecs[1]

    def vdot(a, b):
        return sum(float(np.sum(vg.interior(s, sp, a[sp]) * vg.interior(s, sp, b[sp]))) for sp in range(12))

    cells = s.nx * s.ny * s.nz
    # the model's own step (slow tendency, HEVI substeps, sponge): one TL/AD
    # step per 15 s model step, checkpoints with recomputation
    own = {"what": "TL/AD of the model's own step (vibe_gb300_step_tl/_ad composed over the window, "
                   "vibe_gb300_window_* with tlad = NULL): WENO5 advective-form scalars with exact weight "
                   "derivatives, momentum, buoyancy, pi' pressure gradient, consistent HEVI substeps, sponge; "
                   "one TL/AD step per model step (no sub-stepping)"}
    for name, prec, tol in (("fp64", vg.FP64, 1e-10), ("mixed", vg.MIXED, 1e-5)):
        m, dx, dy = model_and_vectors(prec)
        try:
            with vg.Window(m, None, WIN["dt"], NSUB, WIN["n_steps"], WIN["every"]) as w:
                ldx = w.tl(dx)
                tl_ms = w.stats()[0]
                ady = w.ad(dy)
                ad_ms, ck, sg = w.stats()
            lhs, rhs = vdot(ldx, dy), vdot(dx, ady)
            res = {"tl_window_ms": tl_ms, "ad_window_ms": ad_ms, "dot_lhs": lhs, "dot_rhs": rhs,
                   "dot_rel_err": abs(lhs - rhs) / max(abs(lhs), abs(rhs)), "dot_tol": tol,
                   "tl_cell_steps_per_s": cells * WIN["n_steps"] / (tl_ms * 1e-3),
                   "ad_cell_steps_per_s": cells * WIN["n_steps"] / (ad_ms * 1e-3),
                   "checkpoint_bytes": ck, "segment_bytes": sg}
            if name == "fp64":
                # (M(x + e dx) - M(x)) / e against the window TL, M = the 120 nonlinear steps
                x0 = m.state()
                m.step(WIN["dt"], NSUB, WIN["n_steps"])
                mx = m.state()
                nl = np.sqrt(vdot(ldx, ldx))
                fd = {}
                for k in range(2, 12):
                    e = 10.0 ** -k
                    m.set_state([a + e * b for a, b in zip(x0, dx)])
                    m.step(WIN["dt"], NSUB, WIN["n_steps"])
                    d = [(a - b) / e - c for a, b, c in zip(m.state(), mx, ldx)]
                    fd["%.0e" % e] = np.sqrt(vdot(d, d)) / nl
                m.set_state(x0)
                res["fd_window_rel_err"] = fd
            own[name] = res
        finally:
            m.close()
    out["model_step"] = own
    out["collocated_reference_check"] = "the reference's own TL/AD (tangent_linear.cpp: collocated RK3 " \
                                        "without acoustic substeps) over the same trajectory: fp64 / mixed below"
    for name, prec, tprec, tol in (("fp64", vg.FP64, 0, 1e-10), ("mixed", vg.MIXED, 1, 1e-5)):
        m, dx, dy = model_and_vectors(prec)
        t = vg.TLAD(s.nx, s.ny, s.nz, s.dx, s.dy, s.z_top, np.diff(m.zeta()), m.terrain(), tprec)
        w = vg.Window(m, t, WIN["dt"], NSUB, WIN["n_steps"], WIN["every"], WIN["tl_sub"])
        try:
            ldx = w.tl(dx)
            tl_ms = w.stats()[0]
            ady = w.ad(dy)
            ad_ms, ck, sg = w.stats()
        finally:
            w.close()
        lhs, rhs = vdot(ldx, dy), vdot(dx, ady)
        tl_steps = WIN["n_steps"] * WIN["tl_sub"]
        res = {"tl_window_ms": tl_ms, "ad_window_ms": ad_ms, "dot_lhs": lhs, "dot_rhs": rhs,
               "dot_rel_err": abs(lhs - rhs) / max(abs(lhs), abs(rhs)), "dot_tol": tol,
               "tl_cell_steps_per_s": cells * tl_steps / (tl_ms * 1e-3),
               "ad_cell_steps_per_s": cells * tl_steps / (ad_ms * 1e-3),
               "checkpoint_bytes": ck, "segment_bytes": sg,
               "model_steps": {"tl": WIN["n_steps"] - 1, "ad": 2 * WIN["n_steps"] - WIN["n_steps"] // WIN["every"]}}
        if name == "fp64":
            # finite differences of the nonlinear collocated tendency against the TL tendency
            x0 = m.state()
            t.set_base(x0)
            f = t.tl_tendency(dx)
            n0 = t.nl_tendency(x0)
            nf = np.sqrt(sum(float(np.sum(a * a)) for a in f))
            fd = {}
            for k in range(3, 9):
                e = 10.0 ** -k
                n1 = t.nl_tendency([a + e * b for a, b in zip(x0, dx)])
                d = sum(float(np.sum(((a - b) / e - c) ** 2)) for a, b, c in zip(n1, n0, f))
                fd["%.0e" % e] = np.sqrt(d) / nf
            res["fd_tendency_rel_err"] = fd
        out[name] = res
        t.close()
        m.close()
    return out


def field_errors(vg, setup, got, ref):
    """Per-field max and RMS error of got against ref over the interior,
    relative to the field's max |ref| (u, v, w: the common velocity scale)."""
    ins = [vg.interior(setup, sp, ref[sp]) for sp in range(7)]
    vscale = max(float(np.abs(ins[sp]).max()) for sp in range(3))
    out = {}
    for sp in range(7):
        d = vg.interior(setup, sp, got[sp]) - ins[sp]
        scale = vscale if sp < 3 else float(np.abs(ins[sp]).max())
        if scale == 0.0:
            out[vg.SPECIES[sp]] = {"max_abs": float(np.abs(d).max())}
            continue
        out[vg.SPECIES[sp]] = {"max_rel": float(np.abs(d).max() / scale),
                               "rms_rel": float(np.sqrt(np.mean(d * d)) / scale)}
    return out


def perturbed_state(setup, theta, rho, zeta, seed=1, nx_full=NX, ny_full=NY, x_off=0, y_off=0, noise=0.5):
    """theta/pi storage arrays with the seeded perturbations (numpy set-up)."""
    rng = np.random.default_rng(seed)
    h = 4
    th = theta.reshape(setup.nz + 8, setup.ny + 8, setup.nx + 8).copy()
    r = rho.reshape(setup.nz + 8, setup.ny + 8, setup.nx + 8)
    zc = 0.5 * (zeta[:-1] + zeta[1:]) * setup.z_top
    nz = setup.nz
    noise = rng.uniform(-noise, noise, size=(nz, ny_full, nx_full))
    low = zc < 1000.0
    x = (np.arange(setup.nx) + x_off + 0.5) * setup.dx
    y = (np.arange(setup.ny) + y_off + 0.5) * setup.dy
    interior = th[h:h + nz, h:h + setup.ny, h:h + setup.nx]
    interior[low] += noise[low][:, y_off:y_off + setup.ny, x_off:x_off + setup.nx]
    amp = rng.uniform(1.0, 3.0, 20)
    rad = rng.uniform(1000.0, 4000.0, 20)
    xc = rng.uniform(0.0, nx_full * setup.dx, 20)
    yc = rng.uniform(0.0, ny_full * setup.dy, 20)
    zcen = rng.uniform(1000.0, 5000.0, 20)
    for b in range(20):  # cos^2 bubbles as init_warm_bubble (initial_conditions.cpp:144-156)
        ix = np.nonzero(np.abs(x - xc[b]) < rad[b])[0]
        iy = np.nonzero(np.abs(y - yc[b]) < rad[b])[0]
        iz = np.nonzero(np.abs(zc - zcen[b]) < rad[b])[0]
        if not (ix.size and iy.size and iz.size):
            continue
        Z, Y, X = np.meshgrid(zc[iz], y[iy], x[ix], indexing="ij")
        r2 = ((X - xc[b]) / rad[b]) ** 2 + ((Y - yc[b]) / rad[b]) ** 2 + ((Z - zcen[b]) / rad[b]) ** 2
        c = np.cos(0.5 * np.pi * np.sqrt(np.minimum(r2, 1.0)))
        sub = interior[iz[0]:iz[-1] + 1, iy[0]:iy[-1] + 1, ix[0]:ix[-1] + 1]
        sub += np.where(r2 < 1.0, amp[b] * c * c, 0.0)
    # enforce_state_equation (initial_conditions.cpp:110-121), dry: gamma_f = 1
    val = r[h:h + nz, h:h + setup.ny, h:h + setup.nx] * 287.05 * interior / 100000.0
    pi = np.zeros_like(th)
    pi[h:h + nz, h:h + setup.ny, h:h + setup.nx] = np.power(val, 287.05 / 717.63)
    return th.ravel(), pi.ravel()


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during a region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            time.sleep(0.3)
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) == 7:
                self.rows.append(parts)

    def __exit__(self, *exc):
        if self.proc:
            time.sleep(0.2)
            self.proc.terminate()
            self.proc.wait(timeout=5)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[c] for r in self.rows for c in range(4) if r[3 + c].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return HBM_FALLBACK, "fallback"


def traffic_of(kernel, cells):
    """DRAM bytes per launch of `kernel` scaled to `cells`, from the committed
    ncu summary profiles/dram_traffic.md (rows "| kernel | cells | bytes per
    launch |"), or None when the summary has no row for it."""
    p = os.path.join(ROOT, "profiles", "dram_traffic.md")
    try:
        with open(p) as f:
            for line in f:
                cols = [c.strip() for c in line.strip().strip("|").split("|")]
                if len(cols) >= 3 and cols[0] == kernel:
                    return float(cols[2]) * cells / float(cols[1])
    except (OSError, ValueError):
        return None
    return None


# ---- CPU baseline / reference arm (oracle port on host cores) ---------------
def _oracle():
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_ctypes as oc
    if not os.path.exists(oc.PORT_SO):
        subprocess.run(["make", "-C", oc.ORACLE_DIR, "-s"], check=True)
    return oc


def cpu_sample_run(args, record=None):
    """One worker: steps a horizontal sample of the workload on the oracle
    port (the reference's serial FP64 algorithm). Returns (cells, seconds).
    record: a dict that receives the sample's state before and after the
    first timed step (the checker for mixed_vs_oracle_error)."""
    nx, ny, steps, warmup, seed = args[:5]
    y_off = args[5] if len(args) > 5 else 0  # rows of the 512 x 512 domain before this sample
    oc = _oracle()
    s = oc.defaults()
    for k, v in dict(CASE, nx=nx, ny=ny).items():
        setattr(s, k, v)
    m = oc.Model(s, "port")
    th, pi = perturbed_state(s, m.get(4), m.get(3), m.zeta(), seed=seed, x_off=0, y_off=y_off)
    m.set(4, th)
    m.set(5, pi)
    for _i in range(warmup):
        m.rk3_step(DT, NSUB)
    secs = 0.0
    for i in range(steps):
        if record is not None and i == 0:
            record["x0"] = [m.get(q) for q in range(7)]
        t0 = time.perf_counter()
        m.rk3_step(DT, NSUB)
        secs += time.perf_counter() - t0
        if record is not None and i == 0:
            record["x1"] = [m.get(q) for q in range(7)]
    return nx * ny * NZ * steps, secs


def oracle_errors(vg, nx, ny, record):
    """Per-field max / RMS relative error of one GPU step (mixed and FP64)
    from the oracle's state, against the oracle's next state, on the CPU
    baseline's sample of the workload (each field over its own scale,
    velocities over the common velocity scale; qv, zero in the dry case,
    absolutely)."""
    s = case_setup(vg.Setup, nx, ny)
    x0, x1 = record["x0"], record["x1"]
    ins = [vg.interior(s, q, x1[q]) for q in range(7)]
    vs = max(float(np.abs(ins[q]).max()) for q in range(3))
    out = {"sample": "%dx%dx%d horizontal sample of the workload (the CPU baseline's), one step from the "
                     "oracle's state" % (nx, ny, NZ)}
    for prec, name in ((vg.MIXED, "mixed"), (vg.FP64, "fp64")):
        with vg.Model(s, prec) as m:
            for q in range(7):
                m.set(q, x0[q])
            m.step(DT, NSUB, 1)
            got = m.state()[:7]
        fields = {}
        for q in range(7):
            scale = vs if q < 3 else float(np.abs(ins[q]).max())
            scale = scale if scale > 0.0 else 1.0
            d = vg.interior(s, q, got[q]) - ins[q]
            fields[vg.SPECIES[q]] = {"max_rel": float(np.abs(d).max()) / scale,
                                     "rms_rel": float(np.sqrt(np.mean(d * d))) / scale}
        out[name] = {"max_rel": max(f["max_rel"] for f in fields.values()), "fields": fields}
    return out


# The CPU-runnable warm-bubble case (64 x 64 x 40, dx = dy = dz = 250 m,
# +2 K bubble of 2 km radius at (8, 8, 2) km, WENO5 scalars, dt = 2 s, 6
# substeps): its single-core oracle rate is reported beside the bench line.
CONFIG1 = dict(nx=64, ny=64, nz=40, dx=250.0, dy=250.0, z_top=10000.0, zeta_first=1.0, zeta_stretch=1.0,
               ref_kind=0, theta0=300.0, p_surf=100000.0, bubble_amplitude=2.0, bubble_radius_x=2000.0,
               bubble_radius_z=2000.0, bubble_xc=8000.0, bubble_yc=8000.0, bubble_zc=2000.0, qv_surface=0.0,
               advection=5, weno_scalars=1, weno_advective=1, pgf_perturbation=1, split_fast=1, acoustic_mode=0,
               u_background=0.0, shear_u=0.0)


def cpu_config1_run(steps=3):
    oc = _oracle()
    s = oc.defaults()
    for k, v in CONFIG1.items():
        setattr(s, k, v)
    m = oc.Model(s, "port")
    t0 = time.perf_counter()
    for _ in range(steps):
        m.rk3_step(2.0, 6)
    return 64 * 64 * 40 * steps, time.perf_counter() - t0


def reference_arm(args):
    """The reference's CPU path (the oracle port, the reference's serial FP64
    algorithm) on every host core over the GPU arm's workload itself: the
    512 x 512 x 80 domain with the rank-0 member's perturbations, cut into
    one strip of whole rows per core (each strip a model with its own lateral
    boundaries, the same work per cell as the whole domain)."""
    import multiprocessing as mp
    cores = os.cpu_count() or 1
    rows = -(-NY // cores)
    strips = [(y0, min(rows, NY - y0)) for y0 in range(0, NY, rows)]
    # a whole-domain step takes seconds on the host cores: at most 10 timed
    # steps after one warm-up step keep the run within a few minutes
    steps, warmup = min(args.steps, 10), min(args.warmup, 1)
    with mp.get_context("spawn").Pool(len(strips)) as pool:
        t0 = time.perf_counter()
        res = pool.map(cpu_sample_run, [(NX, h, steps, warmup, member_seed(0), y0) for (y0, h) in strips])
        wall = time.perf_counter() - t0
    cells = sum(r[0] for r in res)
    secs = max(r[1] for r in res)
    value = cells / secs
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": steps, "warmup": warmup, "ms_per_step": 1e3 * secs / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "512x512x80 single domain, dx=1km, dt=6s, 6 substeps/stage (the whole domain "
                               "in %d strips of %d rows, one per core)" % (len(strips), rows),
                   "same_config": True},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": len(strips), "kind": "port",
                         "sample": "the whole 512x512x80 workload as %d strips of %dx%dx%d (last %d rows), one "
                                   "per core, %d timed steps each (wall %.1f s)"
                                   % (len(strips), NX, rows, NZ, strips[-1][1], steps, wall)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


# ---- ranks: one process per GPU, each advancing its own replica -------------
class Ranks:
    """Replica ranks under torchrun (weak scaling: every rank advances its own
    ensemble member). The data path has no collective; the only ones are the
    timing barrier and the max over ranks of the timed region."""

    def __init__(self, world, rank, backend="nccl", device=None):
        import torch
        self.torch = torch
        self.world, self.rank, self.device = world, rank, device
        self.dist = None
        if world > 1:
            import torch.distributed as dist
            if backend == "nccl":
                dist.init_process_group("nccl", device_id=device)
            else:
                dist.init_process_group(backend)
            self.dist = dist

    def barrier(self):
        if self.dist is not None:
            self.dist.barrier()
        if self.device is not None and self.device.type == "cuda":
            self.torch.cuda.synchronize()

    def max(self, x):
        if self.dist is None:
            return x
        t = self.torch.tensor([x], dtype=self.torch.float64, device=self.device or "cpu")
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.dist is not None:
            self.dist.destroy_process_group()
            self.dist = None


def member_seed(rank):
    """Seed of the perturbations of the replica a rank advances."""
    return 1 + rank


def whole_job_rate(world, cells, steps, ms_max):
    """Cell-updates/s of all ranks together over the slowest rank's time."""
    return world * cells * steps / (ms_max * 1e-3)


# ---- GPU arm -----------------------------------------------------------------
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--nx", type=int, default=NX, help="domain size (profiling runs use smaller cases)")
    ap.add_argument("--ny", type=int, default=NY)
    ap.add_argument("--no-si", action="store_true", help="skip the semi-implicit (Helmholtz) leg")
    ap.add_argument("--no-nest", action="store_true", help="skip the batched nests leg")
    ap.add_argument("--no-window", action="store_true", help="skip the TL/AD assimilation-window leg")
    ap.add_argument("--no-tune", action="store_true", help="skip the autotuner (built-in launch shapes)")
    ap.add_argument("--no-physics", action="store_true", help="skip the Kessler physics-coupling leg")
    ap.add_argument("--no-ckernels", action="store_true", help="skip the C-ABI kernel leg")
    ap.add_argument("--only", choices=["all", "mixed", "fp64", "physics", "nest", "si", "window", "ckernels"],
                    default="all",
                    help="mixed / fp64: time that path only (no e2e, no other legs); physics / nest / si / "
                         "window / ckernels: that leg only")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank == 0:
            reference_arm(args)
        return

    # CPU baseline first (rank 0 at N=1 only), before any CUDA work
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        oracle_record = {}
        cells, secs = cpu_sample_run((128, 128, 2, 0, 1), oracle_record)
        cpu = {"value": cells / secs, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": "128x128x80 horizontal sample of the workload, 2 RK3 steps, single thread (%.1f s)" % secs}
        c1, s1 = cpu_config1_run()
        cpu["warm_bubble_64x64x40"] = {"value": c1 / s1, "unit": UNIT, "cores": 1,
                                       "sample": "3 RK3 steps (dt 2 s, 6 substeps), single thread (%.1f s)" % s1}

    import torch
    torch.cuda.set_device(local)
    ranks = Ranks(world, rank, "nccl", torch.device("cuda", local))
    barrier, max_over_ranks = ranks.barrier, ranks.max

    import vibe_gb300 as vg
    if args.only == "physics":
        print(json.dumps({"only": "physics", "physics_coupling": physics_leg(vg, torch, nx=args.nx, ny=args.ny)}))
        ranks.close()
        return
    if args.only == "nest":
        print(json.dumps({"only": "nest", "batched_nests": nest_leg(vg, torch, args.warmup)}))
        ranks.close()
        return
    if args.only == "si":
        print(json.dumps({"only": "si", "semi_implicit": si_leg(vg)}))
        ranks.close()
        return
    if args.only == "window":
        print(json.dumps({"only": "window", "assimilation_window": window_leg(vg, torch)}))
        ranks.close()
        return
    if args.only == "ckernels":
        print(json.dumps({"only": "ckernels", "c_abi_kernels": ckernels_leg(vg, torch)}))
        ranks.close()
        return
    setup = case_setup(vg.Setup, args.nx, args.ny)
    cells = args.nx * args.ny * NZ

    def make(prec):
        m = vg.Model(setup, prec)
        th, pi = perturbed_state(setup, m.get(4), m.get(3), m.zeta(), seed=member_seed(rank),
                                 nx_full=args.nx, ny_full=args.ny)
        m.set(4, th)
        m.set(5, pi)
        m.save_snapshot()  # the initial state, kept on the device
        return m

    def timed_steps(m, k):
        """k steps from the initial state; every RESTART steps the state is put
        back from the device snapshot (inside the timed region): the workload's
        superadiabatic noise makes it blow up after ~25 steps in FP64 too."""
        ext = torch.cuda.ExternalStream(m.stream())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        m.restore_snapshot()
        barrier()
        e0.record(ext)
        done = 0
        while done < k:
            c = min(RESTART, k - done)
            if done:
                m.restore_snapshot()
            m.step_async(DT, NSUB, c)
            done += c
        e1.record(ext)
        m.sync()
        barrier()
        return e0.elapsed_time(e1), (k - 1) // RESTART

    if args.only == "fp64":  # the plain FP64 path alone (profiling runs)
        f64 = make(vg.FP64)
        f64.step(DT, NSUB, 1)
        ms_64, _ = timed_steps(f64, args.steps)
        f64.set_kernel_timing(True)
        ms_kt, _ = timed_steps(f64, 2)
        ktimes = f64.kernel_times()
        f64.close()
        print(json.dumps({"only": "fp64", "cells": cells, "ms_per_step": ms_64 / args.steps,
                          "value": world * cells * args.steps / (ms_64 * 1e-3), "kernel_ms": ktimes,
                          "eager_ms_per_step": ms_kt / 2}))
        ranks.close()
        return

    # ---- mixed path (the headline) ----
    mx = make(vg.MIXED)
    # launch shapes for this grid (same update, FP32 rounding aside)
    tuning = None if args.no_tune else mx.autotune(DT, NSUB)
    mx.step(DT, NSUB, args.warmup)  # the first step runs eagerly, the next capture the step graphs
    with ClockSampler(local) as clk:
        ms_mx, restarts = timed_steps(mx, args.steps)  # graph replay
    ms_mx = max_over_ranks(ms_mx)
    # per-kernel-class device times (event spans; eager launches) for the roofline
    mx.set_kernel_timing(True)
    kt_steps = max(2, min(5, args.steps))
    ms_kt, _ = timed_steps(mx, kt_steps)
    ktimes = mx.kernel_times()
    mx.set_kernel_timing(False)
    launches = mx.launches_per_step(NSUB) * args.steps + restarts  # + one to_working per restart

    if args.only == "mixed":
        mx.close()
        print(json.dumps({"only": "mixed", "cells": cells, "ms_per_step": ms_mx / args.steps,
                          "value": world * cells * args.steps / (ms_mx * 1e-3), "kernel_ms": ktimes,
                          "eager_ms_per_step": ms_kt / kt_steps}))
        return
    # ---- end to end through the public API with host buffers: every step
    # uploads its input state from pinned host memory and reads its result
    # back (vibe_gb300_step_io: uploads, steps and downloads of consecutive
    # steps overlap on three streams)
    mx.restore_snapshot()
    pin_in = [torch.empty(mx.size(sp), dtype=torch.float64, pin_memory=True) for sp in range(7)]
    pin_out = [torch.empty(mx.size(sp), dtype=torch.float64, pin_memory=True) for sp in range(7)]
    p_in, p_out = [p.data_ptr() for p in pin_in], [p.data_ptr() for p in pin_out]
    mx.get_state_ptrs(p_in)
    mx.sync()
    # every step starts from the same host input, so the run can be long
    # enough that the pipeline's fill (the first upload) and drain (the last
    # download) do not dominate
    e2e_steps = max(6, 2 * args.steps)
    ext = torch.cuda.ExternalStream(mx.stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    mx.step_io(p_in, p_out, DT, NSUB)  # sets up the pipeline's streams and staging buffers
    mx.sync()
    barrier()
    e0.record(ext)
    for _ in range(e2e_steps):
        mx.step_io(p_in, p_out, DT, NSUB)
    mx.io_join()
    e1.record(ext)
    mx.sync()
    barrier()
    ms_e2e = max_over_ranks(e0.elapsed_time(e1))
    h2d = sum(mx.size(sp) for sp in range(7)) * 8
    # ---- accuracy: mixed vs plain FP64 after ERR_STEPS steps from the same state
    mx.restore_snapshot()
    budget0 = mx.energy_budget()
    mx.step(DT, NSUB, ERR_STEPS)
    st_mx = [mx.get(sp) for sp in range(7)]
    budget_mx = mx.energy_budget()
    mx.close()

    # ---- plain FP64 path (timed over the same ERR_STEPS steps) ----
    f64 = make(vg.FP64)
    f64.step(DT, NSUB, 1)
    ms_64, _ = timed_steps(f64, ERR_STEPS)
    ms_64 = max_over_ranks(ms_64)
    k64 = ERR_STEPS
    st_64 = [f64.get(sp) for sp in range(7)]
    budget_64 = f64.energy_budget()
    f64.close()
    accuracy = field_errors(vg, setup, st_mx, st_64)

    si = si_leg(vg) if not args.no_si else None
    nest = nest_leg(vg, torch, args.warmup) if not args.no_nest else None
    window = window_leg(vg, torch) if not args.no_window else None
    physics = physics_leg(vg, torch) if not args.no_physics else None
    ckern = None
    if not args.no_ckernels:
        try:
            ckern = ckernels_leg(vg, torch)
        except Exception as e:  # a side leg: its failure must not cost the headline line
            ckern = {"error": repr(e)}

    value = whole_job_rate(world, cells, args.steps, ms_mx)
    value64 = whole_job_rate(world, cells, k64, ms_64)
    e2e = whole_job_rate(world, cells, e2e_steps, ms_e2e)

    # roofline of the dominant kernel class (live CUDA-event times)
    peak, peak_kind = measured_peak()
    # algorithmic bytes per cell of one launch of each kernel class (FP32 fields 4 B, FP64 8 B):
    # stage: 56 (stage 1: win = w0), 84 (stage 2), 112 (stage 3, + its tendency);
    # column: read u v w rho pi, write w rho pi u v; finish: read S0, R3, 5 substep
    # fields, 7 stage fields, write S1, W0; after a stage's last substep, in
    # place: u/v update (read u v pi, write u v) and, when the column kernel
    # defers its w/rho' corrections (variant 5, the built-in one), those
    # corrections too in the same column march (+ read w rho, write w rho)
    col = tuning.get("column_kernel", -1) if isinstance(tuning, dict) else -1
    defer = col in (-1, 5)
    per_cell = {0: (56.0 + 84.0 + 112.0) / 3.0, 1: 40.0, 2: 216.0, 3: 36.0 if defer else 20.0}
    names = {0: "k_mx_stage", 1: "k_mx_hevi_tmad" if defer else "k_mx_hevi_tma", 2: "k_mx_finish",
             3: "k_mx_fix" if defer else "k_mx_fb_mom(u,v)"}
    dom = max(ktimes, key=lambda c: ktimes[c][0])
    tot_ms, spans = ktimes[dom]
    avg_s = tot_ms / max(spans, 1) * 1e-3
    bytes_launch = per_cell[dom] * cells
    achieved = bytes_launch / avg_s / 1e9
    share = {names[c]: round(ktimes[c][0] / max(sum(v[0] for v in ktimes.values()), 1e-9), 4) for c in ktimes}

    if rank != 0:
        ranks.close()
        return
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_mx / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64-state/f32-compute", "data": "synthetic",
        "config": {"workload": "512x512x80 single domain (dx=1 km, stretched dz 50->708 m, 20 km top), WENO5 "
                               "scalars, dt=6 s, 6 HEVI substeps per RK3 stage",
                   "cells": cells, "dt_s": DT, "substeps_per_stage": NSUB, "precision": "mixed",
                   "l2": "inputs (1.7 GB state) >> 129 MB L2; no flush", "parallelism": "replica per GPU"},
        "fp64_value": value64, "fp64_ms_per_step": ms_64 / k64, "mixed_over_fp64": value / value64,
        "mixed_vs_fp64_error": {"steps": ERR_STEPS, "fields": accuracy},
        "conservation": {
            "steps": ERR_STEPS, "note": "FP64 global sums on the device (dyn::energy_budget); the lateral "
                                        "boundaries are open (clamped), so mass and energy also cross them",
            "mass_rel_change": {"mixed": budget_mx["mass"] / budget0["mass"] - 1.0,
                                "fp64": budget_64["mass"] / budget0["mass"] - 1.0},
            "total_energy_rel_change": {"mixed": budget_mx["total"] / budget0["total"] - 1.0,
                                        "fp64": budget_64["total"] / budget0["total"] - 1.0},
            "mixed_vs_fp64_mass": budget_mx["mass"] / budget_64["mass"] - 1.0},
        "restarts": {"every_steps": RESTART, "in_timed_region": restarts,
                     "why": "superadiabatic theta noise in 50 m layers grows convectively (e-fold ~40 s) and the "
                            "state blows up after ~25-30 steps in the FP64 path as well; the timed run puts the "
                            "initial state back from a device snapshot (D2D copy, timed) every 20 steps"},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": h2d,
                "note": "per step: the input state uploaded from pinned host memory (7 species, FieldT "
                        "layout), one step, the result downloaded into other pinned buffers; vibe_gb300_step_io "
                        "overlaps the copies of neighbouring steps with the compute (two copy streams)"},
        "roofline": {"bound": "hbm", "kernel": names[dom], "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                     "traffic": traffic_of(names[dom], cells), "algorithmic_bytes_per_launch": bytes_launch,
                     "avg_launch_ms": avg_s * 1e3, "launches": spans, "time_share": share},
        "step_roofline": {"bytes_per_cell_update": 1944, "achieved": 1944.0 * value / world / 1e9,
                          "peak": peak, "unit": "GB/s", "frac": 1944.0 * value / world / 1e9 / peak},
        "gpu_launches": launches,
        "tuning": tuning,
        "clocks": clk.summary(),
    }
    if si is not None:
        line["semi_implicit"] = si
    if nest is not None:
        line["batched_nests"] = nest
    if window is not None:
        line["assimilation_window"] = window
    if physics is not None:
        line["physics_coupling"] = physics
    if ckern is not None:
        line["c_abi_kernels"] = ckern
    if cpu is not None:
        line["cpu_baseline"] = cpu
        line["mixed_vs_oracle_error"] = oracle_errors(vg, 128, 128, oracle_record)
    print(json.dumps(line))
    ranks.close()


if __name__ == "__main__":
    main()
