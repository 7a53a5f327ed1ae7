"""Nest transfer cases shared by the CPU and GPU tests: seeded FieldT
fields of every stagger on a parent and a child grid, and placements that
cover the edges (child partly beyond the parent, restriction boxes at the
parent's border, Davies zones wider than the child)."""
import numpy as np

STAGGERS = [1, 2, 3, 0, 0, 0, 0]  # u v w rho theta pi qv
CASES = [
    # parent dims, child dims, placement
    ((12, 10, 5), (19, 16, 5), dict(i0=6, j0=3, iext=6, jext=5, ratio=3, boundary_zone=5)),
    ((9, 7, 4), (13, 11, 4), dict(i0=-2, j0=-1, iext=4, jext=3, ratio=2, boundary_zone=3)),
    ((16, 14, 6), (10, 31, 7), dict(i0=13, j0=0, iext=3, jext=14, ratio=3, boundary_zone=12)),
    ((5, 5, 3), (7, 6, 3), dict(i0=0, j0=0, iext=5, jext=5, ratio=4, boundary_zone=1)),
]


def fields(oc, dims, seed):
    rng = np.random.default_rng(seed)
    nx, ny, nz = dims
    return [rng.standard_normal(oc.fieldt_size(nx, ny, nz, s)) for s in STAGGERS]
