"""Seeded synthetic workloads standing in for the reference's MATLAB/MTEX
inputs (no public dataset is involved).

Each builder returns ``(Problem, pix, rodrigues)`` in the reference's input
format (src/microstructure_gen.m:866-892): 1-based phase ids, grains
1..ngrains, pore phase ngrains+1, one Rodrigues vector per grain.

  c1 : 100^3, 64 periodic-Voronoi grains, cubic 240/150/120 GPa, no pores,
       exx = 1e-3, tol 1e-8 (the reference's CPU-runnable case)
  c2 : 300^3 / 2000 grains or 500^3 / 8000 grains, C44 from Zener ratio
       A = 2 (90 GPa), 1 % spherical pores with lognormal radii (mu = ln 3
       voxels, sigma = 0.4), exx = 1e-3
  c3 : 400^3, 4000 Laguerre grains with lognormal volumes (sigma 0.5),
       A in {0.5, 1, 2, 5}, 3 % ellipsoidal 4:1:1 voids
"""
from __future__ import annotations

import numpy as np

from . import (Problem, micro_ellipsoidal_pores, micro_grains, micro_spherical_pores)

C11 = 240.0e9
C12 = 150.0e9


def c44_from_zener(A: float) -> float:
    return A * (C11 - C12) / 2.0


def polycrystal(n: int, ngrains: int, seed: int, *, A: float | None = None, c44: float | None = None,
                pore_frac: float = 0.0, pore_kind: str = "sphere", laguerre_sigma: float = 0.0,
                strain=(1.0e-3, 0.0, 0.0, 0.0, 0.0, 0.0), **kw):
    """Generic periodic polycrystal on an n^3 grid."""
    pix, rod = micro_grains(n, n, n, ngrains, seed, laguerre_sigma=laguerre_sigma)
    if pore_frac > 0.0:
        if pore_kind == "sphere":
            micro_spherical_pores(pix, n, n, n, pore_frac, ngrains + 1, seed + 7919)
        else:
            micro_ellipsoidal_pores(pix, n, n, n, pore_frac, ngrains + 1, seed + 7919)
    if c44 is None:
        c44 = c44_from_zener(A if A is not None else 2.0)
    prob = Problem(n, n, n, ngrains + 1, flag_m=1, c11=C11, c12=C12, c44=c44, strain=tuple(strain), **kw)
    return prob, pix, rod


def c1(n: int = 100, ngrains: int = 64, seed: int = 1, **kw):
    return polycrystal(n, ngrains, seed, c44=120.0e9, **kw)


def c2(n: int = 500, ngrains: int | None = None, seed: int = 2, **kw):
    if ngrains is None:
        ngrains = 8000 if n >= 500 else (2000 if n >= 300 else max(8, int(2000 * (n / 300.0) ** 3)))
    return polycrystal(n, ngrains, seed, A=2.0, pore_frac=0.01, pore_kind="sphere", **kw)


def c3(n: int = 400, ngrains: int | None = None, A: float = 2.0, seed: int = 3, **kw):
    if ngrains is None:
        ngrains = 4000 if n >= 400 else max(8, int(4000 * (n / 400.0) ** 3))
    return polycrystal(n, ngrains, seed, A=A, pore_frac=0.03, pore_kind="ellipsoid",
                       laguerre_sigma=0.5, **kw)


def random_field(ns: int, seed: int) -> np.ndarray:
    """A seeded random nodal vector (3*ns, SoA) for apply tests."""
    return np.random.default_rng(seed).standard_normal(3 * ns)


def rve(n, ngrains, seed, A=2.0, pore_frac=0.0, shape=None):
    """One RVE as the batch / serving APIs take it (dict)."""
    nx, ny, nz = shape if shape is not None else (n, n, n)
    pix, rod = micro_grains(nx, ny, nz, ngrains, seed)
    if pore_frac > 0.0:
        micro_spherical_pores(pix, nx, ny, nz, pore_frac, ngrains + 1, seed + 7919)
    return dict(shape=(nx, ny, nz), ngrains=ngrains, c11=C11, c12=C12, c44=c44_from_zener(A), pix=pix,
                rodrigues=rod)


def ensemble(count, seed=4, edge=(32, 96), grains=(8, 200), zener=(0.5, 0.75, 1, 1.5, 2, 3, 4, 5),
             pores=(0.0, 0.02)):
    """The batched effective-stiffness ensemble: uneven RVE edges drawn
    uniformly from `edge`, grain counts from `grains`, Zener ratios from
    `zener`, pore fractions uniform in `pores`."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = int(rng.integers(edge[0], edge[1] + 1))
        ng = int(rng.integers(grains[0], grains[1] + 1))
        A = float(rng.choice(zener))
        pf = float(rng.uniform(*pores))
        out.append(rve(n, ng, seed * 1000 + i, A=A, pore_frac=pf))
    return out
