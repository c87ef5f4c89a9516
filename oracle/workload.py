"""Seeded benchmark inputs for the oracle side, built without the CUDA library.

TEST INFRASTRUCTURE ONLY: used by the CPU arms of ``bench.py`` and by tests.
It loads ``oracle/_build/libe3d_workload.so``, the package's host generator
(``elas3d-xtal_gb300/csrc/microgen.cpp``, declared in ``include/e3d_micro.h``)
compiled on its own by ``oracle/Makefile``, and repeats the recipes of
``elas3d-xtal_gb300/workloads.py`` (the same seeds, grain counts, pore
distributions and material constants), so the CPU oracle solves bit for bit the
input the GPU arm solves.  ``tests/test_micro.py`` checks that equality.

Input format as the reference's ppixel_hdf5 reads it
(src/elas3dxtal_pcg.f90:2879-2990): 1-based phase ids, grains 1..ngrains,
pore phase ngrains+1, one Rodrigues vector per grain.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess

import numpy as np

import oracle as O

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libe3d_workload.so")
_lib = None

C11 = 240.0e9
C12 = 150.0e9


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            subprocess.run(["make", "-s", "-C", _HERE], check=True)
        L = C.CDLL(_LIB_PATH)
        dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int32)
        i32, f64 = C.c_int32, C.c_double
        L.e3d_micro_grains.argtypes = [i32, i32, i32, i32, f64, C.c_uint64, ip, dp]
        L.e3d_micro_grains.restype = i32
        L.e3d_micro_spherical_pores.argtypes = [i32, i32, i32, f64, f64, f64, i32, C.c_uint64, ip]
        L.e3d_micro_spherical_pores.restype = i32
        L.e3d_micro_ellipsoidal_pores.argtypes = [i32, i32, i32, f64, f64, f64, f64, i32, C.c_uint64, ip]
        L.e3d_micro_ellipsoidal_pores.restype = i32
        _lib = L
    return _lib


def _seed(s: int) -> int:
    return int(s) & (2 ** 64 - 1)


def grains(nx, ny, nz, ngrains, seed, laguerre_sigma=0.0):
    pix = np.empty(nx * ny * nz, np.int32)
    rod = np.empty(3 * ngrains)
    rc = lib().e3d_micro_grains(nx, ny, nz, ngrains, float(laguerre_sigma), _seed(seed),
                                O._ip(pix), O._dp(rod))
    if rc != 0:
        raise RuntimeError(f"e3d_micro_grains failed ({rc})")
    return pix, rod


def spherical_pores(pix, nx, ny, nz, frac, pore_phase, seed, log_mu=math.log(3.0), log_sigma=0.4):
    rc = lib().e3d_micro_spherical_pores(nx, ny, nz, float(frac), float(log_mu), float(log_sigma),
                                         int(pore_phase), _seed(seed), O._ip(pix))
    if rc < 0:
        raise RuntimeError(f"e3d_micro_spherical_pores failed ({rc})")
    return rc


def ellipsoidal_pores(pix, nx, ny, nz, frac, pore_phase, seed, aspect=4.0, log_mu=math.log(2.0),
                      log_sigma=0.3):
    rc = lib().e3d_micro_ellipsoidal_pores(nx, ny, nz, float(frac), float(aspect), float(log_mu),
                                           float(log_sigma), int(pore_phase), _seed(seed), O._ip(pix))
    if rc < 0:
        raise RuntimeError(f"e3d_micro_ellipsoidal_pores failed ({rc})")
    return rc


def polycrystal(n, ngrains, seed, *, c44, pore_frac=0.0, pore_kind="sphere", laguerre_sigma=0.0,
                strain=(1.0e-3, 0.0, 0.0, 0.0, 0.0, 0.0), tol=1.0e-8, ldemb=10000):
    """(oracle Problem, pix, rodrigues) of a periodic n^3 polycrystal."""
    pix, rod = grains(n, n, n, ngrains, seed, laguerre_sigma)
    if pore_frac > 0.0:
        if pore_kind == "sphere":
            spherical_pores(pix, n, n, n, pore_frac, ngrains + 1, seed + 7919)
        else:
            ellipsoidal_pores(pix, n, n, n, pore_frac, ngrains + 1, seed + 7919)
    exx, eyy, ezz, exz, eyz, exy = strain
    prob = O.Problem(n, n, n, ngrains + 1, flag_m=1, c11=C11, c12=C12, c44=c44, exx=exx, eyy=eyy, ezz=ezz,
                     exz=exz, eyz=eyz, exy=exy, tol=tol, ldemb=ldemb)
    return prob, pix, rod


def c2(n=500, ngrains=None, seed=2, **kw):
    """500^3 / 8000 grains (300^3 / 2000 below 500), Zener ratio 2 (C44 = 90
    GPa), 1 % spherical pores with lognormal radii (mu = ln 3, sigma = 0.4)."""
    if ngrains is None:
        ngrains = 8000 if n >= 500 else (2000 if n >= 300 else max(8, int(2000 * (n / 300.0) ** 3)))
    return polycrystal(n, ngrains, seed, c44=2.0 * (C11 - C12) / 2.0, pore_frac=0.01, pore_kind="sphere", **kw)
