"""Generates the committed golden fixtures tests/golden/*.npz from the CPU oracle.

The reference ships no golden vectors and cannot be built (Fortran + HDF5), so
these fixtures record the oracle's outputs on small seeded inputs; the CPU
tests check that the oracle still reproduces them and the GPU tests compare the
CUDA path against them.  Run from the repository root:

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as O  # noqa: E402


def case(name, nx, ny, nz, ngrains, seed, strain, pores=True, c=(206e9, 133e9, 119e9), blocky=False):
    rng = np.random.default_rng(seed)
    nphase = ngrains + 1
    if blocky:  # grains as 2x2x2 blocks, a few pores
        blocks = rng.integers(1, ngrains + 1, size=((nx + 1) // 2, (ny + 1) // 2, (nz + 1) // 2))
        full = np.repeat(np.repeat(np.repeat(blocks, 2, 0), 2, 1), 2, 2)[:nx, :ny, :nz]
        pix = full.transpose(2, 1, 0).ravel().astype(np.int32)
        if pores:
            pix[rng.choice(pix.size, size=max(1, pix.size // 50), replace=False)] = nphase
    else:
        pix = rng.integers(1, nphase + (1 if pores else 0), size=nx * ny * nz).astype(np.int32)
    rod = rng.normal(size=3 * ngrains)
    s = np.asarray(strain, float)
    p = O.Problem(nx, ny, nz, nphase, c11=c[0], c12=c[1], c44=c[2], exx=s[0], eyy=s[1], ezz=s[2],
                  exz=s[3], eyz=s[4], exy=s[5])
    o = O.Oracle(p, pix, rod).femat()
    x = np.random.default_rng(seed + 1).normal(size=3 * p.ns)
    u0 = o.affine_u()
    g0, U0 = o.energy(u0)
    r = O.run(p, pix, rod)
    out = dict(
        shape=np.array([nx, ny, nz, nphase]), material=np.array(c), strain=s, pix=pix, rod=rod, x=x,
        Kx=o.apply(x), b=o.b, C=np.array(o.C), cmod=o.cmod_array(), dk=o.dk_array(),
        minv=o.block_jacobi(), utot0=np.array(U0), gg0=np.array(g0 @ g0), lstep=np.array(r["lstep"]),
        utot=np.array(r["utot"]), strav=r["strav"], epsav=r["epsav"], history=r["history"], u=r["u"],
    )
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(name, "ns", p.ns, "iterations", r["lstep"], "U", r["utot"])


if __name__ == "__main__":
    case("random_6x5x4", 6, 5, 4, 4, seed=101, strain=[2e-4, -1e-4, 3e-4, 1e-4, -2e-4, 5e-5])
    case("blocky_10x10x10", 10, 10, 10, 8, seed=202, strain=[1e-3, 0, 0, 0, 0, 0],
         c=(240e9, 150e9, 120e9), blocky=True)
    case("odd_9x7x5", 9, 7, 5, 3, seed=303, strain=[0, 0, 1e-3, 0, 0, 0], blocky=True)
