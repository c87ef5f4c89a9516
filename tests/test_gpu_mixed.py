"""Mixed precision (E3D_PREC_MIXED): FP32 stencil + FP32 block-Jacobi inside an
FP64 residual-replacement loop.  Results are compared with the FP64 oracle:
energy within 1e-8 relative (the accuracy bar of this form), averaged
stress within 1e-7, and the recomputed true residual meets the criterion."""
import numpy as np
import pytest

import elas3d_xtal_gb300 as e3d
import oracle as O
from elas3d_xtal_gb300 import workloads as W

pytestmark = pytest.mark.gpu

ENERGY_TOL = 1e-8
STRESS_TOL = 1e-7


def _oracle_problem(p):
    s = p.strain
    return O.Problem(p.nx, p.ny, p.nz, p.nphase, flag_m=p.flag_m, c11=p.c11, c12=p.c12, c44=p.c44,
                     e1=p.e1, nu1=p.nu1, exx=s[0], eyy=s[1], ezz=s[2], exz=s[3], eyz=s[4], exy=s[5],
                     tol=p.tol, ldemb=p.max_iter, criterion=p.criterion,
                     divergence_reset=p.divergence_reset)


def _rel(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b)))


@pytest.mark.parametrize("maker,n,refine", [("c1", 20, 50), ("c2", 24, 50), ("c3", 24, 20)])
def test_mixed_solve_matches_fp64_oracle(maker, n, refine):
    p, pix, rod = getattr(W, maker)(n=n)
    p.precision = e3d.PREC_MIXED
    p.refine_every = refine
    with e3d.Elas3D(p) as g:
        g.upload(pix, rod)
        res = g.run()
    ref = O.run(_oracle_problem(p), pix, rod)
    assert res["exit_reason"] == e3d.EXIT_CONVERGED
    assert res["refinements"] >= 1
    assert abs(res["utot"] - ref["utot"]) <= ENERGY_TOL * abs(ref["utot"])
    assert _rel(res["strav"], ref["strav"]) < STRESS_TOL
    # the exit test is re-checked on the FP64 true residual
    assert res["rel_res"] < p.tol


def test_mixed_shear_load_and_pores():
    p, pix, rod = W.c2(n=20)
    p.strain = (0.0, 0.0, 0.0, 5e-4, 0.0, 0.0)
    p.precision = e3d.PREC_MIXED
    with e3d.Elas3D(p) as g:
        g.upload(pix, rod)
        res = g.run()
    ref = O.run(_oracle_problem(p), pix, rod)
    assert res["exit_reason"] == e3d.EXIT_CONVERGED
    assert abs(res["utot"] - ref["utot"]) <= ENERGY_TOL * abs(ref["utot"])


def test_mixed_iterate_split_equals_solve():
    p, pix, rod = W.c1(n=16, ngrains=8, seed=4)
    p.precision = e3d.PREC_MIXED
    p.refine_every = 7
    a = e3d.Elas3D(p).upload(pix, rod)
    ra = a.run()
    b = e3d.Elas3D(p).upload(pix, rod).femat().init_affine()
    b.energy()
    b.solve_begin()
    st = None
    for _ in range(10000):
        st = b.iterate(3)
        if st["exit_reason"] != e3d.EXIT_RUNNING:
            break
    assert st["exit_reason"] == e3d.EXIT_CONVERGED
    assert abs(st["iterations"] - ra["iterations"]) <= 3
    ub, ua = b.get_u(), a.get_u()
    assert _rel(ub, ua) < 1e-6


def test_handle_reused_after_breakdown_ignores_stale_directions():
    """A solve that breaks down (NaN displacement) leaves NaN in the FP32
    search-direction buffers; the next solve on the same handle must not use
    them (the correction update deferred to the next stencil pass has nothing
    pending at a solve's first step) and must equal a fresh handle's solve."""
    p, pix, rod = W.c2(n=20)
    p.precision = e3d.PREC_MIXED
    p.refine_every = 20

    def solve(g):
        g.init_affine()
        g.energy()
        r = g.dembx()
        return r, g.get_u()

    with e3d.Elas3D(p) as g:
        g.upload(pix, rod).femat()
        g.set_u(np.full(3 * p.ns, np.nan))
        with pytest.raises(e3d.E3DError):
            g.energy()
            g.solve_begin()
            g.iterate(10)
        r2, u2 = solve(g)
    with e3d.Elas3D(p) as f:
        f.upload(pix, rod).femat()
        r1, u1 = solve(f)
    assert r1["exit_reason"] == e3d.EXIT_CONVERGED
    assert r2["exit_reason"] == e3d.EXIT_CONVERGED
    assert r2["iterations"] == r1["iterations"]
    assert np.array_equal(u1, u2)


@pytest.mark.parametrize("criterion", [e3d.CRIT_REF, e3d.CRIT_PRECOND_REL])
def test_mixed_replacement_on_residual_drop(criterion):
    """refine_decades: an FP64 replacement whenever the FP32 residual has fallen
    three decades below the last FP64 one, with the fixed period out of the way
    (1000).  The solve still ends on an FP64 residual and meets the FP64 oracle,
    with fewer replacements than one every 50 iterations."""
    p, pix, rod = W.c2(n=24)
    p.criterion = criterion
    p.precision = e3d.PREC_MIXED
    ref = O.run(_oracle_problem(p), pix, rod)
    p.refine_every = 50
    with e3d.Elas3D(p) as g:
        g.upload(pix, rod)
        fixed = g.run()
    p.refine_every, p.refine_decades = 1000, 3
    with e3d.Elas3D(p) as g:
        g.upload(pix, rod)
        res = g.run()
    assert res["exit_reason"] == e3d.EXIT_CONVERGED
    assert res["rel_res"] < p.tol
    assert abs(res["iterations"] - fixed["iterations"]) <= 3
    assert 1 <= res["refinements"] <= fixed["refinements"]
    tol = ENERGY_TOL * abs(ref["utot"])
    if criterion == e3d.CRIT_REF:  # the reference's loose stop: see test_gpu_parity_configs.py
        p.criterion = e3d.CRIT_PRECOND_REL
        tol = max(tol, 0.01 * abs(ref["utot"] - O.run(_oracle_problem(p), pix, rod)["utot"]))
    assert abs(res["utot"] - ref["utot"]) <= tol
