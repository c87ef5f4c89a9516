"""TMA-fed FP32 stencil (node planes staged in shared memory by
cp.async.bulk.tensor through an mbarrier ring) against the FP32 stencil with
per-thread loads and against the FP64 oracle.

Both FP32 paths do the same per-node arithmetic on the same values in the same
order; they may launch different numbers of blocks (the ring kernel runs one
255-register block per SM), which regroups the FP64 block partial sums of the
dot products, so their solves agree to rounding: iteration counts within 1,
energies within 1e-11 relative, displacements within 1e-7.  Against the oracle
the mixed-form bar holds: energy within 1e-8."""
import numpy as np
import pytest

import elas3d_xtal_gb300 as e3d
import oracle as O

pytestmark = pytest.mark.gpu


def _oracle_problem(p):
    s = p.strain
    return O.Problem(p.nx, p.ny, p.nz, p.nphase, flag_m=p.flag_m, c11=p.c11, c12=p.c12, c44=p.c44,
                     e1=p.e1, nu1=p.nu1, exx=s[0], eyy=s[1], ezz=s[2], exz=s[3], eyz=s[4], exy=s[5],
                     tol=p.tol, ldemb=p.max_iter, criterion=p.criterion,
                     divergence_reset=p.divergence_reset)


def _case(nx, ny, nz, ngrains, seed):
    pix, rod = e3d.micro_grains(nx, ny, nz, ngrains, seed)
    e3d.micro_spherical_pores(pix, nx, ny, nz, 0.02, ngrains + 1, seed + 1, log_mu=np.log(1.5))
    p = e3d.Problem(nx, ny, nz, ngrains + 1, c11=240e9, c12=150e9, c44=90e9,
                    strain=(1e-3, 0.0, -2e-4, 3e-4, 0.0, 1e-4))
    p.precision = e3d.PREC_MIXED
    p.refine_every = 50
    return p, pix, rod


def _solve(p, pix, rod, tma, monkeypatch):
    if tma:
        monkeypatch.setenv("E3D_TMA", "1")
    else:
        monkeypatch.delenv("E3D_TMA", raising=False)
    with e3d.Elas3D(p) as g:
        path = g.stencil_path()
        g.upload(pix, rod)
        res = g.run()
        u = g.get_u()
    return path, res, u


def _rel(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b)))


SHAPES = [
    (36, 20, 17, 10),   # partial tiles in x (width 4) and y (width 4)
    (64, 16, 40, 12),   # full tiles, several z chunks
    (32, 8, 16, 4),     # one tile column: +x and +y halos wrap to the tile itself
    (4, 12, 9, 3),      # nx smaller than every box
    (8, 2, 20, 5),      # 2-node periodic y
    (12, 33, 7, 6),     # odd ny, short z
]


@pytest.mark.parametrize("shape", SHAPES)
def test_tma_stencil_matches_per_thread_loads(shape, monkeypatch):
    p, pix, rod = _case(*shape, seed=sum(shape))
    path_t, rt, ut = _solve(p, pix, rod, True, monkeypatch)
    path_r, rr, ur = _solve(p, pix, rod, False, monkeypatch)
    assert path_t == "f32_tma" and path_r == "f32"
    assert rt["exit_reason"] == e3d.EXIT_CONVERGED and rr["exit_reason"] == e3d.EXIT_CONVERGED
    assert abs(rt["iterations"] - rr["iterations"]) <= 1
    assert abs(rt["utot"] - rr["utot"]) <= 1e-11 * abs(rr["utot"])
    assert _rel(ut, ur) < 1e-7
    ref = O.run(_oracle_problem(p), pix, rod)
    assert abs(rt["utot"] - ref["utot"]) <= 1e-8 * abs(ref["utot"])


def test_unaligned_rows_keep_per_thread_loads(monkeypatch):
    p, pix, rod = _case(30, 8, 8, 4, seed=3)  # 30 * 4 bytes is not a multiple of 16
    path, res, _ = _solve(p, pix, rod, True, monkeypatch)
    assert path == "f32"
    assert res["exit_reason"] == e3d.EXIT_CONVERGED


def test_fp64_form_reports_its_path():
    p, pix, rod = _case(16, 16, 16, 4, seed=9)
    p.precision = e3d.PREC_FP64
    with e3d.Elas3D(p) as g:
        assert g.stencil_path() == "fp64"
