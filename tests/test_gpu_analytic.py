"""The CUDA solvers against closed-form solutions, with no oracle solve in
between: laminates of rotated cubic grains (tests/analytic.py), whose exact
periodic solution the trilinear elements represent, so that a converged solve
must carry the closed-form energy, <sigma> and <eps>, and every voxel the
stress of its layer.

- FP64 persistent PCG, layers normal to x, y and z on grids of 180k-380k
  nodes, under the true relative-residual stop at 1e-10: energy within 1e-10,
  <sigma> within 1e-10, each voxel's stress within 1e-6 of its layer's;
- mixed precision under the true relative-residual stop at 1e-8: energy within
  1e-8, <sigma> within 1e-7 (the accuracy bar of that form);
- the batched ensemble: the 6x6 effective stiffness of laminate RVEs against
  the exact laminate stiffness within 1e-7;
- the serving loop: laminate requests under arbitrary strains, energy within
  1e-8.

Stiffness per grain comes from the oracle's rotatestiffnessby restatement
(src/elas3dxtal_pcg.f90:2538-2633); the library's own table equals it to
1e-12 (tests/test_gpu_parity.py)."""
import numpy as np
import pytest

import analytic as AN
import elas3d_xtal_gb300 as e3d
import oracle as O
from elas3d_xtal_gb300 import workloads as W

pytestmark = pytest.mark.gpu

STRAIN = (1.0e-3, -3.0e-4, 2.0e-4, 4.0e-4, -2.0e-4, 3.0e-4)  # exx eyy ezz exz eyz exy (tensor)
CASES = [(0, (180, 36, 28), 3.0), (1, (40, 160, 24), 0.5), (2, (48, 36, 220), 5.0)]


def _laminate(axis, shape, A, ng=9, seed=0):
    rng = np.random.default_rng(60 + 7 * axis + seed)
    layers = rng.integers(1, ng + 1, size=shape[axis])
    pix = AN.laminate_pix(shape, layers, axis)
    rod = rng.normal(size=3 * ng)
    c44 = W.c44_from_zener(A)
    cm = O.rotate_stiffness(rod, W.C11, W.C12, c44)
    return layers, pix, rod, c44, cm


def _rel(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b)))


@pytest.mark.parametrize("axis,shape,A", CASES)
def test_fp64_laminate_is_exact(axis, shape, A):
    layers, pix, rod, c44, cm = _laminate(axis, shape, A)
    p = e3d.Problem(*shape, len(rod) // 3 + 1, c11=W.C11, c12=W.C12, c44=c44, strain=STRAIN, tol=1e-10,
                    criterion=e3d.CRIT_PRECOND_REL)
    with e3d.Elas3D(p) as g:
        g.upload(pix, rod)
        res = g.run()
        sig, _ = g.stress_fullfield()
    w, sig_avg, strains = AN.laminate_exact(cm, layers, AN.engineering(STRAIN), axis)
    assert res["exit_reason"] == e3d.EXIT_CONVERGED
    assert abs(res["utot"] - w * p.ns) <= 1e-10 * w * p.ns
    assert _rel(res["strav"], sig_avg) < 1e-10
    assert _rel(res["epsav"], AN.engineering(STRAIN)) < 1e-13
    # voxel by voxel: the stress of the voxel's layer
    layer_stress = np.array([cm[ph - 1] @ e for ph, e in zip(layers, strains)])  # [layer, 6]
    i, j, k = np.meshgrid(*[np.arange(n) for n in shape], indexing="ij")
    layer_of_voxel = (i, j, k)[axis].transpose(2, 1, 0).ravel()
    want = layer_stress[layer_of_voxel].T.ravel()  # component-major, as the library writes it
    assert np.max(np.abs(sig - want)) <= 1e-6 * np.max(np.abs(want))


@pytest.mark.parametrize("axis,shape,A", CASES)
def test_mixed_laminate_meets_the_accuracy_bar(axis, shape, A):
    layers, pix, rod, c44, cm = _laminate(axis, shape, A)
    p = e3d.Problem(*shape, len(rod) // 3 + 1, c11=W.C11, c12=W.C12, c44=c44, strain=STRAIN, tol=1e-8,
                    criterion=e3d.CRIT_PRECOND_REL, precision=e3d.PREC_MIXED, refine_every=50)
    with e3d.Elas3D(p) as g:
        g.upload(pix, rod)
        res = g.run()
    w, sig_avg, _ = AN.laminate_exact(cm, layers, AN.engineering(STRAIN), axis)
    assert res["exit_reason"] == e3d.EXIT_CONVERGED and res["refinements"] >= 1
    assert abs(res["utot"] - w * p.ns) <= 1e-8 * w * p.ns
    assert _rel(res["strav"], sig_avg) < 1e-7


def _rve(axis, shape, A, seed):
    layers, pix, rod, c44, cm = _laminate(axis, shape, A, ng=5, seed=seed)
    rve = dict(shape=shape, ngrains=5, c11=W.C11, c12=W.C12, c44=c44, pix=pix, rodrigues=rod)
    return rve, layers, cm


def test_batch_laminate_effective_stiffness_is_exact():
    spec = [(0, (40, 12, 16), 2.0), (1, (14, 36, 10), 0.5), (2, (16, 20, 44), 5.0), (2, (24, 24, 24), 1.5)]
    rves = [_rve(a, s, A, seed=i) for i, (a, s, A) in enumerate(spec)]
    with e3d.Batch([r for r, _, _ in rves], criterion=e3d.CRIT_PRECOND_REL, tol=1e-8) as b:
        ceff, _ = b.solve()
        res = b.results()
    assert all(r["status"] == e3d.EXIT_CONVERGED for r in res)
    for i, ((a, _, _), (_, layers, cm)) in enumerate(zip(spec, rves)):
        exact = AN.laminate_ceff(cm, layers, a)
        assert np.abs(ceff[i] - exact).max() <= 1e-7 * np.abs(exact).max(), i


def test_serve_laminate_requests_are_exact():
    rng = np.random.default_rng(11)
    spec = [(0, (36, 10, 12), 3.0), (1, (12, 30, 14), 4.0), (2, (10, 12, 40), 0.75)]
    reqs = []
    for i, (a, s, A) in enumerate(spec):
        rve, layers, cm = _rve(a, s, A, seed=10 + i)
        reqs.append((rve, layers, cm, a, rng.normal(size=6) * 1e-3))
    with e3d.Server(round_iters=20, criterion=e3d.CRIT_PRECOND_REL, tol=1e-8) as srv:
        ids = [srv.submit(r[0], r[4]) for r in reqs]
        for _ in range(100000):
            if srv.step() == 0:
                break
        out = [srv.result(i) for i in ids]
    for (rve, layers, cm, a, strain), r in zip(reqs, out):
        assert r is not None and r["status"] == e3d.EXIT_CONVERGED, r
        w, sig_avg, _ = AN.laminate_exact(cm, layers, AN.engineering(strain), a)
        ns = int(np.prod(rve["shape"]))
        assert abs(r["utot"] - w * ns) <= 1e-8 * w * ns
        assert _rel(r["strav"], sig_avg) < 1e-7


@pytest.mark.parametrize("flag_m,precision", [(1, e3d.PREC_FP64), (0, e3d.PREC_FP64), (1, e3d.PREC_MIXED)])
def test_laminate_with_isotropic_inclusion_layers(flag_m, precision):
    """Layers of the isotropic inclusion phase (E1 = 380 GPa, nu1 = 0.27)
    between rotated cubic grains (flag_m = 1) or isotropic matrix phases
    (flag_m = 0): the phase tables of both material modes against the closed
    form, on a 64 x 40 x 150 laminate."""
    rng = np.random.default_rng(120 + flag_m)
    shape, axis, ng = (64, 40, 150), 2, 6
    layers = rng.integers(1, ng + 2, size=shape[axis])
    layers[:2] = [ng + 1, 1]
    pix = AN.laminate_pix(shape, layers, axis)
    rod = rng.normal(size=3 * ng)
    kw = dict(flag_m=flag_m, c11=W.C11, c12=W.C12, c44=W.c44_from_zener(2.5), e1=380e9, nu1=0.27)
    tol = 1e-10 if precision == e3d.PREC_FP64 else 1e-8
    p = e3d.Problem(*shape, ng + 1, strain=STRAIN, tol=tol, criterion=e3d.CRIT_PRECOND_REL, precision=precision,
                    refine_every=50, **kw)
    with e3d.Elas3D(p) as g:
        g.upload(pix, rod)
        res = g.run()
    # the phase tables depend on the constants and orientations only: a 2 x 2 x 2 oracle problem gives them
    tiny = O.Problem(2, 2, 2, ng + 1, **kw)
    cm = O.Oracle(tiny, np.ones(8, np.int32), rod).femat().cmod_array()
    w, sig_avg, _ = AN.laminate_exact(cm, layers, AN.engineering(STRAIN), axis)
    assert res["exit_reason"] == e3d.EXIT_CONVERGED
    etol, stol = (1e-10, 1e-10) if precision == e3d.PREC_FP64 else (1e-8, 1e-7)
    assert abs(res["utot"] - w * p.ns) <= etol * w * p.ns
    assert _rel(res["strav"], sig_avg) < stol


def test_plain_cg_laminate_is_exact():
    """The identity-preconditioner variant (applications/sec3_1/cg) reaches the
    same closed form."""
    layers, pix, rod, c44, cm = _laminate(2, (40, 24, 60), 2.0)
    p = e3d.Problem(40, 24, 60, len(rod) // 3 + 1, c11=W.C11, c12=W.C12, c44=c44, strain=STRAIN, tol=1e-10,
                    criterion=e3d.CRIT_PRECOND_REL, preconditioner=e3d.PRECOND_NONE, max_iter=50000)
    with e3d.Elas3D(p) as g:
        g.upload(pix, rod)
        res = g.run()
    w, sig_avg, _ = AN.laminate_exact(cm, layers, AN.engineering(STRAIN), 2)
    assert res["exit_reason"] == e3d.EXIT_CONVERGED
    assert abs(res["utot"] - w * p.ns) <= 1e-10 * w * p.ns
    assert _rel(res["strav"], sig_avg) < 1e-9


def test_batch_laminates_with_inclusion_layers():
    """Batched RVEs whose last phase is an isotropic inclusion (batch options
    E1, nu1) in layers between the grains: C_eff against the closed form."""
    rng = np.random.default_rng(130)
    ng, e1, nu1 = 4, 380e9, 0.27
    specs, rves = [(0, (30, 10, 12), 1.5), (2, (12, 10, 34), 4.0)], []
    for i, (a, shape, A) in enumerate(specs):
        layers = rng.integers(1, ng + 2, size=shape[a])
        layers[:2] = [ng + 1, 1]
        rod = rng.normal(size=3 * ng)
        rve = dict(shape=shape, ngrains=ng, c11=W.C11, c12=W.C12, c44=W.c44_from_zener(A),
                   pix=AN.laminate_pix(shape, layers, a), rodrigues=rod)
        tiny = O.Problem(2, 2, 2, ng + 1, c11=W.C11, c12=W.C12, c44=rve["c44"], e1=e1, nu1=nu1)
        cm = O.Oracle(tiny, np.ones(8, np.int32), rod).femat().cmod_array()
        rves.append((rve, layers, cm, a))
    with e3d.Batch([r[0] for r in rves], criterion=e3d.CRIT_PRECOND_REL, tol=1e-8, e1=e1, nu1=nu1) as b:
        ceff, _ = b.solve()
        res = b.results()
    assert all(r["status"] == e3d.EXIT_CONVERGED for r in res)
    for i, (_, layers, cm, a) in enumerate(rves):
        exact = AN.laminate_ceff(cm, layers, a)
        assert np.abs(ceff[i] - exact).max() <= 1e-7 * np.abs(exact).max(), i
