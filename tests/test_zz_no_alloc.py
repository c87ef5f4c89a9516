"""e3d_apply_noalloc: K.x for callers that cannot allocate device memory
(a host framework that owns every device allocation, or a serving loop held to
a fixed HBM budget).  Called through the C ABI with caller-owned device
buffers, compared with the allocating entry point e3d_apply on the same
problem, on two calls in a row (the second call finds the first call's
contents in the shared static scratch), and the first result against the CPU
oracle's K.x.  Collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

import elas3d_xtal_gb300 as e3d
import oracle as O
from elas3d_xtal_gb300 import workloads as W

pytestmark = pytest.mark.gpu

KU_TOL = 1e-12  # the K.u tolerance of tests/test_gpu_parity.py


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _case():
    rng = np.random.default_rng(2024)
    ng = 7
    p = e3d.Problem(40, 24, 20, ng + 1, strain=tuple(rng.normal(size=6) * 1e-3))
    pix = rng.integers(1, ng + 2, size=p.ns).astype(np.int32)  # grains and pores
    rod = rng.normal(size=3 * ng)
    return p, pix, rod


def test_apply_noalloc_matches_apply_twice():
    torch = pytest.importorskip("torch")
    p, pix, rod = _case()
    g = e3d.Elas3D(p).upload(pix, rod).femat()
    L = g.L
    cmod = np.empty(36 * p.nphase)
    assert L.e3d_get_cmod(g.handle, e3d._dp(cmod)) == e3d.E3D_OK  # reference layout cmod(nphase,6,6)
    x1 = W.random_field(p.ns, seed=1)
    x2 = W.random_field(p.ns, seed=2) * 1e-3
    y1_ref = g.apply(x1)
    y2_ref = g.apply(x2)

    dev = torch.device("cuda", 0)
    d_pix = torch.from_numpy(pix).to(dev)
    d_cmod = torch.from_numpy(cmod).to(dev)
    d_x = torch.from_numpy(x1).to(dev)
    d_y = torch.full((3 * p.ns,), float("nan"), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()

    def call():
        return L.e3d_apply_noalloc(p.nx, p.ny, p.nz, p.nphase, C.c_void_p(d_pix.data_ptr()),
                                   C.c_void_p(d_cmod.data_ptr()), C.c_void_p(d_x.data_ptr()),
                                   C.c_void_p(d_y.data_ptr()), None)

    assert call() == e3d.E3D_OK
    assert _rel(d_y.cpu().numpy(), y1_ref) < KU_TOL
    # and against the CPU oracle's K.x (the reference's stencil, restated)
    s = p.strain
    op = O.Problem(p.nx, p.ny, p.nz, p.nphase, c11=p.c11, c12=p.c12, c44=p.c44, exx=s[0], eyy=s[1], ezz=s[2],
                   exz=s[3], eyz=s[4], exy=s[5])
    assert _rel(d_y.cpu().numpy(), O.Oracle(op, pix, rod).femat().apply(x1)) < KU_TOL
    free_before = torch.cuda.mem_get_info(0)[0]
    d_x.copy_(torch.from_numpy(x2).to(dev))
    d_y.fill_(float("nan"))
    torch.cuda.synchronize()
    assert call() == e3d.E3D_OK
    free_after = torch.cuda.mem_get_info(0)[0]
    assert _rel(d_y.cpu().numpy(), y2_ref) < KU_TOL
    assert free_after == free_before  # the call grew no device allocation
    g.close()


def test_apply_noalloc_rejects_oversize_and_bad_phase():
    torch = pytest.importorskip("torch")
    p, pix, rod = _case()
    L = e3d.load_library()
    dev = torch.device("cuda", 0)
    d_pix = torch.from_numpy(pix).to(dev)
    d_cmod = torch.zeros(36 * p.nphase, dtype=torch.float64, device=dev)
    d_x = torch.zeros(3 * p.ns, dtype=torch.float64, device=dev)
    d_y = torch.zeros(3 * p.ns, dtype=torch.float64, device=dev)
    ptrs = [C.c_void_p(t.data_ptr()) for t in (d_pix, d_cmod, d_x, d_y)]
    # a grid whose scratch exceeds E3D_NOALLOC_SCRATCH_BYTES is refused before any device work
    rc = L.e3d_apply_noalloc(1024, 1024, 1024, p.nphase, *ptrs, None)
    assert rc == e3d.E3D_ERR_INPUT
    assert "E3D_NOALLOC_SCRATCH_BYTES" in e3d.last_cuda_error()
    # a phase id outside [1, nphase] is refused before the stencil runs
    bad = pix.copy()
    bad[17] = p.nphase + 1
    d_bad = torch.from_numpy(bad).to(dev)
    rc = L.e3d_apply_noalloc(p.nx, p.ny, p.nz, p.nphase, C.c_void_p(d_bad.data_ptr()), *ptrs[1:], None)
    assert rc == e3d.E3D_ERR_INPUT
