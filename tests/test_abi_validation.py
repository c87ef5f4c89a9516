"""Argument checks of the C ABI that come before any CUDA call, so they hold
on a machine without a GPU: every malformed call returns E3D_ERR_INPUT and
leaves the output handle null."""
import ctypes as C

import numpy as np
import pytest

import elas3d_xtal_gb300 as e3d


@pytest.fixture(scope="module")
def L():
    return e3d.load_library()


def _create(L, **kw):
    p = e3d.Problem(8, 8, 8, 3)
    for k, v in kw.items():
        setattr(p, k, v)
    pc = p.to_c()
    h = C.c_void_p(123)
    return L.e3d_create(C.byref(h), C.byref(pc)), h


@pytest.mark.parametrize("kw", [dict(nx=0), dict(ny=-1), dict(nz=0), dict(nphase=0), dict(max_iter=-1),
                                dict(precision=7), dict(criterion=9), dict(preconditioner=5),
                                dict(nx=1 << 14, ny=1 << 14, nz=1 << 13), dict(refine_decades=-1),
                                dict(refine_decades=16)],
                         ids=["nx0", "ny-1", "nz0", "nphase0", "max_iter-1", "precision", "criterion",
                              "preconditioner", "over-2^40-nodes", "refine_decades-1", "refine_decades16"])
def test_create_rejects_bad_problems(L, kw):
    rc, h = _create(L, **kw)
    assert rc == e3d.E3D_ERR_INPUT
    assert not h.value


def test_null_arguments(L):
    pc = e3d.Problem(8, 8, 8, 3).to_c()
    assert L.e3d_create(None, C.byref(pc)) == e3d.E3D_ERR_INPUT
    h = C.c_void_p()
    assert L.e3d_create(C.byref(h), None) == e3d.E3D_ERR_INPUT
    assert L.e3d_destroy(None) == e3d.E3D_OK
    assert L.e3d_selftest_timeout(0, 2, 0.1) == e3d.E3D_ERR_INPUT
    assert L.e3d_selftest_timeout(0, 0, 0.0) == e3d.E3D_ERR_INPUT


def test_batch_and_server_reject_bad_arguments(L):
    B = e3d._bind_batch(L)
    o = e3d.BatchOptsC()
    B.e3d_batch_opts_defaults(C.byref(o))
    pix = np.ones(8, dtype=np.int32)
    rod = np.zeros(3)
    good = e3d.RveC(2, 2, 2, 1, 240e9, 150e9, 90e9, e3d._ip(pix), e3d._dp(rod))
    h = C.c_void_p(123)
    arr = (e3d.RveC * 1)(good)
    assert B.e3d_batch_create(C.byref(h), arr, 0, C.byref(o)) == e3d.E3D_ERR_INPUT  # no RVE
    assert B.e3d_batch_create(C.byref(h), None, 1, C.byref(o)) == e3d.E3D_ERR_INPUT
    bad = (e3d.RveC * 1)(e3d.RveC(0, 2, 2, 1, 240e9, 150e9, 90e9, e3d._ip(pix), e3d._dp(rod)))
    assert B.e3d_batch_create(C.byref(h), bad, 1, C.byref(o)) == e3d.E3D_ERR_INPUT  # empty grid
    assert not h.value
    nopix = (e3d.RveC * 1)(e3d.RveC(2, 2, 2, 1, 240e9, 150e9, 90e9, None, e3d._dp(rod)))
    assert B.e3d_batch_create(C.byref(h), nopix, 1, C.byref(o)) == e3d.E3D_ERR_INPUT
    o.load_cases = 0x40  # beyond the six unit load cases
    assert B.e3d_batch_create(C.byref(h), arr, 1, C.byref(o)) == e3d.E3D_ERR_INPUT
    so = e3d.ServeOptsC()
    B.e3d_serve_opts_defaults(C.byref(so))
    so.max_active = 0
    assert B.e3d_serve_create(C.byref(h), C.byref(so)) == e3d.E3D_ERR_INPUT
    B.e3d_serve_opts_defaults(C.byref(so))
    so.round_iters = 0
    assert B.e3d_serve_create(C.byref(h), C.byref(so)) == e3d.E3D_ERR_INPUT
    assert B.e3d_serve_submit(None, C.byref(good), e3d._dp(np.zeros(6)), None) == e3d.E3D_ERR_INPUT


def test_apply_noalloc_rejects_before_any_cuda_call(L):
    """The allocation-free K.x refuses malformed calls before it touches the
    device (the pointers below are never dereferenced) and says why."""
    fake = [C.c_void_p(0x10000000 + 0x100000 * k) for k in range(4)]  # pix, cmod, x, y
    big = 2 ** 31 - 1
    # sizes whose tile arithmetic would overflow a 32-bit int
    for dims in [(big, 1, 1), (1, big, 1), (1, 1, big), (big, big, big), (65536, 65536, 2)]:
        assert L.e3d_apply_noalloc(*dims, 3, *fake, None) == e3d.E3D_ERR_INPUT
        assert "E3D_NOALLOC_SCRATCH_BYTES" in e3d.last_cuda_error()
    assert L.e3d_apply_noalloc(0, 4, 4, 3, *fake, None) == e3d.E3D_ERR_INPUT
    assert "at least 1" in e3d.last_cuda_error()
    assert L.e3d_apply_noalloc(4, 4, 4, 3, None, *fake[1:], None) == e3d.E3D_ERR_INPUT
    assert "NULL" in e3d.last_cuda_error()
    # y = K x cannot be formed in place: x and y must not overlap
    ns = 8 * 8 * 8
    x = 0x20000000
    for y in (x, x + 8 * (3 * ns - 1), x - 8 * (3 * ns - 1)):
        rc = L.e3d_apply_noalloc(8, 8, 8, 3, fake[0], fake[1], C.c_void_p(x), C.c_void_p(y), None)
        assert rc == e3d.E3D_ERR_INPUT
        assert "overlap" in e3d.last_cuda_error()
