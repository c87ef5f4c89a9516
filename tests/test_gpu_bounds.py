"""Bounds-checked debug build (the stand-in for a memory checker): the library
compiled with -DE3D_BOUNDS checks every index of the stencil tiles, halos,
phase-table rows, PCG sweeps and job-engine partials against its buffer's
length and records, without trapping, any index outside it.

The checked library runs a workload that reaches every checked kernel in a
child process (it is selected with E3D_LIBRARY): FP64 and mixed-precision
solves (TMA ring and per-thread-load stencils) on grids with partial tiles,
1- and 2-node periodic directions, pores and shear loads, full-field stress,
K.x through e3d_apply and e3d_apply_noalloc, plain CG, a batch with the
autotuner and with fixed part counts, and a serving queue with a cancellation.
Every group must leave the record empty; the self-test confirms the record
catches a planted index past a buffer's end (redirected to element 0, so no
access leaves the buffer).  The results must equal those of the plain library
on the same inputs, to rounding (the checked kernels may launch other grid
sizes, which regroups the FP64 block partial sums)."""
import ctypes as C
import json
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SHAPES = [
    (36, 20, 17, 10),  # partial tiles in x and y
    (4, 12, 9, 3),     # nx smaller than every TMA box
    (8, 2, 20, 5),     # 2-node periodic y
    (33, 9, 1, 4),     # 1-node periodic z, nx not a multiple of 4 (no TMA)
]


def _import():
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    import __graft_entry__

    pkg = __graft_entry__._load_package()
    from elas3d_xtal_gb300 import workloads as W

    return pkg, W


def _case(e3d, nx, ny, nz, ng, seed):
    pix, rod = e3d.micro_grains(nx, ny, nz, ng, seed)
    e3d.micro_spherical_pores(pix, nx, ny, nz, 0.02, ng + 1, seed + 1, log_mu=np.log(1.5))
    p = e3d.Problem(nx, ny, nz, ng + 1, c11=240e9, c12=150e9, c44=90e9,
                    strain=(1e-3, 0.0, -2e-4, 3e-4, 0.0, 1e-4))
    return p, pix, rod


def workload(check):
    """Runs every form once; check(group) is called after each group."""
    e3d, W = _import()
    out = {}
    for nx, ny, nz, ng in SHAPES:
        key = f"{nx}x{ny}x{nz}"
        p, pix, rod = _case(e3d, nx, ny, nz, ng, nx + ny + nz)
        with e3d.Elas3D(p) as g:
            r = g.upload(pix, rod).run()
            sig, vm = g.stress_fullfield()
            y = g.apply(W.random_field(p.ns, seed=3))
        out["fp64_" + key] = (r["iterations"], r["utot"], float(np.sum(vm)), float(np.linalg.norm(y)))
        check("fp64_" + key)
        for tma in (True, False):
            if tma:
                os.environ["E3D_TMA"] = "1"
            else:
                os.environ.pop("E3D_TMA", None)
            p.precision = e3d.PREC_MIXED
            p.refine_every = 20
            with e3d.Elas3D(p) as g:
                r = g.upload(pix, rod).run()
                path = g.stencil_path()
            tag = f"mixed_{path}_{key}"
            out[tag] = (r["iterations"], r["utot"])
            check(tag)
        os.environ.pop("E3D_TMA", None)
    p, pix, rod = _case(e3d, 20, 12, 10, 6, 9)
    p.preconditioner = e3d.PRECOND_NONE
    with e3d.Elas3D(p) as g:
        r = g.upload(pix, rod).run()
    out["plain_cg"] = (r["iterations"], r["utot"])
    check("plain_cg")
    # allocation-free K.x on caller-owned device buffers
    import torch

    p, pix, rod = _case(e3d, 36, 20, 17, 10, 5)
    with e3d.Elas3D(p) as g:
        g.upload(pix, rod).femat()
        cmod = np.empty(36 * p.nphase)
        assert g.L.e3d_get_cmod(g.handle, e3d._dp(cmod)) == e3d.E3D_OK
    L = e3d.load_library()
    dev = torch.device("cuda", 0)
    d_pix = torch.from_numpy(pix).to(dev)
    d_cmod = torch.from_numpy(cmod).to(dev)
    d_x = torch.from_numpy(W.random_field(p.ns, seed=4)).to(dev)
    d_y = torch.zeros(3 * p.ns, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    rc = L.e3d_apply_noalloc(p.nx, p.ny, p.nz, p.nphase, C.c_void_p(d_pix.data_ptr()), C.c_void_p(d_cmod.data_ptr()),
                             C.c_void_p(d_x.data_ptr()), C.c_void_p(d_y.data_ptr()), None)
    assert rc == e3d.E3D_OK
    out["noalloc"] = (0, float(torch.linalg.norm(d_y).item()))
    check("noalloc")
    rves = [W.rve(12, 4, 5, A=2.0), W.rve(0, 6, 6, A=0.5, pore_frac=0.02, shape=(20, 9, 14)),
            W.rve(0, 3, 7, A=2.5, shape=(1, 7, 6)), W.rve(0, 2, 8, A=3.0, shape=(2, 2, 3))]
    for parts in (0, 3):
        with e3d.Batch(rves, parts=parts) as b:
            ceff, _ = b.solve()
            res = b.results()
        if parts:
            for r in sorted(res, key=lambda r: (r["rve"], r["load_case"])):
                out[f"batch_{r['rve']}_{r['load_case']}"] = (r["iterations"], r["utot"])
        check(f"batch_parts{parts}")
    rng = np.random.default_rng(7)
    reqs = [(W.rve(n, 5, 200 + n, A=1.5), rng.normal(size=6) * 1e-3) for n in (14, 10, 18)]
    with e3d.Server(round_iters=5, max_active=2, round_balance=False) as srv:
        ids = [srv.submit(*r) for r in reqs]
        srv.step()
        srv.cancel(ids[2])  # queued
        for _ in range(100000):
            if srv.step() == 0:
                break
        for k in (0, 1):
            r = srv.result(ids[k])
            out[f"serve_{k}"] = (r["iterations"], r["utot"])
    check("serve")
    return out


def _child():
    e3d, _ = _import()
    assert e3d.load_library()._name == e3d.BOUNDS_LIB_PATH
    selftest = int(e3d.load_library().e3d_selftest_bounds(0))
    records = {}

    def check(group):
        records[group] = e3d.debug_bounds()

    check("start")
    res = workload(check)
    print(json.dumps({"selftest": selftest, "records": records, "results": res}))


@pytest.mark.gpu
def test_bounds_checked_build_is_clean_and_agrees():
    e3d, _ = _import()
    import importlib.util

    spec = importlib.util.spec_from_file_location("e3d_build", os.path.join(ROOT, "elas3d-xtal_gb300", "build.py"))
    builder = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(builder)
    lib = builder.build(bounds=True)
    assert lib == e3d.BOUNDS_LIB_PATH
    env = dict(os.environ, E3D_LIBRARY=lib)
    env.pop("E3D_TMA", None)
    proc = subprocess.run([sys.executable, os.path.abspath(__file__), "--child"], env=env, capture_output=True,
                          text=True, timeout=900)
    assert proc.returncode == 0, proc.stdout[-2000:] + proc.stderr[-4000:]
    child = json.loads(proc.stdout.strip().splitlines()[-1])
    assert child["selftest"] == e3d.E3D_OK
    for group, rec in child["records"].items():
        assert rec is not None, "the child loaded a library without the checks"
        assert rec["count"] == 0, (group, rec)
    # the plain library (this process) on the same inputs
    assert e3d.debug_bounds() is None
    ref = workload(lambda group: None)
    got = child["results"]
    assert sorted(got) == sorted(ref)
    assert any(k.startswith("mixed_f32_tma") for k in ref) and any(k.startswith("mixed_f32_") and "tma" not in k
                                                                   for k in ref)
    for k, v in ref.items():
        it, vals = v[0], v[1:]
        assert abs(got[k][0] - it) <= 1, (k, got[k], v)
        for a, b in zip(got[k][1:], vals):
            assert abs(a - b) <= 1e-9 * abs(b), (k, got[k], v)


def test_plain_library_reports_no_bounds_record():
    """Without the checks the query says so and the self-test runs no kernel."""
    e3d, _ = _import()
    L = e3d.load_library()
    if L._name == e3d.BOUNDS_LIB_PATH:
        pytest.skip("the checked library is loaded")
    rep = (C.c_int64 * 5)(*([7] * 5))
    assert L.e3d_debug_bounds(rep) == e3d.E3D_ERR_STATE
    assert list(rep) == [0] * 5
    assert L.e3d_selftest_bounds(0) == e3d.E3D_ERR_STATE
    assert L.e3d_debug_bounds(None) == e3d.E3D_ERR_INPUT


if __name__ == "__main__" and "--child" in sys.argv:
    _child()
