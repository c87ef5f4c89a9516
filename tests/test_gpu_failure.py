"""Failure detection without a GPU fault.

Every device-side wait of the library (the persistent kernels' grid barrier,
the job engine's job barriers, the TMA ring's mbarrier waits) is bounded by a
wall-clock limit; when it runs out the kernel raises an error flag, leaves, and
the host call returns E3D_ERR_TIMEOUT.  Here the wait is made to run out on
purpose -- a barrier whose partner block never arrives, an mbarrier phase whose
bytes no copy delivers -- with a short limit, and the context must stay usable:
a solve right afterwards converges as usual."""
import time

import pytest

import elas3d_xtal_gb300 as e3d
from elas3d_xtal_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("which", [0, 1], ids=["grid_barrier", "mbarrier"])
def test_unsatisfiable_wait_reports_timeout_and_context_survives(which):
    L = e3d.load_library()
    t0 = time.perf_counter()
    rc = L.e3d_selftest_timeout(0, which, 0.2)
    dt = time.perf_counter() - t0
    assert rc == e3d.E3D_ERR_TIMEOUT
    assert 0.15 < dt < 10.0
    p, pix, rod = W.c1(n=12, ngrains=6, seed=1)
    with e3d.Elas3D(p) as g:
        g.upload(pix, rod)
        res = g.run()
    assert res["exit_reason"] == e3d.EXIT_CONVERGED


def test_selftest_rejects_bad_arguments():
    L = e3d.load_library()
    assert L.e3d_selftest_timeout(0, 2, 0.1) == e3d.E3D_ERR_INPUT
    assert L.e3d_selftest_timeout(0, 0, 0.0) == e3d.E3D_ERR_INPUT
    assert L.e3d_selftest_timeout(0, 0, 60.0) == e3d.E3D_ERR_INPUT
