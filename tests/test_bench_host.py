"""Host-side pieces of bench.py that run without a GPU: the CPU legs (the
oracle iterations they time, the reference arm's process and its config) and
the committed ncu traffic figures the roofline reads."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def _oracle_case(n=8):
    O = bench._oracle()
    import workload as OW

    return O, *OW.c2(n=n, ldemb=1_000_000)


def test_oracle_iterations_time_one_continuing_solve():
    O, op, pix, rod = _oracle_case()
    dt, done, cores, t_setup = bench.oracle_iterations(O, op, pix, rod, 2, 3)
    assert done == 3 and dt > 0 and cores >= 1 and t_setup > 0
    # warm-up + timed iterations are one solve: the same iterate as 5 in a row
    o = O.Oracle(op, pix, rod).femat()
    u = o.affine_u()
    g, _ = o.energy(u)
    r = o.dembx(u, g, float(g @ g), max_steps=5)
    assert r["lstep"] == 5


def test_oracle_iterations_respect_a_budget():
    O, op, pix, rod = _oracle_case()
    _, done, _, _ = bench.oracle_iterations(O, op, pix, rod, 1, 5, budget_s=1e-9)
    assert done == 1  # the budget admits one iteration at least


def test_reference_arm_loads_no_package_library_and_prints_the_same_config():
    code = "\n".join([
        "import runpy, sys",
        "sys.argv = ['bench.py', '--impl', 'reference', '--n', '12', '--steps', '4', '--warmup', '2']",
        "try:",
        "    runpy.run_path('bench.py', run_name='__main__')",
        "except SystemExit as ex:",
        "    assert not ex.code",
        "maps = open('/proc/self/maps').read()",
        "print('PKG_SO' if 'libe3d_gpu' in maps else 'NO_PKG_SO')",
        "print('PKG' if 'elas3d_xtal_gb300' in sys.modules else 'NO_PKG')"])
    out = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    lines = out.stdout.strip().splitlines()
    assert lines[-2:] == ["NO_PKG_SO", "NO_PKG"]
    line = json.loads(lines[-3])
    assert line["impl"] == "reference" and line["steps"] == 4 and line["warmup"] == 2
    assert line["metric"] == bench.METRIC and line["unit"] == bench.UNIT
    p, _, _ = bench._workload(12)
    assert line["config"] == bench.plain_config(12, p.ns, p.nphase - 1, 1)
    assert line["cpu_baseline"]["kind"] == "port" and line["e2e"]["h2d_bytes_per_step"] == 0


@pytest.mark.parametrize("mixed,lo,hi", [(False, 300.0, 450.0), (True, 120.0, 250.0)])
def test_committed_traffic_figures(mixed, lo, hi):
    per_node, _ = bench._traffic_per_node(mixed)
    assert per_node is not None and lo < per_node < hi
