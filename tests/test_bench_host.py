"""Host-side pieces of bench.py that run without a GPU: the bounded CPU
baseline and the committed ncu traffic figures the roofline reads."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def test_cpu_oracle_rate_respects_its_budget():
    p, pix, rod = bench._workload(8)
    rate, cores, dt, done = bench.cpu_oracle_rate(p, pix, rod, 1, 5, budget_s=1e-9)
    assert done == 1 and rate > 0 and cores >= 1  # the budget admits one iteration at least
    rate, cores, dt, done = bench.cpu_oracle_rate(p, pix, rod, 0, 3, budget_s=1e-9)
    assert done == 3  # no warm-up: nothing to size the sample with, all requested iterations run


@pytest.mark.parametrize("mixed,lo,hi", [(False, 300.0, 450.0), (True, 120.0, 250.0)])
def test_committed_traffic_figures(mixed, lo, hi):
    per_node, _ = bench._traffic_per_node(mixed)
    assert per_node is not None and lo < per_node < hi
