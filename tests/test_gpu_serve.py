"""Continuous-batching server: requests admitted while others run, results
against the FP64 oracle, the same result alone and in the mix, admission
bounded by the HBM budget."""
import numpy as np
import pytest

import elas3d_xtal_gb300 as e3d
import oracle as O
from elas3d_xtal_gb300 import workloads as W

pytestmark = pytest.mark.gpu

ENERGY_TOL = 1e-8


def _oracle(rve, strain):
    nx, ny, nz = rve["shape"]
    s = strain
    p = O.Problem(nx, ny, nz, rve["ngrains"] + 1, c11=rve["c11"], c12=rve["c12"], c44=rve["c44"],
                  exx=s[0], eyy=s[1], ezz=s[2], exz=s[3], eyz=s[4], exy=s[5])
    return O.run(p, rve["pix"], rve["rodrigues"])


def _requests():
    rng = np.random.default_rng(7)
    reqs = []
    for i, n in enumerate([14, 22, 10, 18, 26]):
        rve = W.rve(n, int(rng.integers(4, 12)), 100 + i, A=float(rng.uniform(0.5, 5.0)),
                    pore_frac=float(rng.uniform(0, 0.03)))
        strain = rng.normal(size=6) * 1e-3
        reqs.append((rve, strain))
    return reqs


def _drain(srv, ids, rounds=100000):
    for _ in range(rounds):
        if srv.step() == 0:
            break
    return [srv.result(i) for i in ids]


def test_serve_results_match_oracle_and_mix():
    reqs = _requests()
    # alone: request 1 in a fresh server
    with e3d.Server(round_iters=10, round_balance=False) as srv:
        rid = srv.submit(*reqs[1])
        alone = _drain(srv, [rid])[0]
    # mixed: staggered arrivals while others are on the device
    with e3d.Server(round_iters=10, round_balance=False) as srv:
        ids = [srv.submit(*reqs[0]), srv.submit(*reqs[1])]
        srv.step()
        srv.step()
        ids += [srv.submit(*r) for r in reqs[2:]]
        out = _drain(srv, ids)
    for (rve, strain), r in zip(reqs, out):
        assert r is not None and r["status"] == e3d.EXIT_CONVERGED, r
        ref = _oracle(rve, strain)
        assert abs(r["utot"] - ref["utot"]) <= ENERGY_TOL * abs(ref["utot"])
        assert r["seconds"] > 0
    mixed = out[1]
    assert mixed["iterations"] == alone["iterations"]
    assert abs(mixed["utot"] - alone["utot"]) <= 1e-12 * abs(alone["utot"])
    assert np.array_equal(mixed["strav"], alone["strav"])


def test_serve_hbm_budget_bounds_admission():
    reqs = _requests()
    with e3d.Server(round_iters=20) as probe:
        probe.submit(*reqs[4])
        probe.step()
        _, one = probe.memory()  # peak: the request may already be done after one round
    budget = int(one * 1.5)  # room for the largest request alone
    with e3d.Server(round_iters=20, hbm_budget=budget) as srv:
        ids = [srv.submit(*r) for r in reqs]
        out = _drain(srv, ids)
        now, peak = srv.memory()
    assert all(r is not None and r["status"] == e3d.EXIT_CONVERGED for r in out)
    assert peak <= budget and now == 0


def test_serve_cancel_queued_and_active_requests():
    reqs = _requests()
    with e3d.Server(round_iters=5, max_active=2, round_balance=False) as srv:
        ids = [srv.submit(*r) for r in reqs[:4]]
        srv.step()  # requests 0 and 1 active, 2 and 3 queued
        srv.cancel(ids[1])  # active
        srv.cancel(ids[3])  # queued
        with pytest.raises(e3d.E3DError):
            srv.cancel(12345)  # unknown id
        out = _drain(srv, ids)
        now, _ = srv.memory()
        with pytest.raises(e3d.E3DError):
            srv.cancel(ids[0])  # already finished
    assert out[1]["status"] == e3d.EXIT_CANCELLED and out[1]["iterations"] > 0
    assert out[3]["status"] == e3d.EXIT_CANCELLED and out[3]["iterations"] == 0
    for k in (0, 2):
        assert out[k]["status"] == e3d.EXIT_CONVERGED
        ref = _oracle(*reqs[k])
        assert abs(out[k]["utot"] - ref["utot"]) <= ENERGY_TOL * abs(ref["utot"])
    assert now == 0


def test_serve_refuses_bad_phase_ids_at_submission():
    reqs = _requests()
    rve, strain = reqs[2]
    bad = dict(rve)
    bad["pix"] = rve["pix"].copy()
    bad["pix"][5] = rve["ngrains"] + 2  # one past the pore phase
    with e3d.Server(round_iters=5, max_active=2) as srv:
        with pytest.raises(e3d.E3DError):
            srv.submit(bad, strain)
        rid = srv.submit(rve, strain)  # the server is unaffected
        out = _drain(srv, [rid])
    assert out[0]["status"] == e3d.EXIT_CONVERGED


def test_serve_round_balance_changes_scheduling_only():
    """With round balancing a small solve runs more iterations per round than
    a large one; results are a function of the request alone, so they are
    bitwise those of fixed rounds, in fewer rounds."""
    reqs = _requests()
    out, rounds = {}, {}
    for bal in (False, True):
        with e3d.Server(round_iters=8, round_balance=bal) as srv:
            ids = [srv.submit(*r) for r in reqs]
            n = 0
            while srv.step() > 0:
                n += 1
            out[bal] = [srv.result(i) for i in ids]
            rounds[bal] = n
    for a, b in zip(out[False], out[True]):
        assert a["status"] == b["status"] == e3d.EXIT_CONVERGED
        assert a["iterations"] == b["iterations"] and a["utot"] == b["utot"]
        assert np.array_equal(a["strav"], b["strav"])
    assert rounds[True] < rounds[False]
