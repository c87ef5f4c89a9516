"""The multi-process path of bench.py on CPU ranks (gloo, world size 2):
replicas synchronise only through a barrier and the max-over-ranks of the
timing; the reference arm runs on rank 0 alone and the other ranks exit 0."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench

    ws, r, local, pg = bench._dist()
    assert pg.get_backend() == "gloo"
    bench._barrier(pg)
    m = bench._max_over_ranks(pg, 1.5 + rank)
    pg.destroy_process_group()
    q.put((rank, ws, m))


def test_barrier_and_max_over_ranks_gloo():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("CPU-rank test")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=5) for _ in range(2))
    assert res == [(0, 2, 2.5), (1, 2, 2.5)]


def test_reference_arm_rank0_only():
    pytest.importorskip("torch")
    port = _free_port()
    outs = []
    procs = []
    for r in range(2):
        env = dict(os.environ, RANK=str(r), WORLD_SIZE="2", LOCAL_RANK=str(r), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), OMP_NUM_THREADS="2")
        procs.append(subprocess.Popen([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                                       "--n", "10", "--steps", "2", "--warmup", "0", "--gpus", "2"],
                                      env=env, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    for p in procs:
        out, err = p.communicate(timeout=300)
        assert p.returncode == 0, err
        outs.append(out.strip())
    line = json.loads(outs[0])
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port"
    assert line["e2e"]["h2d_bytes_per_step"] == 0
    assert outs[1] == ""
