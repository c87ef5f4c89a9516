#!/usr/bin/env python
"""Benchmark: plain FP64 PCG of the voxel-FE elasticity solve on GB300.

Metric: DOF-iterations per second (3*ns*iterations / PCG time) on the
500^3 periodic polycrystal (375M DOF, 8000 Voronoi grains, uniform SO(3)
orientations, cubic 240/150 GPa with Zener ratio A = 2, 1 % zero-stiffness
spherical pores, exx = 1e-3) -- seeded synthetic input with the shapes and
distributions of that configuration.  One step = one PCG iteration
(apply + dot products + updates).

  value : device-resident state, K iterations timed with CUDA events on the
          library's stream (vectors are 3 GB each, far larger than L2)
  e2e   : the same metric through the C ABI from pinned host buffers: upload,
          femat, affine guess, energy, block-Jacobi, K iterations, stress and
          the download of u are all inside the timed region
  --impl reference : the CPU oracle (C/OpenMP restatement of the reference's
          PCG) on this machine's host cores, same workload and metric

Multi-GPU (torchrun): replicas only -- each rank solves its own copy, no
collective on the data path ("scaling": "weak").
"""
from __future__ import annotations

import argparse
import importlib.util
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG_DIR = os.path.join(ROOT, "elas3d-xtal_gb300")
METRIC = "DOF-iters/s (plain FP64 PCG, 500^3 polycrystal)"
UNIT = "DOF-iter/s"
BYTES_PER_NODE_ITER = 364.0   # algorithmic HBM bytes per node per PCG iteration (FP64)
FLOPS_PER_NODE_ITER = 1200.0  # algorithmic flops per node per PCG iteration (dense stencil)


def _load_package():
    if "elas3d_xtal_gb300" in sys.modules:
        return sys.modules["elas3d_xtal_gb300"]
    spec = importlib.util.spec_from_file_location(
        "elas3d_xtal_gb300", os.path.join(PKG_DIR, "__init__.py"), submodule_search_locations=[PKG_DIR])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["elas3d_xtal_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


class ClockSampler:
    """nvidia-smi clock / throttle samples every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []
        self._t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return self
        self._t = threading.Thread(target=self._read, daemon=True)
        self._t.start()
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self._t:
            self._t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def _peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _traffic_per_node():
    """DRAM bytes per node per iteration of the PCG kernel from the committed
    ncu capture summary (profiles/pcg_fp64_traffic.json), if present."""
    path = os.path.join(ROOT, "profiles", "pcg_fp64_traffic.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["dram_bytes_per_node_iter"]), float(d.get("fp64_inst_per_node_iter", 0.0)) or None
    except Exception:
        return None, None


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if ws > 1:
        import torch.distributed as dist

        backend = "nccl" if _cuda_ok() else "gloo"
        if backend == "nccl":
            import torch

            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
        pg = dist
    return ws, rank, local, pg


def _cuda_ok():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


def _barrier(pg):
    if pg is not None:
        pg.barrier()


def _max_over_ranks(pg, v: float) -> float:
    if pg is None:
        return v
    import torch

    dev = "cuda" if pg.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def _workload(n: int):
    _load_package()
    from elas3d_xtal_gb300 import workloads as W

    p, pix, rod = W.c2(n=n)
    p.max_iter = 1_000_000
    return p, pix, rod


def _oracle():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    return O


def cpu_oracle_rate(p, pix, rod, warmup: int, iters: int):
    """Oracle PCG iterations on the host cores; returns (DOF-iter/s, cores, seconds)."""
    O = _oracle()
    s = p.strain
    op = O.Problem(p.nx, p.ny, p.nz, p.nphase, flag_m=p.flag_m, c11=p.c11, c12=p.c12, c44=p.c44,
                   e1=p.e1, nu1=p.nu1, exx=s[0], eyy=s[1], ezz=s[2], exz=s[3], eyz=s[4], exy=s[5],
                   tol=p.tol, ldemb=p.max_iter)
    o = O.Oracle(op, pix, rod).femat()
    u = o.affine_u()
    g, _ = o.energy(u)
    gg0 = float(g @ g)
    if warmup > 0:
        r = o.dembx(u, g, gg0, max_steps=warmup)
        u, g = r["u"], r["g"]
    t0 = time.perf_counter()
    r = o.dembx(u, g, gg0, max_steps=iters)
    dt = time.perf_counter() - t0
    done = r["lstep"]
    return 3.0 * p.ns * done / dt, O.num_threads(), dt, done


def run_reference(args):
    ws, rank, local, pg = _dist()
    if rank != 0:
        return 0
    p, pix, rod = _workload(args.n)
    rate, cores, dt, done = cpu_oracle_rate(p, pix, rod, args.warmup, args.steps)
    sample = (f"{done} PCG iterations of the {args.n}^3 workload after {args.warmup} warm-up iterations "
              f"(each dembx call includes its block-Jacobi build, as in the reference)")
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / max(done, 1) * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded generator, shapes/distributions of the 500^3 config)",
        "config": {"workload": f"c2_polycrystal_{args.n}", "grid": [args.n] * 3, "dof": 3 * p.ns,
                   "grains": p.nphase - 1, "implementation": "CPU oracle (C/OpenMP port of dembx_OpenMP)"},
        "cpu_baseline": {"value": rate, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    ws, rank, local, pg = _dist()
    import numpy as np

    e3d = _load_package()
    p, pix, rod = _workload(args.n)
    p.device = local
    K, Wm = args.steps, args.warmup
    ns = p.ns

    # ---- device-resident measurement
    g = e3d.Elas3D(p)
    g.upload(pix, rod).femat().init_affine()
    g.energy()
    g.solve_begin()
    st = g.iterate(Wm)
    it0, ms0, l0 = st["iterations"], st["ms_iter"], g.launch_count()
    _barrier(pg)
    clocks = ClockSampler(local).start()
    time.sleep(0.3)
    t0 = time.perf_counter()
    st = g.iterate(K)
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    launches = g.launch_count() - l0
    done = st["iterations"] - it0
    if done != K or st["exit_reason"] != e3d.EXIT_RUNNING:
        raise RuntimeError(f"expected {K} running iterations, got {done} (exit {st['exit_reason']})")
    ms = st["ms_iter"] - ms0
    ms = _max_over_ranks(pg, ms)
    value = ws * 3.0 * ns * K / (ms / 1e3)
    g.close()

    # ---- end to end through the C ABI from pinned host buffers
    e2e = None
    try:
        import torch

        pin = torch.cuda.is_available()
        tpix = torch.from_numpy(pix.astype(np.int32))
        trod = torch.from_numpy(rod.astype(np.float64))
        tu = torch.empty(3 * ns, dtype=torch.float64)
        if pin:
            tpix, trod, tu = tpix.pin_memory(), trod.pin_memory(), tu.pin_memory()
        import ctypes as C

        L = e3d.load_library()
        dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int32)
        h = e3d.Elas3D(p)
        _barrier(pg)
        t0 = time.perf_counter()
        e3d._check(L.e3d_upload(h.handle, C.cast(tpix.data_ptr(), ip), C.cast(trod.data_ptr(), dp)), "upload")
        h.femat().init_affine()
        h.energy()
        h.solve_begin()
        st2 = h.iterate(K)
        s6 = np.zeros(6)
        e6 = np.zeros(6)
        e3d._check(L.e3d_stress(h.handle, e3d._dp(s6), e3d._dp(e6)), "stress")
        e3d._check(L.e3d_get_u(h.handle, C.cast(tu.data_ptr(), dp)), "get_u")
        t_e2e = time.perf_counter() - t0
        t_e2e = _max_over_ranks(pg, t_e2e)
        assert st2["iterations"] == K
        h.close()
        h2d = pix.nbytes + rod.nbytes
        d2h = tu.numel() * 8 + 96
        e2e = {"value": ws * 3.0 * ns * K / t_e2e, "unit": UNIT,
               "h2d_bytes_per_step": h2d / K, "d2h_bytes_per_step": d2h / K,
               "seconds": t_e2e, "pinned_host_buffers": bool(pin)}
    except Exception as ex:  # report, do not hide
        e2e = {"value": None, "unit": UNIT, "error": str(ex)}

    # ---- roofline of the dominant kernel (pcg_persistent_kernel)
    hbm, hbm_src = _peaks()
    t_iter = ms / 1e3 / K
    achieved = BYTES_PER_NODE_ITER * ns / t_iter / 1e9
    traffic_node, fp64_inst_node = _traffic_per_node()
    fp64_peak, fp32_peak = e3d.probe_peaks(local)
    roof = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
            "frac": achieved / hbm, "peak_source": f"{hbm_src} copy bandwidth (MEASURED_PEAKS.json)",
            "traffic": traffic_node * ns if traffic_node else None,
            "kernel": "pcg_persistent_kernel (one PCG iteration)",
            "algorithmic_bytes_per_node": BYTES_PER_NODE_ITER}
    comp = {"bound": "fp64", "peak_tflops": fp64_peak, "peak_source": "measured DFMA probe (e3d_probe_peaks)",
            "fp32_peak_tflops": fp32_peak,
            "algorithmic_tflops_dense_equiv": FLOPS_PER_NODE_ITER * ns / t_iter / 1e12}
    if fp64_inst_node:
        # executed FP64 instructions (ncu), each FMA counted as 2 flops at most
        comp["executed_fp64_inst_per_node"] = fp64_inst_node
        comp["executed_fp64_inst_per_s"] = fp64_inst_node * ns / t_iter
        comp["frac_of_fp64_issue_peak"] = fp64_inst_node * ns / t_iter / (fp64_peak * 1e12 / 2.0)
    roof["fp64_pipe"] = comp

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": K, "warmup": Wm,
        "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded generator, shapes/distributions of the 500^3 config)",
        "config": {"workload": f"c2_polycrystal_{args.n}", "grid": [args.n] * 3, "dof": 3 * ns,
                   "grains": p.nphase - 1, "zener_A": 2.0, "pores": "1% spherical, r ~ lognormal(ln 3, 0.4)",
                   "precision": "fp64", "criterion": "reference (sqrt(z.g/|g0|^2))",
                   "step": "one PCG iteration (fused apply + updates, persistent kernel)",
                   "l2": "inputs larger than L2 (3 GB per vector)", "parallelism": f"replicas x{ws}",
                   "e2e": "C-ABI calls from pinned host buffers: upload..K iterations..stress, get_u"},
        "e2e": e2e, "gpu_launches": launches, "clocks": clk, "roofline": roof,
        "wall_ms_per_step": wall / K * 1e3,
    }
    # ---- CPU baseline (rank 0, N = 1 only): the oracle on the host cores
    if ws == 1 and not args.no_cpu:
        try:
            rate, cores, dt, done = cpu_oracle_rate(p, pix, rod, 0, args.cpu_iters)
            line["cpu_baseline"] = {
                "value": rate, "unit": UNIT, "cores": cores, "kind": "port",
                "sample": f"{done} oracle PCG iterations of the same {args.n}^3 workload "
                          f"({dt:.1f} s, includes one block-Jacobi build)"}
        except Exception as ex:
            line["cpu_baseline"] = {"value": None, "unit": UNIT, "cores": None, "kind": "port",
                                    "sample": f"failed: {ex}"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if pg is not None:
        pg.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=500, help="grid edge (default: the 500^3 config)")
    ap.add_argument("--cpu-iters", type=int, default=3)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    args = ap.parse_args()
    if args.warmup < 0 or args.steps < 1:
        ap.error("steps >= 1 and warmup >= 0")
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
