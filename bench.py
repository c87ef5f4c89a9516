#!/usr/bin/env python
"""Benchmark: plain FP64 PCG of the voxel-FE elasticity solve on GB300.

Metric: DOF-iterations per second (3*ns*iterations / PCG time) on the
500^3 periodic polycrystal (375M DOF, 8000 Voronoi grains, uniform SO(3)
orientations, cubic 240/150 GPa with Zener ratio A = 2, 1 % zero-stiffness
spherical pores, exx = 1e-3) -- seeded synthetic input with the shapes and
distributions of that configuration.  One step = one PCG iteration
(apply + dot products + updates).

  value : device-resident state, K iterations timed with CUDA events on the
          library's stream (an iteration streams 364 B per node in FP64, 184
          in the mixed form: 45 / 23 GB at 500^3, far more than the L2 holds)
  e2e   : the same metric through the C ABI from pinned host buffers: upload,
          femat, affine guess, energy, block-Jacobi, K iterations, stress and
          the download of u are all inside the timed region
  time_to_solution, mixed, batch, serve : the rest of the headline metric on
          the same line -- full 500^3 solves (FP64 and mixed, with the mixed
          result's error against FP64), the mixed inner-loop rate with its
          roofline, batched solves/s and served solves/s with p50/p99 latency,
          each against plain sequential FP64 GPU solves (--no-forms skips them)
  --impl reference : the CPU oracle (C/OpenMP restatement of the reference's
          PCG) on this machine's host cores, same workload, config and metric;
          it loads only the oracle's own libraries

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
BYTES_PER_NODE_ITER_MIXED = 184.0  # the same with FP32 vectors, int32 phases and FP32 Minv (mixed inner loop)
METRIC_MIXED = "DOF-iters/s (mixed-precision PCG inner loop incl. FP64 replacement, 500^3 polycrystal)"
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


def _traffic_per_node(mixed: bool = False):
    """DRAM bytes per node per iteration of the PCG kernel from the committed
    ncu capture summary (profiles/pcg_fp64_traffic.json, or pcg_f32_traffic.json
    for the mixed inner loop), if present."""
    path = os.path.join(ROOT, "profiles", "pcg_f32_traffic.json" if mixed else "pcg_fp64_traffic.json")
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
    """The GPU arm's input: the package's seeded generator."""
    _load_package()
    from elas3d_xtal_gb300 import workloads as W

    p, pix, rod = W.c2(n=n)
    p.max_iter = 1_000_000
    return p, pix, rod


def _oracle():
    d = os.path.join(ROOT, "oracle")
    if d not in sys.path:
        sys.path.insert(0, d)
    import oracle as O

    return O


def plain_config(n: int, ns: int, ngrains: int, ws: int) -> dict:
    """The workload description both arms print, key for key."""
    return {"workload": f"c2_polycrystal_{n}", "grid": [n] * 3, "dof": 3 * ns, "grains": ngrains,
            "zener_A": 2.0, "pores": "1% spherical, r ~ lognormal(ln 3, 0.4)", "precision": "fp64",
            "criterion": "reference (sqrt(z.g/|g0|^2))",
            "step": "one PCG iteration (apply + dot products + updates) over the whole grid",
            "l2": f"each iteration streams {BYTES_PER_NODE_ITER * ns / 1e9:.2f} GB, more than the 126 MB L2 holds",
            "parallelism": f"replicas x{ws}"}


def oracle_iterations(O, op, pix, rod, warmup: int, steps: int, budget_s: float | None = None):
    """Oracle PCG iterations on the host cores.  Set-up (femat, energy, the
    block-Jacobi build, z0) is not timed; `warmup` iterations run untimed, then
    `steps` more iterations of the same solve are timed (capped so that they
    take about budget_s seconds when it is given).  Returns (seconds,
    iterations timed, threads, set-up seconds)."""
    t0 = time.perf_counter()
    o = O.Oracle(op, pix, rod).femat()
    u = o.affine_u()
    g, _ = o.energy(u)
    gg0 = float(g @ g)
    pcg = o.pcg(u, g, gg0)
    del u, g
    t_setup = time.perf_counter() - t0
    try:
        if warmup > 0:
            tw = time.perf_counter()
            if pcg.iterate(warmup) >= 0:
                raise RuntimeError("the oracle solve ended during the warm-up")
            tw = (time.perf_counter() - tw) / warmup
            if budget_s is not None:
                steps = max(1, min(steps, int(budget_s / max(tw, 1e-9))))
        t0 = time.perf_counter()
        ended = pcg.iterate(steps)
        dt = time.perf_counter() - t0
    finally:
        info = pcg.close()
    done = steps if ended < 0 else info["lstep"] - warmup
    return dt, done, O.num_threads(), t_setup


def run_reference(args):
    """The reference's CPU PCG (the oracle port of dembx_OpenMP) on the host
    cores: the same 500^3 input, built by the same generator compiled on its
    own (no CUDA library in this process), every requested warm-up and timed
    iteration of one solve."""
    ws, rank, local, pg = _dist()
    if rank != 0:
        return 0
    O = _oracle()
    import workload as OW

    op, pix, rod = OW.c2(n=args.n, ldemb=1_000_000)
    dt, done, cores, t_setup = oracle_iterations(O, op, pix, rod, args.warmup, args.steps)
    rate = 3.0 * op.ns * done / dt
    sample = (f"{done} timed PCG iterations of one solve of the {args.n}^3 workload after {args.warmup} untimed "
              f"warm-up iterations; femat, energy and the block-Jacobi build ({t_setup:.1f} s) are set-up, "
              f"outside the timed region as on the GPU side")
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": ws,
        "steps": done, "warmup": args.warmup, "ms_per_step": dt / max(done, 1) * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded generator, shapes/distributions of the 500^3 config)",
        "config": plain_config(args.n, op.ns, op.nphase - 1, ws),
        "implementation": "CPU oracle: C/OpenMP restatement of dembx_OpenMP (src/elas3dxtal_pcg.f90:1356-2043)",
        "cpu_baseline": {"value": rate, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def _roofline(e3d, bytes_node, ns, t_iter, mixed, path, local):
    hbm, hbm_src = _peaks()
    achieved = bytes_node * ns / t_iter / 1e9
    traffic_node, fp64_inst_node = _traffic_per_node(mixed)
    roof = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
            "frac": achieved / hbm, "peak_source": f"{hbm_src} copy bandwidth (MEASURED_PEAKS.json)",
            "traffic": traffic_node * ns if traffic_node else None,
            "kernel": f"pcg_persistent_kernel<{'float' if mixed else 'double'}> (one PCG iteration; stencil path {path})",
            "algorithmic_bytes_per_node": bytes_node}
    if not mixed:
        fp64_peak, fp32_peak = e3d.probe_peaks(local)
        comp = {"bound": "fp64", "peak_tflops": fp64_peak, "peak_source": "measured DFMA probe (e3d_probe_peaks)",
                "fp32_peak_tflops": fp32_peak,
                "algorithmic_tflops_dense_equiv": FLOPS_PER_NODE_ITER * ns / t_iter / 1e12}
        if fp64_inst_node:
            # executed FP64 instructions (ncu), each FMA counted as 2 flops at most
            comp["executed_fp64_inst_per_node"] = fp64_inst_node
            comp["executed_fp64_inst_per_s"] = fp64_inst_node * ns / t_iter
            comp["frac_of_fp64_issue_peak"] = fp64_inst_node * ns / t_iter / (fp64_peak * 1e12 / 2.0)
        roof["fp64_pipe"] = comp
    return roof


E2E_RUNS = 3  # end-to-end runs per bench line (median reported)


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
    path = g.stencil_path()
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
        runs = []
        for _rep in range(E2E_RUNS):  # each from a fresh handle; the median is reported
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
            runs.append(_max_over_ranks(pg, time.perf_counter() - t0))
            assert st2["iterations"] == K
            h.close()
        t_e2e = float(np.median(runs))
        h2d = pix.nbytes + rod.nbytes
        d2h = tu.numel() * 8 + 96
        e2e = {"value": ws * 3.0 * ns * K / t_e2e, "unit": UNIT,
               "h2d_bytes_per_step": h2d / K, "d2h_bytes_per_step": d2h / K,
               "seconds": t_e2e, "runs_seconds": runs, "pinned_host_buffers": bool(pin)}
    except Exception as ex:  # report, do not hide
        e2e = {"value": None, "unit": UNIT, "error": str(ex)}

    roof = _roofline(e3d, BYTES_PER_NODE_ITER, ns, ms / 1e3 / K, False, path, local)
    cfg = plain_config(args.n, ns, p.nphase - 1, ws)
    cfg["e2e"] = ("C-ABI calls from pinned host buffers: upload..K iterations..stress, get_u; "
                  f"median of {E2E_RUNS} runs, each from a fresh handle")
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": K, "warmup": Wm,
        "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded generator, shapes/distributions of the 500^3 config)",
        "config": cfg, "e2e": e2e, "gpu_launches": launches, "clocks": clk, "roofline": roof,
        "wall_ms_per_step": wall / K * 1e3,
    }
    # ---- CPU baseline (rank 0, N = 1 only): the oracle on the host cores
    if ws == 1 and not args.no_cpu:
        try:
            O = _oracle()
            s = p.strain
            op = O.Problem(p.nx, p.ny, p.nz, p.nphase, flag_m=p.flag_m, c11=p.c11, c12=p.c12, c44=p.c44,
                           e1=p.e1, nu1=p.nu1, exx=s[0], eyy=s[1], ezz=s[2], exz=s[3], eyz=s[4], exy=s[5],
                           tol=p.tol, ldemb=p.max_iter)
            dt, done, cores, _ = oracle_iterations(O, op, pix, rod, 0, args.cpu_iters)
            line["cpu_baseline"] = {
                "value": 3.0 * ns * done / dt, "unit": UNIT, "cores": cores, "kind": "port",
                "sample": f"{done} oracle PCG iterations of the same {args.n}^3 solve ({dt:.1f} s; "
                          f"set-up and block-Jacobi build not timed)"}
        except Exception as ex:
            line["cpu_baseline"] = {"value": None, "unit": UNIT, "cores": None, "kind": "port",
                                    "sample": f"failed: {ex}"}
    # ---- the rest of the headline metric (N = 1 only)
    if ws == 1 and not args.no_forms:
        for key, fn in (("mixed", mixed_rate), ("time_to_solution", form_solve), ("batch", form_batch),
                        ("serve", form_serve)):
            t0 = time.perf_counter()
            try:
                line[key] = fn(args)
            except Exception as ex:  # report, do not hide
                line[key] = {"error": f"{type(ex).__name__}: {ex}"}
            line[key]["bench_seconds"] = time.perf_counter() - t0
        if line["mixed"].get("ms_per_iteration"):
            line["mixed"]["speedup_vs_fp64_iteration"] = (ms / K) / line["mixed"]["ms_per_iteration"]
    if rank == 0:
        print(json.dumps(line), flush=True)
    if pg is not None:
        pg.destroy_process_group()
    return 0


# ---------------------------------------------------------------------------
# The rest of the headline metric: the mixed inner-loop rate, full solves FP64
# vs mixed, the batched effective-stiffness ensemble and the continuous-batching
# server.  Each returns a dict; `--form` prints one alone, the default run puts
# all of them on the plain line.
def mixed_rate(args) -> dict:
    """Mixed-precision PCG on the same 500^3 workload: the FP32 inner
    iteration alone, then 100 iterations with the FP64 residual replacement
    every 50 inside the window."""
    e3d = _load_package()
    p, pix, rod = _workload(args.n)
    p.precision = e3d.PREC_MIXED
    p.refine_every = 50
    ns = p.ns
    with e3d.Elas3D(p) as g:
        g.upload(pix, rod).femat().init_affine()
        g.energy()
        g.solve_begin()
        st = g.iterate(3)
        path = g.stencil_path()
        clocks = ClockSampler(p.device).start()
        time.sleep(0.3)
        n_in = 46  # iterations 4..49: no replacement inside
        st1 = g.iterate(n_in)
        ms_in = st1["ms_iter"] - st["ms_iter"]
        n_rep = 100  # iterations 50..149: replacements after 50 and 100
        st2 = g.iterate(n_rep)
        ms_rep = st2["ms_iter"] - st1["ms_iter"]
        clk = clocks.stop()
        if st2["iterations"] != 3 + n_in + n_rep or st2["exit_reason"] != e3d.EXIT_RUNNING:
            raise RuntimeError(f"mixed solve ended early ({st2['iterations']} iterations)")
        refinements = st2["refinements"] - st1["refinements"]
    t_in = ms_in / 1e3 / n_in
    t_rep = ms_rep / 1e3 / n_rep
    return {"metric": METRIC_MIXED, "value": 3.0 * ns / t_rep, "unit": UNIT,
            "ms_per_iteration": t_rep * 1e3, "replacements_in_window": refinements,
            "inner": {"value": 3.0 * ns / t_in, "ms_per_iteration": t_in * 1e3,
                      "roofline": _roofline(e3d, BYTES_PER_NODE_ITER_MIXED, ns, t_in, True, path, 0)},
            "roofline": _roofline(e3d, BYTES_PER_NODE_ITER_MIXED, ns, t_rep, True, path, 0),
            "speedup_vs_fp64_iteration": None, "clocks": clk,
            "dtype": "f32 stencil/preconditioner/vectors; FP64 dots, scalars, replacement",
            "config": {"workload": f"c2_polycrystal_{args.n}", "refine_every": 50}}


def _full_solve(e3d, p, pix, rod, precision, refine_every=0, refine_decades=0):
    p.precision = precision
    p.refine_every, p.refine_decades = refine_every, refine_decades
    p.max_iter = 100000
    g = e3d.Elas3D(p)
    g.upload(pix, rod)
    t0 = time.perf_counter()
    r = g.run()
    dt = time.perf_counter() - t0
    g.close()
    r["seconds"] = dt
    return r


def form_solve(args) -> dict:
    """Time to solution (femat, energy x2, PCG, stress; upload excluded) of the
    500^3 solve, plain FP64 and mixed, and the mixed result's error.  With
    --workload c3: the 400^3 Laguerre polycrystal with 3 % ellipsoidal voids at
    Zener ratio --zener."""
    e3d = _load_package()
    if args.workload == "c3":
        from elas3d_xtal_gb300 import workloads as W

        p, pix, rod = W.c3(n=args.n, A=args.zener)
    else:
        p, pix, rod = _workload(args.n)
    p.criterion = e3d.CRIT_PRECOND_REL if args.criterion == "precond" else e3d.CRIT_REF
    clocks = ClockSampler(p.device).start()
    a = _full_solve(e3d, p, pix, rod, e3d.PREC_FP64)
    b = _full_solve(e3d, p, pix, rod, e3d.PREC_MIXED, refine_every=50)
    c = _full_solve(e3d, p, pix, rod, e3d.PREC_MIXED, refine_every=1000, refine_decades=3)
    clk = clocks.stop()

    def errs(r):
        return (abs(r["utot"] - a["utot"]) / abs(a["utot"]),
                float(((r["strav"] - a["strav"]) ** 2).sum() ** 0.5 / (a["strav"] ** 2).sum() ** 0.5))

    err, serr = errs(b)
    cerr, cserr = errs(c)
    return {"metric": f"time to solution, {args.n}^3 (s)", "form": "solve", "unit": "s", "higher_is_better": False,
            "value": b["seconds"], "fp64_seconds": a["seconds"], "speedup_mixed_vs_fp64": a["seconds"] / b["seconds"],
            "iterations": {"fp64": a["iterations"], "mixed": b["iterations"]}, "refinements": b["refinements"],
            "energy_rel_err_mixed_vs_fp64": err, "stress_rel_err_mixed_vs_fp64": serr,
            "energy": {"fp64": a["utot"], "mixed": b["utot"]},
            "criterion": args.criterion, "true_rel": {"fp64": a["true_rel"], "mixed": b["true_rel"]},
            "mixed_replacement": "FP64 residual replacement every 50 inner iterations",
            "mixed_on_residual_drop": {
                "seconds": c["seconds"], "speedup_vs_fp64": a["seconds"] / c["seconds"],
                "iterations": c["iterations"], "refinements": c["refinements"],
                "energy_rel_err_vs_fp64": cerr, "stress_rel_err_vs_fp64": cserr,
                "replacement": "when the FP32 residual falls three decades below the last FP64 one, "
                               "at most every 1000 iterations, and at the stop test"},
            "clocks": clk,
            "config": {"workload": (f"c3_laguerre_{args.n}_A{args.zener:g}" if args.workload == "c3"
                                    else f"c2_polycrystal_{args.n}"),
                       "dof": 3 * p.ns, "grains": p.nphase - 1, "zener_A": 2.0 * p.c44 / (p.c11 - p.c12),
                       "includes": "femat, energy x2, PCG, stress (upload excluded)"}}


def _sequential_fp64(e3d, jobs, crit):
    """Plain FP64 GPU solves one after another: (seconds per solve, energies)."""
    secs, energies = [], []
    for rv, s in jobs:
        p = e3d.Problem(*rv["shape"], rv["ngrains"] + 1, c11=rv["c11"], c12=rv["c12"], c44=rv["c44"],
                        strain=tuple(s))
        p.criterion = crit
        rr = _full_solve(e3d, p, rv["pix"], rv["rodrigues"], e3d.PREC_FP64)
        secs.append(rr["seconds"])
        energies.append(rr["utot"])
    return secs, energies


def form_batch(args) -> dict:
    import numpy as np

    e3d = _load_package()
    from elas3d_xtal_gb300 import workloads as W

    if args.rve_edge > 0:  # probe: equal RVEs of one edge
        rves = [W.rve(args.rve_edge, 100, 11 + i, A=2.0, pore_frac=0.01) for i in range(args.rves)]
    else:
        rves = W.ensemble(args.rves, seed=4)
    nodes = sum(int(np.prod(r["shape"])) for r in rves)
    t0 = time.perf_counter()
    crit = e3d.CRIT_PRECOND_REL if args.criterion == "precond" else e3d.CRIT_REF
    b = e3d.Batch(rves, max_iter=args.max_iter, criterion=crit, parts=args.parts, load_cases=args.load_cases,
                  refine_every=args.refine_every)
    t_create = time.perf_counter() - t0
    ceff, sec = b.solve()  # first solve
    clocks = ClockSampler(0).start()
    ceff, sec = b.solve()  # graph replay (timed)
    clk = clocks.stop()
    res = b.results()
    parts = b.parts()
    b.close()
    nj = len(res)
    iters = [r["iterations"] for r in res]
    node_iters = float(sum(int(np.prod(rves[r["rve"]]["shape"])) * r["iterations"] for r in res))
    conv = sum(r["status"] == e3d.EXIT_CONVERGED for r in res)
    # plain sequential FP64 GPU solves of a seeded sample of the same jobs
    rng = np.random.default_rng(0)
    sample = rng.choice(nj, size=min(args.sample, nj), replace=False)
    jobs = []
    for j in sample:
        r = res[int(j)]
        s = [0.0] * 6
        s[r["load_case"]] = 1e-3 if r["load_case"] < 3 else 0.5e-3
        jobs.append((rves[r["rve"]], s))
    seq, energies = _sequential_fp64(e3d, jobs, crit)
    errs = [abs(e - res[int(j)]["utot"]) / abs(e) for j, e in zip(sample, energies)]
    seq_rate = len(seq) / sum(seq) if seq else None
    return {"metric": "batched solves/s (256 RVEs x 6 load cases, mixed precision)", "form": "batch",
            "value": nj / sec, "unit": "solves/s", "higher_is_better": True, "seconds": sec,
            "solves": nj, "converged": conv, "iterations": {"min": min(iters), "max": max(iters),
                                                           "mean": float(np.mean(iters))},
            "parts_hist": {str(k): int((parts == k).sum()) for k in sorted(set(parts.tolist()))},
            "tile_z_hist": {str(t): sum(1 for r in res if r["tile_z"] == t)
                            for t in sorted(set(r["tile_z"] for r in res))},
            "create_seconds": t_create, "rve_nodes": nodes, "clocks": clk,
            "work": {"node_iterations": node_iters, "dof_iters_per_s": 3.0 * node_iters / sec},
            "sequential_fp64": {"solves_per_s": seq_rate, "sample": len(seq),
                                "sample_seconds": sum(seq),
                                "energy_rel_err_vs_batched": ({"max": max(errs), "median": float(np.median(errs))}
                                                              if errs else None)},
            "criterion": args.criterion,
            "speedup_vs_sequential_fp64": (nj / sec) / seq_rate if seq_rate else None,
            "config": {"workload": "ensemble", "rves": len(rves), "edges": "U{32..96}", "grains": "8-200",
                       "zener": "{0.5,0.75,1,1.5,2,3,4,5}", "pores": "0-2 %", "load_cases": 6,
                       "launch": "one persistent launch from a CUDA graph", "refine_every": args.refine_every}}


def form_serve(args) -> dict:
    """Continuous batching: a seeded Poisson stream of single-load-case
    requests against fewer slots than requests, so that most requests join
    while others are on the GPU.  The sequential FP64 baseline serves the
    first `sample` requests one after another at their own arrival times."""
    import numpy as np

    e3d = _load_package()
    from elas3d_xtal_gb300 import workloads as W

    rng = np.random.default_rng(5)
    reqs = []
    for i in range(args.requests):
        n = int(rng.integers(48, args.serve_max_edge + 1))
        ng = int(rng.integers(16, 1001))
        A = float(rng.uniform(0.5, 5.0))
        pf = float(rng.uniform(0.0, 0.03))
        rv = W.rve(n, ng, 5000 + i, A=A, pore_frac=pf)
        lc = int(rng.integers(0, 6))
        s = np.zeros(6)
        s[lc] = 1e-3 if lc < 3 else 0.5e-3
        reqs.append((rv, s))
    gaps = rng.exponential(1.0 / args.rate, size=len(reqs))
    arrivals = np.cumsum(gaps)
    budget = int(150e9)
    crit = e3d.CRIT_PRECOND_REL if args.criterion == "precond" else e3d.CRIT_REF
    srv = e3d.Server(max_active=args.slots, round_iters=args.round_iters, max_iter=20000, hbm_budget=budget,
                     refine_every=args.refine_every, round_balance=bool(args.round_balance),
                     criterion=crit)
    clocks = ClockSampler(0).start()
    t0 = time.perf_counter()
    ids, done_at = [], {}
    busy_arrivals, max_pending, rounds = 0, 0, 0
    pend = 0
    i = 0
    while True:
        now = time.perf_counter() - t0
        while i < len(reqs) and arrivals[i] <= now:
            if pend > 0:
                busy_arrivals += 1  # others are queued or on the GPU: it joins mid-flight
            ids.append(srv.submit(*reqs[i]))
            i += 1
        pend = srv.step()
        rounds += 1
        max_pending = max(max_pending, pend)
        now = time.perf_counter() - t0
        for k, rid in enumerate(ids):
            if rid not in done_at and srv.result(rid) is not None:
                done_at[rid] = now
        if i >= len(reqs) and pend == 0:
            break
        if pend == 0 and i < len(reqs):
            time.sleep(max(0.0, arrivals[i] - now))
    total = time.perf_counter() - t0
    clk = clocks.stop()
    res = [srv.result(r) for r in ids]
    _, peak = srv.memory()
    srv.close()
    lat = np.array([done_at[rid] - arrivals[k] for k, rid in enumerate(ids)])
    conv = sum(r["status"] == e3d.EXIT_CONVERGED for r in res)
    node_iters = float(sum(int(np.prod(rv["shape"])) * r["iterations"] for (rv, _), r in zip(reqs, res)))
    # the same requests as plain sequential FP64 GPU solves, served in arrival order
    m = min(args.sample, len(reqs))
    seq, energies = _sequential_fp64(e3d, reqs[:m], crit)
    errs = [abs(e - r["utot"]) / abs(e) for e, r in zip(energies, res[:m])]
    tq, seq_lat = 0.0, []
    for a, d in zip(arrivals[:m], seq):
        tq = max(tq, a) + d
        seq_lat.append(tq - a)
    served_lat = lat[:m]
    return {"metric": "served solves/s (Poisson 200/s, edges 48-256, mixed precision)", "form": "serve",
            "value": len(reqs) / total, "unit": "solves/s", "higher_is_better": True, "requests": len(reqs),
            "converged": conv, "wall_seconds": total, "latency_s": {"p50": float(np.percentile(lat, 50)),
                                                                   "p99": float(np.percentile(lat, 99)),
                                                                   "max": float(lat.max())},
            "continuous_batching": {"arrived_while_busy": busy_arrivals, "max_pending": max_pending,
                                    "slots": args.slots, "rounds": rounds},
            "peak_hbm_bytes": peak, "hbm_budget": budget, "round_iters": args.round_iters,
            "round_balance": bool(args.round_balance),
            "criterion": args.criterion, "clocks": clk,
            "work": {"node_iterations": node_iters, "dof_iters_per_s": 3.0 * node_iters / total,
                     "iterations": {"min": int(min(r["iterations"] for r in res)),
                                    "max": int(max(r["iterations"] for r in res)),
                                    "mean": float(np.mean([r["iterations"] for r in res]))}},
            "sequential_fp64": ({"sample": m, "solves_per_s": m / sum(seq),
                                 "energy_rel_err_vs_served": {"max": max(errs), "median": float(np.median(errs))},
                                 "latency_s": {"p50": float(np.percentile(seq_lat, 50)),
                                               "p99": float(np.percentile(seq_lat, 99))},
                                 "served_latency_same_requests_s": {"p50": float(np.percentile(served_lat, 50)),
                                                                    "p99": float(np.percentile(served_lat, 99))},
                                 "queue_model": "each sampled request arrives at its own Poisson time and waits "
                                                "for the solves before it"} if m else {"sample": 0}),
            "config": {"workload": "serve", "arrivals": f"Poisson, mean {args.rate}/s, seed 5",
                       "edges": f"U{{48..{args.serve_max_edge}}}", "grains": "16-1000", "zener": "U[0.5,5]",
                       "pores": "0-3 %", "load": "one unit load case per request", "refine_every": args.refine_every}}


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=500, help="grid edge (default: the 500^3 config)")
    ap.add_argument("--cpu-iters", type=int, default=3)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-forms", action="store_true",
                    help="plain line only: skip the mixed rate, full solves, batch and serve keys")
    ap.add_argument("--form", choices=["plain", "mixed", "solve", "batch", "serve"], default="plain",
                    help="plain: the FP64 DOF-iters/s line (with every form on it); otherwise one form alone")
    ap.add_argument("--workload", choices=["c2", "c3"], default="c2",
                    help="solve form: c2 (the plain polycrystal) or c3 (Laguerre grains, 3 %% ellipsoidal voids)")
    ap.add_argument("--zener", type=float, default=2.0, help="solve form, c3: Zener ratio A")
    ap.add_argument("--rves", type=int, default=256, help="batch: ensemble size")
    ap.add_argument("--parts", type=int, default=0, help="batch: blocks per solve (0: autotune)")
    ap.add_argument("--rve-edge", type=int, default=0, help="batch probe: equal RVEs of this edge (0: the ensemble)")
    ap.add_argument("--load-cases", type=int, default=0, help="batch: load-case bit mask (0: all six)")
    ap.add_argument("--max-iter", type=int, default=20000, help="batch: iteration cap per solve")
    ap.add_argument("--refine-every", type=int, default=200,
                    help="batch/serve: FP32 inner iterations between FP64 residual replacements at most (the "
                         "engine also replaces after a 1e-3 residual drop, and every solve ends on an FP64 "
                         "residual; batch at 50 / 100 / 200: 184 / 196 / 204 solves/s)")
    ap.add_argument("--requests", type=int, default=256, help="serve: number of requests")
    ap.add_argument("--rate", type=float, default=200.0, help="serve: mean arrivals per second")
    ap.add_argument("--slots", type=int, default=32, help="serve: concurrent solves")
    ap.add_argument("--round-iters", type=int, default=50, help="serve: iterations per solve per round")
    ap.add_argument("--round-balance", type=int, default=0,
                    help="serve: 1 = smaller solves run up to 8x round-iters per round (0 = fixed rounds)")
    ap.add_argument("--serve-max-edge", type=int, default=256)
    ap.add_argument("--sample", type=int, default=32, help="batch/serve: sequential FP64 reference sample")
    ap.add_argument("--criterion", choices=["ref", "precond"], default="ref",
                    help="forms: ref = sqrt(z.g/|g0|^2) (the reference's test), precond = sqrt(z.g/z0.g0)")
    args = ap.parse_args()
    if args.warmup < 0 or args.steps < 1:
        ap.error("steps >= 1 and warmup >= 0")
    if args.impl == "reference":
        return run_reference(args)
    forms = {"mixed": mixed_rate, "solve": form_solve, "batch": form_batch, "serve": form_serve}
    if args.form in forms:
        print(json.dumps(forms[args.form](args)), flush=True)
        return 0
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
