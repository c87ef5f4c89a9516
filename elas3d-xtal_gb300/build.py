"""Build recipe for the sm_103a library (in-tree, no cmake).

Produces ``elas3d-xtal_gb300/_build/libe3d_gpu.so`` from
``csrc/e3d_gpu.cu`` (nvcc, ``-gencode arch=compute_103a,code=sm_103a``) and
``csrc/microgen.cpp`` (g++, portable flags so the same recipe builds on x86-64
and AArch64).  Translation units compile in parallel; the step is skipped when
the library is newer than every source.

``build(bounds=True)`` makes the bounds-checked debug variant,
``_build/bounds/libe3d_gpu_bounds.so``: the same sources compiled with
``-DE3D_BOUNDS`` (every checked index compared with its buffer's length and
recorded, never trapping; ``e3d_debug_bounds`` reads the record).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libe3d_gpu.so")
DRIVER = os.path.join(OUT, "e3d_run")
BOUNDS_OUT = os.path.join(OUT, "bounds")
BOUNDS_LIB = os.path.join(BOUNDS_OUT, "libe3d_gpu_bounds.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build the library")
    return cand


def _sources():
    drv = os.path.join(PKG, "driver")
    return [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC))
            if f.endswith((".cu", ".cuh", ".cpp", ".h"))] + \
           [os.path.join(INCLUDE, f) for f in sorted(os.listdir(INCLUDE)) if f.endswith(".h")] + \
           [os.path.join(drv, f) for f in sorted(os.listdir(drv)) if f.endswith(".cpp")]


def up_to_date(bounds: bool = False) -> bool:
    targets = [BOUNDS_LIB] if bounds else [LIB, DRIVER]
    if not all(os.path.exists(t) for t in targets):
        return False
    t = min(os.path.getmtime(t) for t in targets)
    return all(os.path.getmtime(s) <= t for s in _sources())


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False, bounds: bool = False) -> str:
    lib = BOUNDS_LIB if bounds else LIB
    if not force and up_to_date(bounds):
        return lib
    out = BOUNDS_OUT if bounds else OUT
    os.makedirs(out, exist_ok=True)
    nvcc = _nvcc()
    cu_units = ["e3d_gpu", "e3d_noalloc", "e3d_batch", "microgen_gpu"]
    cu_objs = [os.path.join(out, u + ".o") for u in cu_units]
    cpp_obj = os.path.join(out, "microgen.o")
    h5_units = ["h5lite", "e3d_h5"]
    h5_objs = [os.path.join(out, u + ".o") for u in h5_units]
    cu_cmds = []
    for u, o in zip(cu_units, cu_objs):
        cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", *(["-DE3D_BOUNDS"] if bounds else []),
               "-I", INCLUDE, "-I", CSRC, "-c", os.path.join(CSRC, u + ".cu"), "-o", o]
        if ptxas_info:
            cmd[1:1] = ["-Xptxas", "-v"]
        cu_cmds.append(cmd)
    cpp_cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-Wall", "-I", INCLUDE,
               "-c", os.path.join(CSRC, "microgen.cpp"), "-o", cpp_obj]

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        return r.stdout + r.stderr

    h5_cmds = [["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", "-I", INCLUDE, "-c", os.path.join(CSRC, u + ".cpp"),
                "-o", o] for u, o in zip(h5_units, h5_objs)]
    with ThreadPoolExecutor(len(cu_cmds) + 1 + len(h5_cmds)) as ex:
        logs = list(ex.map(run, [*cu_cmds, cpp_cmd, *h5_cmds]))
    link = [nvcc, *ARCH, "-shared", "-o", lib + ".tmp", *cu_objs, cpp_obj, *h5_objs, "-Xcompiler", "-fopenmp",
            "-lgomp"]
    logs.append(run(link))
    os.replace(lib + ".tmp", lib)
    if bounds:
        if verbose or ptxas_info:
            sys.stdout.write("".join(logs))
        return lib
    # command-line driver (mirrors `program elas3d`), linked against the library
    drv = ["g++", "-O2", "-std=c++17", "-Wall", "-I", INCLUDE, os.path.join(PKG, "driver", "e3d_run.cpp"),
           "-L", OUT, "-le3d_gpu", "-Wl,-rpath,$ORIGIN", "-o", DRIVER + ".tmp"]
    logs.append(run(drv))
    os.replace(DRIVER + ".tmp", DRIVER)
    if verbose or ptxas_info:
        sys.stdout.write("".join(logs))
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, ptxas_info="-v" in sys.argv, bounds="--bounds" in sys.argv))
