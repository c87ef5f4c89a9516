"""The C-ABI library loads on a machine without a GPU and exports every
function declared in include/*.h (no compute calls)."""
import os
import re
import subprocess

import pytest

import elas3d_xtal_gb300 as e3d

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for h in ("e3d_gpu.h", "e3d_micro.h", "e3d_batch.h"):
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(e3d_[A-Za-z0-9_]+)\s*\(", text))
    return names


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(e3d.LIB_PATH):
        import importlib.util

        spec = importlib.util.spec_from_file_location("e3d_build", os.path.join(ROOT, "elas3d-xtal_gb300", "build.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        try:
            mod.build()
        except RuntimeError as ex:
            pytest.skip(f"cannot build the library here: {ex}")
    return e3d.load_library()


def test_every_declared_symbol_is_exported(lib):
    declared = _declared()
    assert len(declared) >= 30
    for name in sorted(declared):
        assert hasattr(lib, name), name
    assert declared == set(e3d.EXPORTED_SYMBOLS)


def test_exports_match_nm(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", e3d.LIB_PATH], capture_output=True, text=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln and ln.split()[-1].startswith("e3d_")}
    assert _declared() <= exported


def test_strerror_and_defaults_without_gpu(lib):
    assert e3d.strerror(e3d.E3D_ERR_OOM).startswith("device memory")
    p = e3d.ProblemC()
    lib.e3d_problem_defaults(p, 10, 11, 12, 5)
    assert (p.nx, p.ny, p.nz, p.nphase) == (10, 11, 12, 5)
    assert abs(p.tol - 1e-8) < 1e-15 and p.max_iter == 10000 and p.strain[2] == 1e-3
    assert p.c11 == 206e9 and p.flag_m == 1


def test_struct_layout_matches_header(lib):
    import ctypes as C

    # e3d_problem_t: 14 int32/float (56 B) + 11 doubles (88 B) + int64 = 152 B
    assert C.sizeof(e3d.ProblemC) == 152
    assert C.sizeof(e3d.SolveStatsC) == 16 + 6 * 8


def test_fortran_module_matches_the_c_abi():
    """The iso_c_binding module (source only: no Fortran compiler here) names
    only exported symbols and mirrors e3d_problem_t / e3d_solve_stats_t field
    for field."""
    import re

    src = open(os.path.join(ROOT, "elas3d-xtal_gb300", "fortran", "elas3d_gpu_mod.f90")).read()
    names = re.findall(r'bind\(C, name="(e3d_[A-Za-z0-9_]+)"\)', src)
    assert names and set(names) <= set(e3d.EXPORTED_SYMBOLS)

    def fortran_fields(tname):
        body = src.split(f"type, bind(C) :: {tname}")[1].split("end type")[0]
        out = []
        for line in body.splitlines():
            line = line.split("!")[0]
            if "::" in line:
                out += [re.sub(r"\(.*\)", "", f).strip() for f in line.split("::")[1].split(",")]
        return out

    assert fortran_fields("e3d_problem_t") == [f for f, _ in e3d.ProblemC._fields_]
    assert fortran_fields("e3d_solve_stats_t") == [f for f, _ in e3d.SolveStatsC._fields_]


C_CALLER = r"""
#include <stdio.h>
#include <string.h>
#include "e3d_gpu.h"
#include "e3d_batch.h"
#include "e3d_micro.h"

int main(void) {
  e3d_problem_t p;
  e3d_problem_defaults(&p, 8, 8, 8, 3);
  if (p.nx != 8 || p.nphase != 3) return 1;
  e3d_handle_t* h = NULL;
  p.nx = 0; /* refused before any CUDA call */
  if (e3d_create(&h, &p) != E3D_ERR_INPUT || h != NULL) return 2;
  if (strlen(e3d_strerror(E3D_ERR_TIMEOUT)) == 0) return 3;
  e3d_batch_opts_t o;
  e3d_batch_opts_defaults(&o);
  if (o.load_cases != 0) return 4;
  int32_t pix[8];
  double rod[3];
  /* host generator: 2x2x2 voxels, one grain */
  if (e3d_micro_grains(2, 2, 2, 1, 0.0, 1, pix, rod) != 0) return 5;
  for (int i = 0; i < 8; ++i)
    if (pix[i] != 1) return 6;
  printf("ok\n");
  return 0;
}
"""


def test_plain_c_caller_compiles_links_and_runs(lib, tmp_path):
    """A C99 program (no C++ anywhere) includes all three headers with
    -pedantic -Werror, links against the library and calls its GPU-free entry
    points: the ABI is usable from C, and so from cgo, Fortran or any FFI."""
    src = tmp_path / "caller.c"
    src.write_text(C_CALLER)
    exe = tmp_path / "caller"
    libdir = os.path.dirname(e3d.LIB_PATH)
    cmd = ["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", os.path.join(ROOT, "include"),
           str(src), "-L", libdir, "-le3d_gpu", f"-Wl,-rpath,{libdir}", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and r.stdout.strip() == "ok", (r.returncode, r.stdout, r.stderr)
