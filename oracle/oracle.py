"""ctypes binding of the CPU oracle (oracle/e3d_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by the CPU-baseline leg of ``bench.py``.  The product path never imports it.

Parity status: unpinned by reference outputs (the reference ships no tests or
golden vectors and cannot be compiled here); pinned by analytical known-answer
tests and by the independent scipy restatement in ``oracle/np_ref.py``.

Arrays use the reference's layout (src/elas3dxtal_pcg.f90:155-181):
vectors are (3, ns) component-major ("SoA", Fortran u(ns,3)), ``pix`` is
1-based, ``dk`` is Fortran dk(nphase,8,3,8,3) and is returned here as a numpy
array indexed ``dk[j, b, i, a, p]`` (C order view of the Fortran buffer).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libe3d_oracle.so")


class OrcProblem(C.Structure):
    _fields_ = [
        ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
        ("nphase", C.c_int32), ("flag_m", C.c_int32),
        ("c11", C.c_double), ("c12", C.c_double), ("c44", C.c_double),
        ("e1", C.c_double), ("nu1", C.c_double),
        ("exx", C.c_double), ("eyy", C.c_double), ("ezz", C.c_double),
        ("exz", C.c_double), ("eyz", C.c_double), ("exy", C.c_double),
        ("tol", C.c_float), ("ldemb", C.c_int32), ("criterion", C.c_int32),
        ("divergence_reset", C.c_int32), ("block_size", C.c_int32), ("precond", C.c_int32),
    ]


class OrcResult(C.Structure):
    _fields_ = [
        ("utot0", C.c_double), ("utot", C.c_double), ("gg0", C.c_double),
        ("gg", C.c_double), ("rel_res", C.c_double),
        ("lstep", C.c_int32), ("exit_reason", C.c_int32), ("reset_count", C.c_int32),
        ("strav", C.c_double * 6), ("epsav", C.c_double * 6), ("C", C.c_double),
        ("t_femat", C.c_double), ("t_energy", C.c_double), ("t_pcg", C.c_double),
        ("t_stress", C.c_double),
    ]


def build() -> str:
    """Compile the oracle with its Makefile (portable flags) and return the .so path."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = C.CDLL(_LIB_PATH)
        dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int32)
        pp = C.POINTER(OrcProblem)
        L.orc_rotate_stiffness.argtypes = [C.c_int32, dp, C.c_double, C.c_double, C.c_double, dp]
        L.orc_cmod.argtypes = [pp, dp, dp]
        L.orc_dk.argtypes = [pp, dp, dp]
        L.orc_build_ib.argtypes = [C.c_int32, C.c_int32, C.c_int32, ip]
        L.orc_femat_bc.argtypes = [pp, ip, ip, dp, dp, dp]
        L.orc_femat.argtypes = [pp, ip, ip, dp, dp, dp, dp, dp]
        L.orc_affine_u.argtypes = [pp, dp]
        L.orc_apply.argtypes = [pp, ip, ip, dp, dp, dp]
        L.orc_energy.argtypes = [pp, ip, ip, dp, dp, C.c_double, dp, dp, dp]
        L.orc_invert3x3.argtypes = [dp, dp]
        L.orc_block_jacobi.argtypes = [pp, ip, ip, dp, dp]
        L.orc_dembx.argtypes = [pp, ip, ip, dp, dp, dp, dp, C.c_int32, C.c_double, C.c_int32,
                                ip, dp, dp, ip]
        L.orc_dembx.restype = C.c_int32
        L.orc_pcg_begin.argtypes = [pp, ip, ip, dp, dp, dp, dp, C.c_int32, C.c_double, dp]
        L.orc_pcg_begin.restype = C.c_void_p
        L.orc_pcg_iterate.argtypes = [C.c_void_p, C.c_int32]
        L.orc_pcg_iterate.restype = C.c_int32
        L.orc_pcg_end.argtypes = [C.c_void_p, ip, dp, ip]
        L.orc_pcg_end.restype = None
        L.orc_stress.argtypes = [pp, ip, dp, dp, dp, dp]
        L.orc_stress_fullfield.argtypes = [pp, ip, dp, dp, dp, dp]
        L.orc_assig.argtypes = [pp, ip, dp]
        L.orc_run.argtypes = [pp, ip, dp, dp, dp, C.POINTER(OrcResult)]
        L.orc_run.restype = C.c_int32
        L.orc_num_threads.restype = C.c_int32
        L.orc_set_reduction_chunk.argtypes = [C.c_int64]
        L.orc_set_reduction_chunk.restype = None
        _lib = L
    return _lib


def _dp(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a: np.ndarray):
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_int32))


@dataclass
class Problem:
    """Solver constants; defaults follow src/elas3dxtal_pcg.f90:77-148."""
    nx: int
    ny: int
    nz: int
    nphase: int
    flag_m: int = 1
    c11: float = 206.0e9
    c12: float = 133.0e9
    c44: float = 119.0e9
    e1: float = 0.0
    nu1: float = 0.0
    exx: float = 0.0
    eyy: float = 0.0
    ezz: float = 1.0e-3
    exz: float = 0.0
    eyz: float = 0.0
    exy: float = 0.0
    tol: float = 1.0e-8
    ldemb: int = 10000
    criterion: int = 0
    divergence_reset: int = 1
    block_size: int = 8192
    precond: int = 0

    @property
    def ns(self) -> int:
        return self.nx * self.ny * self.nz

    def c_struct(self) -> OrcProblem:
        return OrcProblem(self.nx, self.ny, self.nz, self.nphase, self.flag_m,
                          self.c11, self.c12, self.c44, self.e1, self.nu1,
                          self.exx, self.eyy, self.ezz, self.exz, self.eyz, self.exy,
                          self.tol, self.ldemb, self.criterion, self.divergence_reset,
                          self.block_size, self.precond)


class Oracle:
    """Stateful wrapper mirroring the reference's e3d data type for one problem."""

    def __init__(self, prob: Problem, pix: np.ndarray, rod: np.ndarray):
        self.p = prob
        self.cp = prob.c_struct()
        self.pix = np.ascontiguousarray(pix, dtype=np.int32).reshape(-1)
        assert self.pix.size == prob.ns
        self.rod = np.ascontiguousarray(rod, dtype=np.float64).reshape(-1)
        if self.rod.size == 0:
            self.rod = np.zeros(3, np.float64)
        self.ib = np.empty(27 * prob.ns, np.int32)
        lib().orc_build_ib(prob.nx, prob.ny, prob.nz, _ip(self.ib))
        self.cmod = np.zeros(36 * prob.nphase)
        self.dk = np.zeros(576 * prob.nphase)
        self.b = np.zeros(3 * prob.ns)
        self.C = 0.0

    # femat_OpenMP (src/elas3dxtal_pcg.f90:555-1104)
    def femat(self):
        Cv = C.c_double(0.0)
        lib().orc_femat(C.byref(self.cp), _ip(self.pix), _ip(self.ib), _dp(self.rod),
                        _dp(self.cmod), _dp(self.dk), _dp(self.b), C.byref(Cv))
        self.C = Cv.value
        return self

    def dk_array(self) -> np.ndarray:
        """dk as [p, a, i, b, j] (0-based, reference local node order)."""
        np_ = self.p.nphase
        return self.dk.reshape(3, 8, 3, 8, np_).transpose(4, 3, 2, 1, 0)

    def cmod_array(self) -> np.ndarray:
        """cmod as [p, i, j]."""
        return self.cmod.reshape(6, 6, self.p.nphase).transpose(2, 1, 0)

    def affine_u(self) -> np.ndarray:
        u = np.empty(3 * self.p.ns)
        lib().orc_affine_u(C.byref(self.cp), _dp(u))
        return u

    def apply(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1)
        y = np.empty_like(x)
        lib().orc_apply(C.byref(self.cp), _ip(self.pix), _ip(self.ib), _dp(self.dk), _dp(x), _dp(y))
        return y

    def energy(self, u: np.ndarray):
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(-1)
        g = np.empty_like(u)
        ut = C.c_double(0.0)
        lib().orc_energy(C.byref(self.cp), _ip(self.pix), _ip(self.ib), _dp(self.dk), _dp(self.b),
                         self.C, _dp(u), _dp(g), C.byref(ut))
        return g, ut.value

    def block_jacobi(self) -> np.ndarray:
        minv = np.empty(9 * self.p.ns)
        lib().orc_block_jacobi(C.byref(self.cp), _ip(self.pix), _ip(self.ib), _dp(self.dk), _dp(minv))
        return minv

    def dembx(self, u, g, gg0, max_steps=0):
        u = np.ascontiguousarray(u, dtype=np.float64).copy()
        g = np.ascontiguousarray(g, dtype=np.float64).copy()
        h = np.zeros_like(u)
        hist = np.zeros(max(self.p.ldemb, 1))
        L = C.c_int32(0)
        gg = C.c_double(0.0)
        resets = C.c_int32(0)
        reason = lib().orc_dembx(C.byref(self.cp), _ip(self.pix), _ip(self.ib), _dp(self.dk),
                                 _dp(u), _dp(g), _dp(h), 1, gg0, max_steps, C.byref(L),
                                 C.byref(gg), _dp(hist), C.byref(resets))
        return dict(u=u, g=g, lstep=L.value, gg=gg.value, history=hist[: L.value].copy(),
                    reason=reason, resets=resets.value)

    def pcg(self, u, g, gg0):
        """A PCG solve that runs in steps (see PCG)."""
        return PCG(self, u, g, gg0)

    def stress(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(-1)
        s = np.zeros(6)
        e = np.zeros(6)
        lib().orc_stress(C.byref(self.cp), _ip(self.pix), _dp(self.cmod), _dp(u), _dp(s), _dp(e))
        return s, e

    def stress_fullfield(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(-1)
        sig = np.zeros(6 * self.p.ns)
        vm = np.zeros(self.p.ns)
        lib().orc_stress_fullfield(C.byref(self.cp), _ip(self.pix), _dp(self.cmod), _dp(u),
                                   _dp(sig), _dp(vm))
        return sig, vm

    def assig(self):
        prob = np.zeros(self.p.nphase)
        lib().orc_assig(C.byref(self.cp), _ip(self.pix), _dp(prob))
        return prob


class PCG:
    """dembx_OpenMP (src/elas3dxtal_pcg.f90:1356-2043) in steps: the constructor
    builds the block-Jacobi inverse, z0 = Minv g0 and h = z0; iterate(n) runs n
    more iterations with the search direction carried over; close() frees the
    work arrays.  u and g are copied in and updated in place (``.u``, ``.g``)."""

    def __init__(self, o: "Oracle", u, g, gg0: float):
        self._o = o
        self.u = np.ascontiguousarray(u, dtype=np.float64).copy()
        self.g = np.ascontiguousarray(g, dtype=np.float64).copy()
        self.h = np.zeros_like(self.u)
        self.history = np.zeros(max(o.p.ldemb, 1))
        self._s = lib().orc_pcg_begin(C.byref(o.cp), _ip(o.pix), _ip(o.ib), _dp(o.dk), _dp(self.u),
                                      _dp(self.g), _dp(self.h), 1, float(gg0), _dp(self.history))
        if not self._s:
            raise MemoryError("oracle PCG set-up failed (allocation)")
        self.reason = -1

    def iterate(self, n: int) -> int:
        """Runs up to n iterations; returns the exit reason once the solve has
        ended (0 converged, 1 hAh guard, 2 ldemb), else -1."""
        self.reason = lib().orc_pcg_iterate(self._s, int(n))
        return self.reason

    def close(self) -> dict:
        L = C.c_int32(0)
        gg = C.c_double(0.0)
        resets = C.c_int32(0)
        if self._s:
            lib().orc_pcg_end(self._s, C.byref(L), C.byref(gg), C.byref(resets))
            self._s = None
        return dict(lstep=L.value, gg=gg.value, resets=resets.value, reason=self.reason,
                    history=self.history[: L.value].copy())


def run(prob: Problem, pix: np.ndarray, rod: np.ndarray):
    """program elas3d (src/elas3dxtal_pcg.f90:186-552) without file I/O."""
    pix = np.ascontiguousarray(pix, dtype=np.int32).reshape(-1)
    rod = np.ascontiguousarray(rod, dtype=np.float64).reshape(-1)
    if rod.size == 0:
        rod = np.zeros(3)
    u = np.zeros(3 * prob.ns)
    hist = np.zeros(max(prob.ldemb, 1))
    res = OrcResult()
    cp = prob.c_struct()
    rc = lib().orc_run(C.byref(cp), _ip(pix), _dp(rod), _dp(u), _dp(hist), C.byref(res))
    if rc != 0:
        raise MemoryError("oracle run failed (allocation)")
    out = {f: getattr(res, f) for f, _ in OrcResult._fields_}
    out["strav"] = np.array(res.strav[:])
    out["epsav"] = np.array(res.epsav[:])
    out["u"] = u
    out["history"] = hist[: res.lstep].copy()
    return out


def rotate_stiffness(rod: np.ndarray, c11: float, c12: float, c44: float) -> np.ndarray:
    rod = np.ascontiguousarray(rod, dtype=np.float64).reshape(-1)
    n = rod.size // 3
    out = np.zeros(36 * max(n, 1))
    lib().orc_rotate_stiffness(n, _dp(rod), c11, c12, c44, _dp(out))
    return out[: 36 * n].reshape(n, 6, 6)


def invert3x3(a: np.ndarray) -> np.ndarray:
    """a given as a numpy 3x3 matrix (row i, col j)."""
    col = np.asfortranarray(a, dtype=np.float64).ravel(order="F").copy()
    out = np.zeros(9)
    lib().orc_invert3x3(_dp(col), _dp(out))
    return out.reshape(3, 3, order="F")


def num_threads() -> int:
    return int(lib().orc_num_threads())


def set_reduction_chunk(n: int) -> None:
    """Chunk length of the oracle's dot products (0 restores the default 4096)."""
    lib().orc_set_reduction_chunk(int(n))
