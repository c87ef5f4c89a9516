"""GB300 (sm_103a) voxel-FE elasticity solver -- host API.

A drop-in for the hot path of ELAS3D-Xtal (src/elas3dxtal_pcg.f90): the
matrix-free voxel finite-element PCG solve.  The compute runs in the CUDA
library ``_build/libe3d_gpu.so`` behind the C ABI of ``include/e3d_gpu.h``;
this module binds it with ctypes and mirrors the reference's subroutines on
its shared data type ``e3d``:

    reference (src/elas3dxtal_pcg.f90)      here (class Elas3D)
    ppixel_hdf5            :2879            upload(pix, rodrigues)
    femat_OpenMP           :555             femat()
    affine guess (driver)  :423             init_affine()
    energy_OpenMP          :1107            energy() -> (utot, gg)
    dembx_OpenMP           :1356            dembx() -> stats
    stress_OpenMP          :2149            stress() -> (strav, epsav)
    stress_fullfield_OpenMP:2639            stress_fullfield() -> (sigma, vm)
    assig                  :2410            assig(pix, nphase)
    program elas3d         :186             run()

There is no CPU fallback: if the library or a CUDA device is missing the
calls raise.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
# E3D_LIBRARY selects another build of the same library, e.g. the
# bounds-checked debug variant BOUNDS_LIB_PATH (build.py --bounds).
LIB_PATH = os.environ.get("E3D_LIBRARY") or os.path.join(_PKG, "_build", "libe3d_gpu.so")
BOUNDS_LIB_PATH = os.path.join(_PKG, "_build", "bounds", "libe3d_gpu_bounds.so")

E3D_OK = 0
E3D_ERR_INPUT = 1
E3D_ERR_OOM = 2
E3D_ERR_BREAKDOWN = 3
E3D_ERR_MAXITER = 4
E3D_ERR_TIMEOUT = 5
E3D_ERR_CUDA = 6
E3D_ERR_STATE = 7

EXIT_CONVERGED, EXIT_HAH_GUARD, EXIT_MAXITER, EXIT_BREAKDOWN, EXIT_TIMEOUT, EXIT_RUNNING, EXIT_CANCELLED = range(7)
CRIT_REF, CRIT_PRECOND_REL = 0, 1
PRECOND_BLOCK_JACOBI, PRECOND_NONE = 0, 1
PREC_FP64, PREC_MIXED = 0, 1

# Every symbol include/e3d_gpu.h and include/e3d_micro.h declare.
EXPORTED_SYMBOLS = (
    "e3d_problem_defaults", "e3d_create", "e3d_destroy", "e3d_upload", "e3d_upload_device", "e3d_femat",
    "e3d_init_affine", "e3d_energy", "e3d_solve", "e3d_solve_begin", "e3d_iterate",
    "e3d_stress", "e3d_stress_field", "e3d_run", "e3d_apply", "e3d_apply_device",
    "e3d_set_u", "e3d_get_u", "e3d_get_g", "e3d_get_b", "e3d_get_C", "e3d_get_cmod",
    "e3d_get_dk", "e3d_get_minv", "e3d_get_history", "e3d_device_ptrs",
    "e3d_device_bytes", "e3d_launch_count", "e3d_stencil_path", "e3d_probe_peaks", "e3d_selftest_timeout",
    "e3d_debug_bounds", "e3d_selftest_bounds", "e3d_strerror", "e3d_last_cuda_error",
    "e3d_apply_noalloc", "e3d_checkpoint_save", "e3d_checkpoint_load",
    "e3d_micro_write", "e3d_micro_read_header", "e3d_micro_read",
    "e3d_h5_micro_info", "e3d_h5_micro_read", "e3d_h5_micro_write", "e3d_h5_fullfield_write",
    "e3d_h5_dataset_size", "e3d_h5_read_i32", "e3d_h5_read_f64",
    "e3d_micro_grains", "e3d_micro_spherical_pores", "e3d_micro_ellipsoidal_pores",
    "e3d_micro_grains_device", "e3d_micro_spherical_pores_device", "e3d_micro_ellipsoidal_pores_device",
    "e3d_euler_to_rodrigues",
)


class E3DError(RuntimeError):
    def __init__(self, code: int, what: str):
        self.code = code
        msg = f"{what}: {strerror(code)} (E3D status {code})"
        if code == E3D_ERR_CUDA:
            msg += f" [{last_cuda_error()}]"
        super().__init__(msg)


class ProblemC(C.Structure):
    _fields_ = [
        ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("nphase", C.c_int32),
        ("flag_m", C.c_int32), ("criterion", C.c_int32), ("precision", C.c_int32),
        ("divergence_reset", C.c_int32), ("max_iter", C.c_int32), ("device", C.c_int32),
        ("tol", C.c_float), ("refine_every", C.c_int32),
        ("preconditioner", C.c_int32), ("refine_decades", C.c_int32),
        ("c11", C.c_double), ("c12", C.c_double), ("c44", C.c_double),
        ("e1", C.c_double), ("nu1", C.c_double), ("strain", C.c_double * 6),
        ("hbm_budget", C.c_int64),
    ]


class SolveStatsC(C.Structure):
    _fields_ = [
        ("iterations", C.c_int32), ("exit_reason", C.c_int32), ("resets", C.c_int32),
        ("refinements", C.c_int32), ("gg", C.c_double), ("gg0", C.c_double),
        ("rel_res", C.c_double), ("true_rel", C.c_double), ("ms_setup", C.c_double),
        ("ms_iter", C.c_double),
    ]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


_lib = None


def load_library(path: str | None = None) -> C.CDLL:
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"{p} is missing: build it with elas3d-xtal_gb300/build.py "
                           "(there is no CPU fallback)")
    L = C.CDLL(p)
    vp, dp, ip = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int32)
    L.e3d_problem_defaults.argtypes = [C.POINTER(ProblemC), C.c_int32, C.c_int32, C.c_int32, C.c_int32]
    L.e3d_problem_defaults.restype = None
    L.e3d_create.argtypes = [C.POINTER(vp), C.POINTER(ProblemC)]
    for name in ("e3d_destroy", "e3d_femat", "e3d_init_affine", "e3d_solve_begin"):
        getattr(L, name).argtypes = [vp]
    L.e3d_upload.argtypes = [vp, ip, dp]
    L.e3d_energy.argtypes = [vp, dp, dp]
    L.e3d_solve.argtypes = [vp, C.POINTER(SolveStatsC)]
    L.e3d_iterate.argtypes = [vp, C.c_int32, C.POINTER(SolveStatsC)]
    L.e3d_stress.argtypes = [vp, dp, dp]
    L.e3d_stress_field.argtypes = [vp, dp, dp]
    L.e3d_run.argtypes = [vp, dp, dp, C.POINTER(SolveStatsC)]
    L.e3d_apply.argtypes = [vp, dp, dp]
    L.e3d_apply_device.argtypes = [vp, vp, vp]
    for name in ("e3d_set_u", "e3d_get_u", "e3d_get_g", "e3d_get_b", "e3d_get_C",
                 "e3d_get_cmod", "e3d_get_dk", "e3d_get_minv"):
        getattr(L, name).argtypes = [vp, dp]
    L.e3d_get_history.argtypes = [vp, dp, C.c_int32, ip]
    L.e3d_device_ptrs.argtypes = [vp, C.POINTER(vp), C.POINTER(vp), C.POINTER(vp)]
    L.e3d_device_bytes.argtypes = [vp]
    L.e3d_device_bytes.restype = C.c_int64
    L.e3d_launch_count.argtypes = [vp]
    L.e3d_launch_count.restype = C.c_int64
    L.e3d_stencil_path.argtypes = [vp]
    L.e3d_stencil_path.restype = C.c_int32
    L.e3d_probe_peaks.argtypes = [C.c_int32, dp, dp]
    L.e3d_apply_noalloc.argtypes = [C.c_int32, C.c_int32, C.c_int32, C.c_int32, vp, vp, vp, vp, vp]
    L.e3d_checkpoint_save.argtypes = [vp, C.c_char_p]
    L.e3d_checkpoint_load.argtypes = [vp, C.c_char_p]
    L.e3d_micro_write.argtypes = [C.c_char_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32, ip, dp]
    i64p = C.POINTER(C.c_int64)
    L.e3d_h5_micro_info.argtypes = [C.c_char_p, i64p, i64p, ip]
    L.e3d_h5_micro_read.argtypes = [C.c_char_p, C.c_int64, C.c_int32, ip, dp]
    L.e3d_h5_micro_write.argtypes = [C.c_char_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32, ip, dp]
    L.e3d_h5_fullfield_write.argtypes = [C.c_char_p, C.c_int64, ip, dp, dp]
    L.e3d_h5_dataset_size.argtypes = [C.c_char_p, C.c_char_p, i64p, ip, i64p]
    L.e3d_h5_read_i32.argtypes = [C.c_char_p, C.c_char_p, C.c_int64, ip]
    L.e3d_h5_read_f64.argtypes = [C.c_char_p, C.c_char_p, C.c_int64, dp]
    for fn in (L.e3d_h5_micro_info, L.e3d_h5_micro_read, L.e3d_h5_micro_write, L.e3d_h5_fullfield_write,
               L.e3d_h5_dataset_size, L.e3d_h5_read_i32, L.e3d_h5_read_f64):
        fn.restype = C.c_int32
    L.e3d_micro_read_header.argtypes = [C.c_char_p, ip, ip, ip, ip]
    L.e3d_micro_read.argtypes = [C.c_char_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32, ip, dp]
    L.e3d_strerror.argtypes = [C.c_int32]
    L.e3d_strerror.restype = C.c_char_p
    L.e3d_last_cuda_error.argtypes = []
    L.e3d_last_cuda_error.restype = C.c_char_p
    L.e3d_micro_grains.argtypes = [C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_double, C.c_uint64,
                                   ip, dp]
    L.e3d_micro_spherical_pores.argtypes = [C.c_int32, C.c_int32, C.c_int32, C.c_double, C.c_double,
                                            C.c_double, C.c_int32, C.c_uint64, ip]
    L.e3d_micro_ellipsoidal_pores.argtypes = [C.c_int32, C.c_int32, C.c_int32, C.c_double, C.c_double,
                                              C.c_double, C.c_double, C.c_int32, C.c_uint64, ip]
    L.e3d_micro_grains_device.argtypes = [C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_double, C.c_uint64,
                                          C.c_int32, vp, dp]
    L.e3d_micro_spherical_pores_device.argtypes = [C.c_int32, C.c_int32, C.c_int32, C.c_double, C.c_double,
                                                   C.c_double, C.c_int32, C.c_uint64, C.c_int32, vp]
    L.e3d_micro_ellipsoidal_pores_device.argtypes = [C.c_int32, C.c_int32, C.c_int32, C.c_double, C.c_double,
                                                     C.c_double, C.c_double, C.c_int32, C.c_uint64, C.c_int32, vp]
    L.e3d_upload_device.argtypes = [vp, vp, dp]
    L.e3d_selftest_timeout.argtypes = [C.c_int32, C.c_int32, C.c_double]
    L.e3d_debug_bounds.argtypes = [C.POINTER(C.c_int64)]
    L.e3d_selftest_bounds.argtypes = [C.c_int32]
    L.e3d_euler_to_rodrigues.argtypes = [C.c_int32, dp, dp]
    L.e3d_euler_to_rodrigues.restype = None
    for name in EXPORTED_SYMBOLS:
        fn = getattr(L, name)
        if fn.restype is C.c_int and name not in ("e3d_problem_defaults", "e3d_euler_to_rodrigues"):
            fn.restype = C.c_int32
    if path is None:
        _lib = L
    return L


def strerror(code: int) -> str:
    try:
        return load_library().e3d_strerror(code).decode()
    except Exception:  # library missing: still produce a message
        return f"status {code}"


def last_cuda_error() -> str:
    try:
        return load_library().e3d_last_cuda_error().decode()
    except Exception:
        return ""


def _check(rc: int, what: str, allow=()):
    if rc != E3D_OK and rc not in allow:
        raise E3DError(rc, what)
    return rc


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


@dataclass
class Problem:
    """Runtime form of the reference's compile-time constants
    (src/elas3dxtal_pcg.f90:77-148).  Strains are tensor components."""
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
    strain: tuple = (0.0, 0.0, 1.0e-3, 0.0, 0.0, 0.0)  # exx eyy ezz exz eyz exy
    tol: float = 1.0e-8
    max_iter: int = 10000
    criterion: int = CRIT_REF
    precision: int = PREC_FP64
    divergence_reset: int = 1
    refine_every: int = 0
    preconditioner: int = PRECOND_BLOCK_JACOBI
    refine_decades: int = 0  # MIXED: also replace after this many decades of FP32 residual drop
    device: int = 0
    hbm_budget: int = 0

    @property
    def ns(self) -> int:
        return self.nx * self.ny * self.nz

    def to_c(self) -> ProblemC:
        p = ProblemC()
        p.nx, p.ny, p.nz, p.nphase = self.nx, self.ny, self.nz, self.nphase
        p.flag_m, p.criterion, p.precision = self.flag_m, self.criterion, self.precision
        p.divergence_reset, p.max_iter, p.device = self.divergence_reset, self.max_iter, self.device
        p.tol, p.refine_every = self.tol, self.refine_every
        p.preconditioner, p.refine_decades = self.preconditioner, self.refine_decades
        p.c11, p.c12, p.c44, p.e1, p.nu1 = self.c11, self.c12, self.c44, self.e1, self.nu1
        for i in range(6):
            p.strain[i] = float(self.strain[i])
        p.hbm_budget = int(self.hbm_budget)
        return p


class Elas3D:
    """One problem on one GPU (the reference's ``type(elas3d_data_type) :: e3d``)."""

    def __init__(self, problem: Problem):
        self.p = problem
        self.L = load_library()
        self._h = C.c_void_p()
        pc = problem.to_c()
        _check(self.L.e3d_create(C.byref(self._h), C.byref(pc)), "e3d_create")

    # -- lifecycle
    def close(self):
        if self._h:
            self.L.e3d_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    # -- inputs (ppixel_hdf5)
    def upload_device(self, d_pix, rodrigues: np.ndarray | None):
        """e3d_upload_device: the phase map is already on the device (see micro_grains_device)."""
        rod = None
        if rodrigues is not None and self.p.nphase > 1:
            rod = np.ascontiguousarray(rodrigues, dtype=np.float64).reshape(-1)
        _check(self.L.e3d_upload_device(self._h, _addr(d_pix), _dp(rod) if rod is not None else None),
               "e3d_upload_device")
        return self

    def upload(self, pix: np.ndarray, rodrigues: np.ndarray | None):
        pix = np.ascontiguousarray(pix, dtype=np.int32).reshape(-1)
        if pix.size != self.p.ns:
            raise ValueError(f"pix has {pix.size} entries, expected ns = {self.p.ns}")
        rod = None
        if rodrigues is not None and self.p.nphase > 1:
            rod = np.ascontiguousarray(rodrigues, dtype=np.float64).reshape(-1)
            if self.p.flag_m == 1 and rod.size != 3 * (self.p.nphase - 1):
                raise ValueError(f"orientation has {rod.size} entries, expected {3 * (self.p.nphase - 1)}")
        _check(self.L.e3d_upload(self._h, _ip(pix), _dp(rod) if rod is not None else None), "e3d_upload")
        return self

    # -- reference subroutines
    def femat(self):
        _check(self.L.e3d_femat(self._h), "e3d_femat")
        return self

    def init_affine(self):
        _check(self.L.e3d_init_affine(self._h), "e3d_init_affine")
        return self

    def energy(self):
        ut = C.c_double()
        gg = C.c_double()
        _check(self.L.e3d_energy(self._h, C.byref(ut), C.byref(gg)), "e3d_energy")
        return ut.value, gg.value

    def dembx(self) -> dict:
        st = SolveStatsC()
        rc = self.L.e3d_solve(self._h, C.byref(st))
        _check(rc, "e3d_solve", allow=(E3D_ERR_MAXITER,))
        d = st.as_dict()
        d["status"] = rc
        return d

    solve = dembx

    def solve_begin(self):
        _check(self.L.e3d_solve_begin(self._h), "e3d_solve_begin")

    def iterate(self, n: int) -> dict:
        st = SolveStatsC()
        _check(self.L.e3d_iterate(self._h, int(n), C.byref(st)), "e3d_iterate")
        return st.as_dict()

    def stress(self):
        s = np.zeros(6)
        e = np.zeros(6)
        _check(self.L.e3d_stress(self._h, _dp(s), _dp(e)), "e3d_stress")
        return s, e

    def stress_fullfield(self):
        sig = np.zeros(6 * self.p.ns)
        vm = np.zeros(self.p.ns)
        _check(self.L.e3d_stress_field(self._h, _dp(sig), _dp(vm)), "e3d_stress_field")
        return sig, vm

    def run(self) -> dict:
        ut = np.zeros(2)
        out = np.zeros(12)
        st = SolveStatsC()
        rc = self.L.e3d_run(self._h, _dp(ut), _dp(out), C.byref(st))
        _check(rc, "e3d_run", allow=(E3D_ERR_MAXITER,))
        d = st.as_dict()
        d.update(status=rc, utot0=ut[0], utot=ut[1], strav=out[:6].copy(), epsav=out[6:].copy())
        return d

    # -- test hooks and state transfer
    def apply(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1)
        if x.size != 3 * self.p.ns:
            raise ValueError("x must have 3*ns entries")
        y = np.empty_like(x)
        _check(self.L.e3d_apply(self._h, _dp(x), _dp(y)), "e3d_apply")
        return y

    def _get(self, fn, n):
        out = np.empty(n)
        _check(fn(self._h, _dp(out)), fn.__name__)
        return out

    def set_u(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(-1)
        _check(self.L.e3d_set_u(self._h, _dp(u)), "e3d_set_u")

    def get_u(self):
        return self._get(self.L.e3d_get_u, 3 * self.p.ns)

    def get_g(self):
        return self._get(self.L.e3d_get_g, 3 * self.p.ns)

    def get_b(self):
        return self._get(self.L.e3d_get_b, 3 * self.p.ns)

    def get_C(self) -> float:
        v = C.c_double()
        _check(self.L.e3d_get_C(self._h, C.byref(v)), "e3d_get_C")
        return v.value

    def get_cmod(self):
        """cmod as [p, i, j]."""
        raw = self._get(self.L.e3d_get_cmod, 36 * self.p.nphase)
        return raw.reshape(6, 6, self.p.nphase).transpose(2, 1, 0)

    def get_dk(self):
        """dk as [p, a, i, b, j] (reference local node order, 0-based)."""
        raw = self._get(self.L.e3d_get_dk, 576 * self.p.nphase)
        return raw.reshape(3, 8, 3, 8, self.p.nphase).transpose(4, 3, 2, 1, 0)

    def get_minv(self):
        """M_block_inv(ns,3,3) as [m, i, j]."""
        raw = self._get(self.L.e3d_get_minv, 9 * self.p.ns)
        return raw.reshape(3, 3, self.p.ns).transpose(2, 1, 0)

    def history(self) -> np.ndarray:
        n = max(self.p.max_iter, 1)
        out = np.zeros(n)
        cnt = C.c_int32()
        _check(self.L.e3d_get_history(self._h, _dp(out), n, C.byref(cnt)), "e3d_get_history")
        return out[: cnt.value].copy()

    def checkpoint_save(self, path: str):
        _check(self.L.e3d_checkpoint_save(self._h, os.fsencode(path)), "e3d_checkpoint_save")

    def checkpoint_load(self, path: str):
        _check(self.L.e3d_checkpoint_load(self._h, os.fsencode(path)), "e3d_checkpoint_load")

    def device_bytes(self) -> int:
        return int(self.L.e3d_device_bytes(self._h))

    def launch_count(self) -> int:
        return int(self.L.e3d_launch_count(self._h))

    def stencil_path(self) -> str:
        """'fp64', 'f32' (per-thread loads) or 'f32_tma' (TMA plane ring)."""
        return ("fp64", "f32", "f32_tma")[int(self.L.e3d_stencil_path(self._h))]


def assig(pix: np.ndarray, nphase: int) -> np.ndarray:
    """Phase volume fractions (assig, src/elas3dxtal_pcg.f90:2410-2468)."""
    pix = np.asarray(pix).reshape(-1)
    ok = (pix >= 1) & (pix <= nphase)
    return np.bincount(pix[ok] - 1, minlength=nphase)[:nphase] / float(pix.size)


# ---------------------------------------------------------------------------
# Synthetic microstructures (include/e3d_micro.h)
def micro_grains(nx, ny, nz, ngrains, seed, laguerre_sigma=0.0):
    L = load_library()
    pix = np.empty(nx * ny * nz, np.int32)
    rod = np.empty(3 * ngrains)
    rc = L.e3d_micro_grains(nx, ny, nz, ngrains, float(laguerre_sigma), int(seed) & (2**64 - 1),
                            _ip(pix), _dp(rod))
    if rc != 0:
        raise RuntimeError(f"e3d_micro_grains failed ({rc})")
    return pix, rod


def micro_spherical_pores(pix, nx, ny, nz, frac, pore_phase, seed, log_mu=np.log(3.0), log_sigma=0.4):
    L = load_library()
    assert pix.dtype == np.int32 and pix.flags.c_contiguous
    rc = L.e3d_micro_spherical_pores(nx, ny, nz, float(frac), float(log_mu), float(log_sigma),
                                     int(pore_phase), int(seed) & (2**64 - 1), _ip(pix))
    if rc < 0:
        raise RuntimeError(f"e3d_micro_spherical_pores failed ({rc})")
    return rc


def micro_ellipsoidal_pores(pix, nx, ny, nz, frac, pore_phase, seed, aspect=4.0,
                            log_mu=np.log(2.0), log_sigma=0.3):
    L = load_library()
    assert pix.dtype == np.int32 and pix.flags.c_contiguous
    rc = L.e3d_micro_ellipsoidal_pores(nx, ny, nz, float(frac), float(aspect), float(log_mu),
                                       float(log_sigma), int(pore_phase), int(seed) & (2**64 - 1),
                                       _ip(pix))
    if rc < 0:
        raise RuntimeError(f"e3d_micro_ellipsoidal_pores failed ({rc})")
    return rc


# GPU versions (same microstructures, bit for bit, in device memory).  d_pix is
# a device address of nx*ny*nz int32 (an int, or any object with data_ptr(),
# e.g. a CUDA tensor).
def _addr(buf):
    return C.c_void_p(buf.data_ptr() if hasattr(buf, "data_ptr") else int(buf))


def micro_grains_device(d_pix, nx, ny, nz, ngrains, seed, laguerre_sigma=0.0, device=0):
    L = load_library()
    rod = np.empty(3 * ngrains)
    rc = L.e3d_micro_grains_device(nx, ny, nz, ngrains, float(laguerre_sigma), int(seed) & (2**64 - 1),
                                   int(device), _addr(d_pix), _dp(rod))
    if rc != 0:
        raise RuntimeError(f"e3d_micro_grains_device failed ({rc}): {L.e3d_last_cuda_error().decode()}")
    return rod


def micro_spherical_pores_device(d_pix, nx, ny, nz, frac, pore_phase, seed, log_mu=np.log(3.0), log_sigma=0.4,
                                 device=0):
    L = load_library()
    rc = L.e3d_micro_spherical_pores_device(nx, ny, nz, float(frac), float(log_mu), float(log_sigma),
                                            int(pore_phase), int(seed) & (2**64 - 1), int(device), _addr(d_pix))
    if rc < 0:
        raise RuntimeError(f"e3d_micro_spherical_pores_device failed ({rc})")
    return rc


def micro_ellipsoidal_pores_device(d_pix, nx, ny, nz, frac, pore_phase, seed, aspect=4.0, log_mu=np.log(2.0),
                                   log_sigma=0.3, device=0):
    L = load_library()
    rc = L.e3d_micro_ellipsoidal_pores_device(nx, ny, nz, float(frac), float(aspect), float(log_mu),
                                              float(log_sigma), int(pore_phase), int(seed) & (2**64 - 1),
                                              int(device), _addr(d_pix))
    if rc < 0:
        raise RuntimeError(f"e3d_micro_ellipsoidal_pores_device failed ({rc})")
    return rc


def probe_peaks(device: int = 0):
    """Measured (fp64, fp32) FMA throughput in TFLOP/s."""
    a, b = C.c_double(), C.c_double()
    _check(load_library().e3d_probe_peaks(device, C.byref(a), C.byref(b)), "e3d_probe_peaks")
    return a.value, b.value


def debug_bounds() -> dict | None:
    """Record of the bounds-checked debug build (e3d_debug_bounds), cleared on
    read: {"count", "unit", "line", "index", "limit"}; None when the loaded
    library was built without the checks."""
    rep = (C.c_int64 * 5)()
    rc = load_library().e3d_debug_bounds(rep)
    if rc == E3D_ERR_STATE:
        return None
    _check(rc, "e3d_debug_bounds")
    return dict(zip(("count", "unit", "line", "index", "limit"), (int(v) for v in rep)))


def micro_write(path, pix, rod, shape):
    """Writes the .e3d container (pix 1-based, rod 3*ngrains)."""
    pix = np.ascontiguousarray(pix, dtype=np.int32).reshape(-1)
    rod = np.ascontiguousarray(rod, dtype=np.float64).reshape(-1)
    nx, ny, nz = shape
    rc = load_library().e3d_micro_write(os.fsencode(path), nx, ny, nz, rod.size // 3, _ip(pix), _dp(rod))
    if rc != 0:
        raise OSError(f"e3d_micro_write({path}) failed ({rc})")


def micro_read(path):
    """Reads a .e3d container: returns (pix, rod, (nx, ny, nz)); raises on the
    reference's size / phase-range checks."""
    L = load_library()
    d = [C.c_int32() for _ in range(4)]
    rc = L.e3d_micro_read_header(os.fsencode(path), *[C.byref(v) for v in d])
    if rc != 0:
        raise OSError(f"{path}: not a .e3d file ({rc})")
    nx, ny, nz, ng = (v.value for v in d)
    pix = np.empty(nx * ny * nz, np.int32)
    rod = np.empty(3 * ng)
    rc = L.e3d_micro_read(os.fsencode(path), nx, ny, nz, ng, _ip(pix), _dp(rod))
    if rc != 0:
        raise ValueError(f"{path}: size or phase-range check failed ({rc})")
    return pix, rod, (nx, ny, nz)


# HDF5 files (include/e3d_micro.h): the reference's input and full-field output
def h5_micro_info(path):
    """(npix, norient, (Nx, Ny, Nz) from the "dimensions" attribute or zeros)."""
    L = load_library()
    a, b = C.c_int64(), C.c_int64()
    dims = np.zeros(3, np.int32)
    rc = L.e3d_h5_micro_info(os.fsencode(path), C.byref(a), C.byref(b), _ip(dims))
    if rc != 0:
        raise OSError(f"{path}: {last_cuda_error()} ({rc})")
    return a.value, b.value, tuple(int(v) for v in dims)


def h5_micro_read(path, ns, ngrains):
    """ppixel_hdf5: returns (pix, rod); raises on the reference's checks."""
    L = load_library()
    pix = np.empty(int(ns), np.int32)
    rod = np.empty(max(3 * int(ngrains), 1))
    rc = L.e3d_h5_micro_read(os.fsencode(path), int(ns), int(ngrains), _ip(pix), _dp(rod))
    if rc != 0:
        raise (OSError if rc == -1 else ValueError)(f"{path}: {last_cuda_error()} ({rc})")
    return pix, rod[: 3 * int(ngrains)]


def h5_micro_write(path, pix, rod, shape):
    nx, ny, nz = shape
    pix = np.ascontiguousarray(pix, dtype=np.int32).reshape(-1)
    rod = np.ascontiguousarray(rod, dtype=np.float64).reshape(-1)
    if pix.size != nx * ny * nz or rod.size % 3:
        raise ValueError("pix must hold nx*ny*nz values and rod 3 per grain")
    rc = load_library().e3d_h5_micro_write(os.fsencode(path), nx, ny, nz, rod.size // 3, _ip(pix),
                                           _dp(rod) if rod.size else None)
    if rc != 0:
        raise OSError(f"{path}: {last_cuda_error()} ({rc})")


def h5_fullfield_write(path, pix, vm, sigma):
    pix = np.ascontiguousarray(pix, dtype=np.int32).reshape(-1)
    vm = np.ascontiguousarray(vm, dtype=np.float64).reshape(-1)
    sigma = np.ascontiguousarray(sigma, dtype=np.float64).reshape(-1)
    if vm.size != pix.size or sigma.size != 6 * pix.size:
        raise ValueError("vm must hold ns values and sigma 6*ns")
    rc = load_library().e3d_h5_fullfield_write(os.fsencode(path), pix.size, _ip(pix), _dp(vm), _dp(sigma))
    if rc != 0:
        raise OSError(f"{path}: {last_cuda_error()} ({rc})")


def h5_read(path, name):
    """Dataset `name` of an HDF5 file as int32 or float64 (by its class),
    shaped by its dimensions (HDF5 order)."""
    L = load_library()
    n, rank = C.c_int64(), C.c_int32()
    dims = np.zeros(8, np.int64)
    rc = L.e3d_h5_dataset_size(os.fsencode(path), name.encode(), C.byref(n), C.byref(rank),
                               dims.ctypes.data_as(C.POINTER(C.c_int64)))
    if rc != 0:
        raise (OSError if rc == -1 else KeyError)(f"{path}: {last_cuda_error()} ({rc})")
    shape = tuple(int(v) for v in dims[: rank.value])
    out = np.empty(n.value, np.int32)
    if L.e3d_h5_read_i32(os.fsencode(path), name.encode(), n.value, _ip(out)) != 0:
        out = np.empty(n.value, np.float64)
        rc = L.e3d_h5_read_f64(os.fsencode(path), name.encode(), n.value, _dp(out))
        if rc != 0:
            raise ValueError(f"{path}: {last_cuda_error()} ({rc})")
    return out.reshape(shape)


def euler_to_rodrigues(euler: np.ndarray) -> np.ndarray:
    e = np.ascontiguousarray(euler, dtype=np.float64).reshape(-1)
    out = np.empty_like(e)
    load_library().e3d_euler_to_rodrigues(e.size // 3, _dp(e), _dp(out))
    return out


# ---------------------------------------------------------------------------
# Batched ensembles and the serving loop (include/e3d_batch.h)
class RveC(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("ngrains", C.c_int32),
                ("c11", C.c_double), ("c12", C.c_double), ("c44", C.c_double),
                ("pix", C.POINTER(C.c_int32)), ("rodrigues", C.POINTER(C.c_double))]


class BatchOptsC(C.Structure):
    _fields_ = [("device", C.c_int32), ("max_iter", C.c_int32), ("refine_every", C.c_int32),
                ("criterion", C.c_int32), ("divergence_reset", C.c_int32), ("tol", C.c_float),
                ("load_cases", C.c_int32), ("parts", C.c_int32), ("pad", C.c_int32),
                ("strain", C.c_double), ("e1", C.c_double), ("nu1", C.c_double), ("hbm_budget", C.c_int64)]


class JobResultC(C.Structure):
    _fields_ = [("rve", C.c_int32), ("load_case", C.c_int32), ("status", C.c_int32),
                ("iterations", C.c_int32), ("refinements", C.c_int32), ("resets", C.c_int32),
                ("parts", C.c_int32), ("tile_z", C.c_int32), ("utot0", C.c_double), ("utot", C.c_double),
                ("rel_res", C.c_double), ("true_rel", C.c_double), ("strav", C.c_double * 6),
                ("epsav", C.c_double * 6), ("seconds", C.c_double)]

    def as_dict(self) -> dict:
        d = {f: getattr(self, f) for f, _ in self._fields_ if f not in ("strav", "epsav")}
        d["strav"] = np.array(self.strav[:])
        d["epsav"] = np.array(self.epsav[:])
        return d


class ServeOptsC(C.Structure):
    _fields_ = [("device", C.c_int32), ("max_iter", C.c_int32), ("refine_every", C.c_int32),
                ("criterion", C.c_int32), ("divergence_reset", C.c_int32), ("tol", C.c_float),
                ("max_active", C.c_int32), ("round_iters", C.c_int32), ("parts", C.c_int32),
                ("round_balance", C.c_int32), ("e1", C.c_double), ("nu1", C.c_double), ("hbm_budget", C.c_int64)]


BATCH_SYMBOLS = ("e3d_batch_opts_defaults", "e3d_batch_create", "e3d_batch_solve", "e3d_batch_results",
                 "e3d_batch_parts", "e3d_batch_destroy", "e3d_serve_opts_defaults", "e3d_serve_create",
                 "e3d_serve_submit", "e3d_serve_step", "e3d_serve_result", "e3d_serve_cancel",
                 "e3d_serve_memory", "e3d_serve_destroy")
EXPORTED_SYMBOLS = EXPORTED_SYMBOLS + BATCH_SYMBOLS


def _bind_batch(L):
    if getattr(L, "_e3d_batch_bound", False):
        return L
    vp, dp, ip = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int32)
    L.e3d_batch_opts_defaults.argtypes = [C.POINTER(BatchOptsC)]
    L.e3d_batch_opts_defaults.restype = None
    L.e3d_batch_create.argtypes = [C.POINTER(vp), C.POINTER(RveC), C.c_int32, C.POINTER(BatchOptsC)]
    L.e3d_batch_solve.argtypes = [vp, dp, dp]
    L.e3d_batch_results.argtypes = [vp, C.POINTER(JobResultC), C.c_int32, ip]
    L.e3d_batch_parts.argtypes = [vp, ip, C.c_int32]
    L.e3d_batch_destroy.argtypes = [vp]
    L.e3d_serve_opts_defaults.argtypes = [C.POINTER(ServeOptsC)]
    L.e3d_serve_opts_defaults.restype = None
    L.e3d_serve_create.argtypes = [C.POINTER(vp), C.POINTER(ServeOptsC)]
    L.e3d_serve_submit.argtypes = [vp, C.POINTER(RveC), dp, C.POINTER(C.c_int64)]
    L.e3d_serve_step.argtypes = [vp, ip]
    L.e3d_serve_result.argtypes = [vp, C.c_int64, C.POINTER(JobResultC)]
    L.e3d_serve_memory.argtypes = [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
    L.e3d_serve_cancel.argtypes = [vp, C.c_int64]
    L.e3d_serve_cancel.restype = C.c_int32
    L.e3d_serve_destroy.argtypes = [vp]
    L._e3d_batch_bound = True
    return L


def _rve_struct(rve: dict, keep: list) -> RveC:
    pix = np.ascontiguousarray(rve["pix"], dtype=np.int32).reshape(-1)
    rod = np.ascontiguousarray(rve["rodrigues"], dtype=np.float64).reshape(-1)
    keep += [pix, rod]
    nx, ny, nz = rve["shape"]
    return RveC(nx, ny, nz, int(rve["ngrains"]), float(rve["c11"]), float(rve["c12"]), float(rve["c44"]),
                _ip(pix), _dp(rod))


class Batch:
    """Many RVEs x the six unit load cases in one persistent launch (CUDA graph).

    rves: list of dicts with keys shape (nx,ny,nz), ngrains, c11, c12, c44,
    pix (1-based phase ids), rodrigues (3*ngrains)."""

    def __init__(self, rves, *, max_iter=10000, refine_every=50, tol=1e-8, criterion=CRIT_REF,
                 load_cases=0, parts=0, strain=1e-3, e1=0.0, nu1=0.0, hbm_budget=0, device=0):
        self.L = _bind_batch(load_library())
        o = BatchOptsC()
        self.L.e3d_batch_opts_defaults(C.byref(o))
        o.device, o.max_iter, o.refine_every, o.tol, o.criterion = device, max_iter, refine_every, tol, criterion
        o.load_cases, o.parts, o.strain, o.e1, o.nu1, o.hbm_budget = load_cases, parts, strain, e1, nu1, hbm_budget
        keep = []
        arr = (RveC * len(rves))(*[_rve_struct(r, keep) for r in rves])
        self.n = len(rves)
        self.ncases = bin(load_cases or 0x3F).count("1")
        self._h = C.c_void_p()
        _check(self.L.e3d_batch_create(C.byref(self._h), arr, len(rves), C.byref(o)), "e3d_batch_create")

    def solve(self):
        ceff = np.zeros(36 * self.n)
        sec = C.c_double()
        rc = self.L.e3d_batch_solve(self._h, _dp(ceff), C.byref(sec))
        _check(rc, "e3d_batch_solve", allow=(E3D_ERR_MAXITER,))
        return ceff.reshape(self.n, 6, 6), sec.value

    def results(self):
        nj = self.n * self.ncases
        out = (JobResultC * nj)()
        cnt = C.c_int32()
        _check(self.L.e3d_batch_results(self._h, out, nj, C.byref(cnt)), "e3d_batch_results")
        return [r.as_dict() for r in out[: cnt.value]]

    def parts(self):
        nj = self.n * self.ncases
        arr = np.zeros(nj, np.int32)
        _check(self.L.e3d_batch_parts(self._h, _ip(arr), nj), "e3d_batch_parts")
        return arr

    def close(self):
        if self._h:
            self.L.e3d_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Continuous-batching solve server (admission by slots and HBM budget)."""

    def __init__(self, *, max_active=64, round_iters=50, max_iter=10000, refine_every=50, tol=1e-8,
                 criterion=CRIT_REF, parts=0, round_balance=False, e1=0.0, nu1=0.0, hbm_budget=0, device=0):
        self.L = _bind_batch(load_library())
        o = ServeOptsC()
        self.L.e3d_serve_opts_defaults(C.byref(o))
        o.device, o.max_active, o.round_iters, o.max_iter = device, max_active, round_iters, max_iter
        o.refine_every, o.tol, o.criterion, o.parts = refine_every, tol, criterion, parts
        o.round_balance = 1 if round_balance else 0
        o.e1, o.nu1, o.hbm_budget = e1, nu1, hbm_budget
        self._h = C.c_void_p()
        _check(self.L.e3d_serve_create(C.byref(self._h), C.byref(o)), "e3d_serve_create")

    def submit(self, rve: dict, strain) -> int:
        keep = []
        r = _rve_struct(rve, keep)
        s = np.ascontiguousarray(strain, dtype=np.float64)
        rid = C.c_int64()
        _check(self.L.e3d_serve_submit(self._h, C.byref(r), _dp(s), C.byref(rid)), "e3d_serve_submit")
        return rid.value

    def step(self) -> int:
        pend = C.c_int32()
        _check(self.L.e3d_serve_step(self._h, C.byref(pend)), "e3d_serve_step")
        return pend.value

    def result(self, rid: int):
        r = JobResultC()
        rc = self.L.e3d_serve_result(self._h, int(rid), C.byref(r))
        if rc == E3D_ERR_STATE:
            return None
        _check(rc, "e3d_serve_result")
        return r.as_dict()

    def cancel(self, rid: int):
        """Withdraw a queued or active request (between steps)."""
        _check(self.L.e3d_serve_cancel(self._h, int(rid)), "e3d_serve_cancel")

    def memory(self):
        a, b = C.c_int64(), C.c_int64()
        _check(self.L.e3d_serve_memory(self._h, C.byref(a), C.byref(b)), "e3d_serve_memory")
        return a.value, b.value

    def close(self):
        if self._h:
            self.L.e3d_serve_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
