"""Synthetic microstructure generator (include/e3d_micro.h), CPU only.

The seeds and orientations are recomputed here with a Python replica of the
generator's RNG (xoshiro256** seeded through splitmix64), so the Voronoi
assignment is checked against brute force."""
import os

import numpy as np
import pytest

import elas3d_xtal_gb300 as e3d

M64 = (1 << 64) - 1


class PyRng:
    def __init__(self, seed):
        x = seed & M64
        self.s = []
        for _ in range(4):
            x = (x + 0x9E3779B97F4A7C15) & M64
            z = x
            z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
            z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
            self.s.append(z ^ (z >> 31))

    @staticmethod
    def rotl(v, k):
        return ((v << k) | (v >> (64 - k))) & M64

    def next(self):
        s = self.s
        r = (self.rotl((s[1] * 5) & M64, 7) * 9) & M64
        t = (s[1] << 17) & M64
        s[2] ^= s[0]
        s[3] ^= s[1]
        s[1] ^= s[2]
        s[0] ^= s[3]
        s[2] ^= t
        s[3] = self.rotl(s[3], 45)
        return r

    def uniform(self):
        return (self.next() >> 11) * (1.0 / 9007199254740992.0)


def _seeds(n, ng, seed):
    r = PyRng(seed)
    pts = np.array([[r.uniform() * n, r.uniform() * n, r.uniform() * n] for _ in range(ng)])
    return pts


def _lib_ok():
    try:
        e3d.load_library()
        return True
    except Exception:
        return False


pytestmark = pytest.mark.skipif(not _lib_ok(), reason="library not built")


@pytest.mark.parametrize("n,ng,seed", [(12, 5, 1), (20, 30, 7), (16, 200, 3)])
def test_voronoi_is_nearest_seed(n, ng, seed):
    pix, rod = e3d.micro_grains(n, n, n, ng, seed)
    assert pix.min() >= 1 and pix.max() <= ng
    pts = _seeds(n, ng, seed)
    m = np.arange(n ** 3)
    c = np.stack([m % n, (m // n) % n, m // (n * n)], axis=1) + 0.5
    d = c[:, None, :] - pts[None, :, :]
    d -= n * np.round(d / n)
    d2 = (d ** 2).sum(-1)
    best = d2.min(1)
    chosen = d2[m, pix - 1]
    assert np.all(chosen <= best + 1e-9)


def test_orientations_are_unit_quaternions_with_positive_w():
    pix, rod = e3d.micro_grains(8, 8, 8, 400, 11)
    r = rod.reshape(-1, 3)
    qw = 1.0 / np.sqrt(1.0 + (r ** 2).sum(1))
    q = np.concatenate([qw[:, None], r * qw[:, None]], axis=1)
    assert np.allclose((q ** 2).sum(1), 1.0)
    # uniform on SO(3): <q_w^2> = 1/4 ... with q_w >= 0, E|q_w| = 0.5*... check loose moments
    assert abs(np.mean(q[:, 1:] ** 2) - 0.25) < 0.03


def test_deterministic_and_seed_dependent():
    a = e3d.micro_grains(10, 11, 12, 9, 5)
    b = e3d.micro_grains(10, 11, 12, 9, 5)
    c = e3d.micro_grains(10, 11, 12, 9, 6)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert not np.array_equal(a[0], c[0])


@pytest.mark.parametrize("kind", ["sphere", "ellipsoid"])
def test_pores_reach_target_fraction(kind):
    n, ng = 40, 20
    pix, rod = e3d.micro_grains(n, n, n, ng, 9)
    if kind == "sphere":
        e3d.micro_spherical_pores(pix, n, n, n, 0.02, ng + 1, 4)
    else:
        e3d.micro_ellipsoidal_pores(pix, n, n, n, 0.03, ng + 1, 4)
    frac = (pix == ng + 1).mean()
    target = 0.02 if kind == "sphere" else 0.03
    assert target <= frac < target + 0.02


def test_laguerre_has_all_ids_in_range():
    pix, rod = e3d.micro_grains(24, 24, 24, 40, 3, laguerre_sigma=0.5)
    assert pix.min() >= 1 and pix.max() <= 40
    assert np.unique(pix).size > 30


def test_euler_to_rodrigues_matches_rotation():
    import np_ref as R

    rng = np.random.default_rng(0)
    eul = rng.uniform(0, 1, size=(10, 3)) * np.array([2 * np.pi, np.pi, 2 * np.pi])
    rod = e3d.euler_to_rodrigues(eul).reshape(-1, 3)

    def rz(a):
        return np.array([[np.cos(a), -np.sin(a), 0], [np.sin(a), np.cos(a), 0], [0, 0, 1]])

    def rx(a):
        return np.array([[1, 0, 0], [0, np.cos(a), -np.sin(a)], [0, np.sin(a), np.cos(a)]])

    for (p1, P, p2), r in zip(eul, rod):
        assert np.allclose(R.rodrigues_to_Q(r), rz(p1) @ rx(P) @ rz(p2), atol=1e-12)


def test_e3d_container_roundtrip_and_checks(tmp_path):
    pix, rod = e3d.micro_grains(9, 8, 7, 5, 2)
    path = str(tmp_path / "m.e3d")
    e3d.micro_write(path, pix, rod, (9, 8, 7))
    p2, r2, shape = e3d.micro_read(path)
    assert shape == (9, 8, 7) and np.array_equal(p2, pix) and np.array_equal(r2, rod)
    bad = pix.copy()
    bad[3] = 7  # ngrains + 2: outside [1, ngrains + 1]
    e3d.micro_write(path, bad, rod, (9, 8, 7))
    with pytest.raises(ValueError):
        e3d.micro_read(path)
    with open(path, "r+b") as f:  # corrupt the magic
        f.write(b"XXXX")
    with pytest.raises(OSError):
        e3d.micro_read(path)


def test_driver_help_runs_without_gpu():
    import subprocess

    drv = os.path.join(os.path.dirname(e3d.LIB_PATH), "e3d_run")
    out = subprocess.run([drv, "--help"], capture_output=True, text=True)
    assert out.returncode == 0 and "--generate" in out.stdout


def test_oracle_side_workload_equals_package_workload():
    """The CPU arms of the bench build their input with the generator compiled
    on its own (oracle/workload.py, no CUDA library); it must be bit for bit the
    input the package builds."""
    import oracle as O
    import workload as OW
    from elas3d_xtal_gb300 import workloads as W

    for n in (24, 41):
        p, pix, rod = W.c2(n=n)
        op, opix, orod = OW.c2(n=n)
        assert np.array_equal(pix, opix) and np.array_equal(rod, orod)
        assert (op.nx, op.ny, op.nz, op.nphase) == (p.nx, p.ny, p.nz, p.nphase)
        assert (op.c11, op.c12, op.c44, op.flag_m) == (p.c11, p.c12, p.c44, p.flag_m)
        assert (op.exx, op.eyy, op.ezz, op.exz, op.eyz, op.exy) == tuple(p.strain)
        assert np.float32(op.tol) == np.float32(p.tol)
        assert isinstance(op, O.Problem)
