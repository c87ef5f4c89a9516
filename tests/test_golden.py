"""Committed golden fixtures (tests/golden/make_golden.py): the oracle must
still reproduce them (CPU) and the CUDA path must match them (GPU)."""
import glob
import os

import numpy as np
import pytest

import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))


def _load(path):
    d = dict(np.load(path))
    nx, ny, nz, nphase = (int(v) for v in d["shape"])
    s = d["strain"]
    c = d["material"]
    p = O.Problem(nx, ny, nz, nphase, c11=c[0], c12=c[1], c44=c[2], exx=s[0], eyy=s[1], ezz=s[2],
                  exz=s[3], eyz=s[4], exy=s[5])
    return p, d


def _rel(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / max(np.linalg.norm(np.ravel(b)), 1e-300))


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(f) for f in FIXTURES])
def test_oracle_reproduces_golden(path):
    p, d = _load(path)
    o = O.Oracle(p, d["pix"], d["rod"]).femat()
    assert _rel(o.cmod_array(), d["cmod"]) < 1e-14
    assert _rel(o.dk_array(), d["dk"]) < 1e-14
    assert _rel(o.b, d["b"]) < 1e-13
    assert abs(o.C - float(d["C"])) <= 1e-12 * abs(float(d["C"]))
    assert _rel(o.apply(d["x"]), d["Kx"]) < 1e-13
    assert _rel(o.block_jacobi(), d["minv"]) < 1e-13
    r = O.run(p, d["pix"], d["rod"])
    assert r["lstep"] == int(d["lstep"])
    assert abs(r["utot"] - float(d["utot"])) <= 1e-12 * abs(float(d["utot"]))
    assert _rel(r["strav"], d["strav"]) < 1e-11


@pytest.mark.gpu
@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(f) for f in FIXTURES])
def test_gpu_matches_golden(path):
    import elas3d_xtal_gb300 as e3d

    p, d = _load(path)
    s = d["strain"]
    c = d["material"]
    gp = e3d.Problem(p.nx, p.ny, p.nz, p.nphase, c11=c[0], c12=c[1], c44=c[2], strain=tuple(s))
    with e3d.Elas3D(gp) as g:
        g.upload(d["pix"], d["rod"]).femat()
        assert _rel(g.get_dk(), d["dk"]) < 1e-12
        assert _rel(g.get_b(), d["b"]) < 1e-12
        assert _rel(g.apply(d["x"]), d["Kx"]) < 1e-12
        res = g.run()
        assert abs(res["iterations"] - int(d["lstep"])) <= 2
        assert abs(res["utot0"] - float(d["utot0"])) <= 1e-9 * abs(float(d["utot0"]))
        assert abs(res["utot"] - float(d["utot"])) <= 1e-9 * abs(float(d["utot"]))
        assert _rel(res["strav"], d["strav"]) < 1e-9
        assert _rel(res["epsav"], d["epsav"]) < 1e-9
