"""Checkpoint / resume, the unpreconditioned CG variant and the command-line
driver, on the GPU."""
import os
import subprocess

import numpy as np
import pytest

import elas3d_xtal_gb300 as e3d
import oracle as O
from elas3d_xtal_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _oracle_problem(p):
    s = p.strain
    return O.Problem(p.nx, p.ny, p.nz, p.nphase, flag_m=p.flag_m, c11=p.c11, c12=p.c12, c44=p.c44,
                     e1=p.e1, nu1=p.nu1, exx=s[0], eyy=s[1], ezz=s[2], exz=s[3], eyz=s[4], exy=s[5],
                     tol=p.tol, ldemb=p.max_iter, criterion=p.criterion,
                     divergence_reset=p.divergence_reset, precond=p.preconditioner)


@pytest.mark.parametrize("precision", [e3d.PREC_FP64, e3d.PREC_MIXED])
def test_checkpoint_resume_continues_exactly(tmp_path, precision):
    p, pix, rod = W.c2(n=20, ngrains=10, seed=3)
    p.precision = precision
    p.refine_every = 10
    ref = e3d.Elas3D(p).upload(pix, rod)
    r_ref = ref.run()
    u_ref = ref.get_u()
    a = e3d.Elas3D(p).upload(pix, rod).femat().init_affine()
    a.energy()
    a.solve_begin()
    a.iterate(17)
    path = str(tmp_path / "state.ckpt")
    a.checkpoint_save(path)
    a.close()
    b = e3d.Elas3D(p).upload(pix, rod).femat()
    b.checkpoint_load(path)
    st = b.iterate(p.max_iter)
    assert st["exit_reason"] == e3d.EXIT_CONVERGED
    assert st["iterations"] == r_ref["iterations"]
    u = b.get_u()
    if precision == e3d.PREC_FP64:
        assert np.array_equal(u, u_ref)  # exact continuation
    else:
        assert np.linalg.norm(u - u_ref) <= 1e-6 * np.linalg.norm(u_ref)
    assert len(b.history()) == st["iterations"]


def test_checkpoint_rejects_other_problem(tmp_path):
    p, pix, rod = W.c1(n=12, ngrains=4, seed=1)
    a = e3d.Elas3D(p).upload(pix, rod).femat().init_affine()
    a.energy()
    a.solve_begin()
    a.iterate(3)
    path = str(tmp_path / "s.ckpt")
    a.checkpoint_save(path)
    q, pix2, rod2 = W.c1(n=14, ngrains=4, seed=1)
    b = e3d.Elas3D(q).upload(pix2, rod2).femat()
    with pytest.raises(e3d.E3DError) as ei:
        b.checkpoint_load(path)
    assert ei.value.code == e3d.E3D_ERR_INPUT


def test_unpreconditioned_cg_variant_matches_oracle():
    p, pix, rod = W.c1(n=14, ngrains=6, seed=8)
    p.preconditioner = e3d.PRECOND_NONE
    p.divergence_reset = 0
    with e3d.Elas3D(p) as g:
        g.upload(pix, rod)
        res = g.run()
    ref = O.run(_oracle_problem(p), pix, rod)
    assert res["exit_reason"] == e3d.EXIT_CONVERGED
    assert abs(res["iterations"] - ref["lstep"]) <= 2
    assert abs(res["utot"] - ref["utot"]) <= 1e-9 * abs(ref["utot"])


@pytest.mark.parametrize("fmt", ["h5", "e3d"])
def test_driver_end_to_end(tmp_path, fmt):
    """The driver reads the microstructure as ppixel_hdf5 does (an HDF5 file
    with "pix" and "orientation", or the .e3d container) and writes the
    reference's text outputs and fullfield_poly.h5."""
    drv = os.path.join(os.path.dirname(e3d.LIB_PATH), "e3d_run")
    pix, rod = e3d.micro_grains(14, 14, 14, 6, 4)
    inp = str(tmp_path / f"input_structure_poly.{fmt}")
    if fmt == "h5":
        e3d.h5_micro_write(inp, pix, rod, (14, 14, 14))
    else:
        e3d.micro_write(inp, pix, rod, (14, 14, 14))
    out = subprocess.run([drv, "--input", inp, "--outdir", str(tmp_path), "--fullfield", "--json",
                          "--strain", "1e-3", "0", "0", "0", "0", "0"], capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    for f in ("output_SS316L_polycrystal.txt", "cg_history_polycrystal.txt", "cgitr_SS316L_polycrystal.txt",
              "fullfield_poly.h5"):
        assert os.path.getsize(tmp_path / f) > 0
    log = open(tmp_path / "output_SS316L_polycrystal.txt").read()
    op = O.Problem(14, 14, 14, 7, exx=1e-3, ezz=0.0)
    ref = O.run(op, pix, rod)
    assert f"Number of conjugate steps= {ref['lstep']}" in log or "Number of conjugate steps=" in log
    energy = float(log.split(" Energy=")[1].split()[0])
    assert abs(energy - ref["utot"]) <= 1e-9 * abs(ref["utot"])
    import json

    metrics = json.loads([ln for ln in out.stdout.splitlines() if ln.startswith("{")][-1])
    assert metrics["utot"] == pytest.approx(ref["utot"], rel=1e-9)
    assert metrics["iterations"] == int(log.split("Number of conjugate steps=")[1].split()[0])
    assert metrics["dof"] == 3 * 14 ** 3 and metrics["precision"] == "fp64"
    ff = str(tmp_path / "fullfield_poly.h5")
    assert np.array_equal(e3d.h5_read(ff, "pix"), pix)
    o = O.Oracle(op, pix, rod).femat()
    sig_ref, vm_ref = o.stress_fullfield(ref["u"])
    sig = e3d.h5_read(ff, "stress_tensor")
    assert sig.shape == (6, 14 ** 3)
    den = np.linalg.norm(sig_ref)
    assert np.linalg.norm(sig.ravel() - sig_ref) <= 1e-6 * den  # the converged fields of two solvers
    assert np.linalg.norm(e3d.h5_read(ff, "vm") - vm_ref) <= 1e-6 * np.linalg.norm(vm_ref)


def test_upload_refuses_out_of_range_phases_and_recovers():
    """The phase range check (src/elas3dxtal_pcg.f90:2986-2989) runs on the
    device after one copy of the map: a refused map leaves no upload behind
    (femat refuses), and a correct upload afterwards solves like a fresh one."""
    p, pix, rod = W.c1(n=10, ngrains=4, seed=3)
    with e3d.Elas3D(p) as g:
        for bad_value in (0, p.nphase + 1):
            bad = pix.copy()
            bad[p.ns // 2] = bad_value
            with pytest.raises(e3d.E3DError) as ei:
                g.upload(bad, rod)
            assert ei.value.code == e3d.E3D_ERR_INPUT
            with pytest.raises(e3d.E3DError) as ei:
                g.femat()
            assert ei.value.code == e3d.E3D_ERR_STATE
        g.upload(pix, rod)
        res = g.run()
    with e3d.Elas3D(p) as g2:
        g2.upload(pix, rod)
        ref = g2.run()
    assert res["iterations"] == ref["iterations"] and res["utot"] == ref["utot"]
