"""The CPU oracle against analytical known-answer tests and the independent
scipy restatement (oracle/np_ref.py).  The reference ships no golden vectors,
so these pin the oracle (CPU only)."""
import numpy as np
import pytest

import np_ref as R
import oracle as O

C11, C12, C44 = 206e9, 133e9, 119e9


def _rand_problem(nx, ny, nz, ng, seed, pores=True, strain=None, **kw):
    rng = np.random.default_rng(seed)
    nphase = ng + 1
    pix = rng.integers(1, nphase + (1 if pores else 0), size=nx * ny * nz).astype(np.int32)
    rod = rng.normal(size=3 * ng)
    s = rng.normal(size=6) * 1e-3 if strain is None else np.asarray(strain, float)
    p = O.Problem(nx, ny, nz, nphase, exx=s[0], eyy=s[1], ezz=s[2], exz=s[3], eyz=s[4], exy=s[5], **kw)
    return p, pix, rod, s


def _rel(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / max(np.linalg.norm(np.ravel(b)), 1e-300))


# ---------------------------------------------------------------- stiffness
def test_rotation_matches_tensor_rotation_with_xz_yz_swap():
    """rotatestiffnessby equals P R(Q^T)[C] P (xz/yz slots swapped)."""
    rng = np.random.default_rng(0)
    rod = rng.normal(size=3 * 5)
    got = O.rotate_stiffness(rod, C11, C12, C44)
    Cc = R.cubic_voigt(C11, C12, C44)
    for g in range(5):
        ref = R.reference_rotated(Cc, rod[3 * g:3 * g + 3])
        assert np.abs(got[g] - ref).max() < 1e-12 * C11


def test_zener_one_is_orientation_independent():
    c44 = (C11 - C12) / 2.0
    rng = np.random.default_rng(1)
    got = O.rotate_stiffness(rng.normal(size=12), C11, C12, c44)
    iso = R.cubic_voigt(C11, C12, c44)
    assert np.abs(got - iso).max() < 1e-12 * C11


def test_dk_matches_gauss_and_is_psd_with_six_rigid_modes():
    p, pix, rod, _ = _rand_problem(3, 3, 3, 4, seed=2)
    o = O.Oracle(p, pix, rod).femat()
    dk = o.dk_array()
    cm = o.cmod_array()
    for ph in range(p.nphase - 1):
        K = dk[ph].reshape(24, 24)
        Kg = R.element_stiffness(cm[ph])
        assert np.abs(K - Kg).max() < 1e-13 * np.abs(Kg).max()
        w = np.linalg.eigvalsh(0.5 * (K + K.T))
        assert (w > -1e-6 * w.max()).all()
        assert (np.abs(w) < 1e-9 * w.max()).sum() == 6
    assert np.abs(dk[p.nphase - 1]).max() == 0.0  # zero-stiffness pore phase


def test_cmod_matches_independent_table():
    for flag in (0, 1):
        p, pix, rod, _ = _rand_problem(2, 2, 2, 3, seed=3, flag_m=flag)
        p.e1, p.nu1 = 30e9, 0.2
        o = O.Oracle(p, pix, rod).femat()
        ref = R.cmod_table(p.nphase, flag, p.c11, p.c12, p.c44, rod, p.e1, p.nu1)
        assert np.abs(o.cmod_array() - ref).max() < 1e-12 * C11


# ---------------------------------------------------------------- stencil
@pytest.mark.parametrize("shape", [(3, 4, 5), (6, 6, 6), (1, 2, 3), (7, 3, 2)])
def test_apply_b_C_match_sparse_assembly(shape):
    nx, ny, nz = shape
    p, pix, rod, s = _rand_problem(nx, ny, nz, 4, seed=nx * 7 + ny)
    o = O.Oracle(p, pix, rod).femat()
    sm = R.SparseModel(nx, ny, nz, pix, o.cmod_array(), s)
    x = np.random.default_rng(5).normal(size=3 * p.ns)
    assert _rel(o.apply(x), sm.apply(x)) < 1e-13
    assert _rel(o.b, sm.b) < 1e-13
    assert abs(o.C - sm.C) <= 1e-12 * abs(sm.C)


def test_rigid_translation_and_symmetry():
    p, pix, rod, _ = _rand_problem(5, 4, 6, 5, seed=9)
    o = O.Oracle(p, pix, rod).femat()
    rng = np.random.default_rng(3)
    v, w = rng.normal(size=3 * p.ns), rng.normal(size=3 * p.ns)
    Kv, Kw = o.apply(v), o.apply(w)
    assert abs(w @ Kv - v @ Kw) <= 1e-12 * np.linalg.norm(Kv) * np.linalg.norm(w)
    for c in range(3):
        t = np.zeros(3 * p.ns)
        t[c * p.ns:(c + 1) * p.ns] = 1.0
        assert np.linalg.norm(o.apply(t)) <= 1e-13 * np.linalg.norm(Kv) * np.sqrt(p.ns) / np.linalg.norm(v)


def test_homogeneous_affine_is_equilibrium_and_energy_is_exact():
    """One grain: the affine field is the exact solution, g = 0 and
    U = 1/2 eps^T C eps * ns (engineering shear)."""
    s = np.array([1e-3, -2e-4, 5e-4, 3e-4, -1e-4, 2e-4])  # exx eyy ezz exz eyz exy (tensor)
    p = O.Problem(6, 5, 4, 2, exx=s[0], eyy=s[1], ezz=s[2], exz=s[3], eyz=s[4], exy=s[5])
    pix = np.ones(p.ns, np.int32)
    rod = np.array([0.3, -0.2, 0.5])
    o = O.Oracle(p, pix, rod).femat()
    u = o.affine_u()
    g, U = o.energy(u)
    assert np.linalg.norm(g) <= 1e-10 * np.linalg.norm(o.b)
    eng = np.array([s[0], s[1], s[2], 2 * s[3], 2 * s[4], 2 * s[5]])
    Cm = o.cmod_array()[0]
    assert abs(U - 0.5 * eng @ Cm @ eng * p.ns) <= 1e-10 * abs(U)
    sig, eps = o.stress(u)
    assert _rel(eps, eng) < 1e-12
    assert _rel(sig, Cm @ eng) < 1e-12


def test_invert3x3_rules():
    rng = np.random.default_rng(4)
    for _ in range(20):
        A = rng.normal(size=(3, 3))
        A = A @ A.T + 0.1 * np.eye(3)
        assert np.abs(O.invert3x3(A) @ A - np.eye(3)).max() < 1e-10
    assert np.abs(O.invert3x3(np.zeros((3, 3)))).max() == 0.0
    assert np.abs(O.invert3x3(1e-6 * np.eye(3))).max() == 0.0  # |det| = 1e-18 < 1e-14


def test_block_jacobi_matches_sparse_diagonal_blocks():
    p, pix, rod, s = _rand_problem(4, 5, 3, 3, seed=11)
    o = O.Oracle(p, pix, rod).femat()
    minv = o.block_jacobi().reshape(3, 3, p.ns).transpose(2, 1, 0)
    ref = R.SparseModel(4, 5, 3, pix, o.cmod_array(), s).block_jacobi()
    assert np.abs(minv - ref).max() <= 1e-12 * np.abs(ref).max()


def test_pore_only_nodes_get_zero_preconditioner():
    p = O.Problem(4, 4, 4, 3)
    pix = np.full(p.ns, 3, np.int32)  # everything pore
    pix[:8] = 1
    rod = np.zeros(6)
    o = O.Oracle(p, pix, rod).femat()
    minv = o.block_jacobi().reshape(9, p.ns)
    far = 42  # a node whose 8 elements are all pore
    assert np.all(minv[:, far] == 0.0)


# ---------------------------------------------------------------- solve
def test_solve_matches_independent_pcg():
    p, pix, rod, s = _rand_problem(6, 5, 7, 4, seed=21, strain=[1e-3, 0, 0, 0, 0, 0])
    r = O.run(p, pix, rod)
    o = O.Oracle(p, pix, rod).femat()
    sm = R.SparseModel(p.nx, p.ny, p.nz, pix, o.cmod_array(), s)
    u, L = sm.pcg(tol=p.tol)
    assert abs(r["lstep"] - L) <= 2
    _, U = sm.energy(u)
    assert abs(r["utot"] - U) <= 1e-9 * abs(U)


def test_plain_cg_matches_independent_cg():
    """The oracle's identity-preconditioner mode is the unpreconditioned CG of
    the reference's serial and cg variants (no divergence reset there)."""
    p, pix, rod, s = _rand_problem(6, 5, 7, 4, seed=23, strain=[0, 0, 0, 5e-4, 0, 0])
    p.precond = 1
    p.divergence_reset = 0
    r = O.run(p, pix, rod)
    o = O.Oracle(p, pix, rod).femat()
    sm = R.SparseModel(p.nx, p.ny, p.nz, pix, o.cmod_array(), s)
    u, L = sm.pcg(tol=p.tol, reset=False, plain=True)
    assert abs(r["lstep"] - L) <= 2
    _, U = sm.energy(u)
    assert abs(r["utot"] - U) <= 1e-9 * abs(U)
    # and it takes more iterations than the block-Jacobi PCG on the same problem
    p.precond = 0
    assert O.run(p, pix, rod)["lstep"] < r["lstep"]


# Cubic constants (GPa) of the reference's Zener-ratio sweep, keyed by the ratio
# A = 2 C44 / (C11 - C12) that names each case
# (applications/sec3_2/A_*/elas3dxtal_pcg.f90:68-70).
A_SWEEP = {
    0.5: (300.04, 84.95, 53.77), 0.75: (274.65, 97.64, 66.38), 1.0: (256.75, 106.59, 75.08),
    1.5: (232.07, 118.93, 84.85), 2.0: (216.52, 126.70, 89.82), 3.0: (198.66, 135.64, 94.53),
    4.0: (188.74, 140.60, 96.28), 5.0: (182.38, 143.78, 96.50),
}


@pytest.mark.parametrize("A", sorted(A_SWEEP))
def test_zener_sweep_solves_match_independent_pcg(A):
    """The oracle on the reference's own parameter sets: solves match the
    independent scipy PCG (iterations within 2, energy within 1e-9), and a
    single grain under a uniform strain carries <sigma> = cmod eps exactly."""
    c11, c12, c44 = (v * 1e9 for v in A_SWEEP[A])
    assert abs(2.0 * c44 / (c11 - c12) - A) < 1e-3 * A
    p, pix, rod, s = _rand_problem(5, 6, 4, 3, seed=40 + int(10 * A), strain=[1e-3, 0, 0, 0, 5e-4, 0],
                                   c11=c11, c12=c12, c44=c44)
    r = O.run(p, pix, rod)
    o = O.Oracle(p, pix, rod).femat()
    sm = R.SparseModel(p.nx, p.ny, p.nz, pix, o.cmod_array(), s)
    u, L = sm.pcg(tol=p.tol)
    assert abs(r["lstep"] - L) <= 2
    _, U = sm.energy(u)
    assert abs(r["utot"] - U) <= 1e-9 * abs(U)
    # one grain (no pores): the affine field is the solution and <sigma> = cmod eps,
    # eps in engineering shear (tensor shear inputs doubled)
    q, pix1, rod1, s1 = _rand_problem(4, 4, 4, 1, seed=7, pores=False, strain=[2e-4, -1e-4, 3e-4, 1e-4, 0, 2e-4],
                                      c11=c11, c12=c12, c44=c44)
    r1 = O.run(q, pix1, rod1)
    eng = s1 * np.array([1, 1, 1, 2, 2, 2])
    assert _rel(r1["epsav"], eng) < 1e-12
    cm = O.Oracle(q, pix1, rod1).femat().cmod_array()[0]
    assert _rel(r1["strav"], cm @ eng) < 1e-9


def test_effective_modulus_between_voigt_and_reuss():
    rng = np.random.default_rng(8)
    ng, n = 6, 8
    p = O.Problem(n, n, n, ng + 1, c11=240e9, c12=150e9, c44=120e9, exx=1e-3, ezz=0.0, tol=1e-10)
    # coarse random grains (2x2x2 blocks) with no pores
    blocks = rng.integers(1, ng + 1, size=(n // 2,) * 3)
    pix = np.repeat(np.repeat(np.repeat(blocks, 2, 0), 2, 1), 2, 2).transpose(2, 1, 0).ravel().astype(np.int32)
    rod = rng.normal(size=3 * ng)
    r = O.run(p, pix, rod)
    o = O.Oracle(p, pix, rod).femat()
    frac = np.bincount(pix, minlength=ng + 2)[1:ng + 1] / p.ns
    Cs = o.cmod_array()[:ng]
    Cv = np.einsum("g,gij->ij", frac, Cs)
    Sr = np.einsum("g,gij->ij", frac, np.linalg.inv(Cs))
    eps = np.array([1e-3, 0, 0, 0, 0, 0])
    W = 0.5 * eps @ (r["strav"]) * 1.0  # energy density under the imposed strain
    assert 0.5 * eps @ np.linalg.inv(Sr) @ eps <= W * (1 + 1e-9)
    assert W <= 0.5 * eps @ Cv @ eps * (1 + 1e-9)
    assert _rel(r["epsav"][[0]], [1e-3]) < 1e-9


def test_divergence_reset_and_criterion_variants_run():
    p, pix, rod, _ = _rand_problem(5, 5, 5, 3, seed=31, strain=[0, 0, 1e-3, 0, 0, 0])
    for crit in (0, 1):
        for reset in (0, 1):
            p.criterion, p.divergence_reset = crit, reset
            r = O.run(p, pix, rod)
            assert r["exit_reason"] == 0 and r["lstep"] > 0


def test_reduction_order_changes_rounding_only():
    """Another chunk length for the oracle's dot products is another valid FP64
    summation order: the solve ends at the same energy to rounding, the
    history agrees closely, and the default comes back with 0."""
    p, pix, rod, _ = _rand_problem(10, 9, 8, 5, seed=41, strain=[1e-3, 0, 0, 0, 2e-4, 0])
    a = O.run(p, pix, rod)
    try:
        O.set_reduction_chunk(64)
        b = O.run(p, pix, rod)
    finally:
        O.set_reduction_chunk(0)
    c = O.run(p, pix, rod)
    assert abs(a["utot"] - b["utot"]) <= 1e-12 * abs(a["utot"])
    assert abs(a["lstep"] - b["lstep"]) <= 1
    n = min(a["history"].size, b["history"].size)
    assert np.max(np.abs(a["history"][:n] - b["history"][:n]) / a["history"][:n]) < 1e-6
    assert np.array_equal(a["history"], c["history"]) and a["utot"] == c["utot"]


def test_pcg_in_steps_equals_dembx():
    """The stepwise PCG (set-up, iterations in several calls, tear-down) is the
    same solve as one dembx call, bit for bit."""
    p, pix, rod, _ = _rand_problem(7, 6, 5, 3, seed=43, strain=[0, 5e-4, 0, 0, 0, 1e-4])
    o = O.Oracle(p, pix, rod).femat()
    u = o.affine_u()
    g, _ = o.energy(u)
    gg0 = float(g @ g)
    r = o.dembx(u, g, gg0)
    s = o.pcg(u, g, gg0)
    while s.iterate(3) < 0:
        pass
    d = s.close()
    assert d["lstep"] == r["lstep"] and d["reason"] == r["reason"] == 0
    assert np.array_equal(s.u, r["u"]) and np.array_equal(d["history"], r["history"])


@pytest.mark.parametrize("axis", [0, 1, 2])
def test_laminate_matches_the_closed_form(axis):
    """A laminate of rotated cubic grains (tests/analytic.py): the converged
    solve carries the closed-form energy, <sigma> and <eps> to rounding, and
    an unconverged iterate (the reference's stop test) lies above the exact
    energy, which is the minimum."""
    import analytic as AN

    rng = np.random.default_rng(50 + axis)
    shape = [(12, 5, 6), (5, 11, 4), (6, 5, 13)][axis]
    ng = 4
    layers = rng.integers(1, ng + 1, size=shape[axis])
    pix = AN.laminate_pix(shape, layers, axis)
    rod = rng.normal(size=3 * ng)
    s = np.array([1e-3, -3e-4, 2e-4, 4e-4, -2e-4, 3e-4])
    c11, c12, c44 = (v * 1e9 for v in A_SWEEP[3.0])
    for crit in (1, 0):
        p = O.Problem(*shape, ng + 1, c11=c11, c12=c12, c44=c44, exx=s[0], eyy=s[1], ezz=s[2], exz=s[3],
                      eyz=s[4], exy=s[5], tol=1e-10, criterion=crit)
        r = O.run(p, pix, rod)
        cm = O.Oracle(p, pix, rod).femat().cmod_array()
        w, sig, _ = AN.laminate_exact(cm, layers, AN.engineering(s), axis)
        assert r["exit_reason"] == 0
        assert _rel(r["epsav"], AN.engineering(s)) < 1e-13
        if crit == 1:
            assert abs(r["utot"] - w * p.ns) <= 1e-12 * w * p.ns
            assert _rel(r["strav"], sig) < 1e-12
        else:
            assert 0 <= r["utot"] - w * p.ns <= 1e-8 * w * p.ns


def test_start_gradient_is_the_interface_force_of_the_affine_stress():
    """K u_affine + b (the gradient at the reference's affine start guess,
    src/elas3dxtal_pcg.f90:423-438 and :1332-1340) equals, node by node, the
    sum over the node's eight elements of sigma_e . s / 4 with sigma_e =
    cmod_e . eps and s = +-1 per axis (+ on the element's high side) -- the
    closed form the job engine's set-up uses instead of a stencil pass."""
    p, pix, rod, s = _rand_problem(7, 6, 5, 4, seed=77, strain=[1e-3, -4e-4, 2e-4, 3e-4, -1e-4, 5e-4])
    o = O.Oracle(p, pix, rod).femat()
    g, U = o.energy(o.affine_u())
    cm = o.cmod_array()
    eps = s * np.array([1, 1, 1, 2, 2, 2])
    sig = cm @ eps  # [phase, 6]
    nx, ny, nz = p.nx, p.ny, p.nz
    ph = (pix - 1).reshape(nz, ny, nx)
    g0 = np.zeros((3, nz, ny, nx))
    for a in range(8):
        ox, oy, oz = a & 1, (a >> 1) & 1, (a >> 2) & 1
        # element with lower corner (x-ox, y-oy, z-oz), periodic
        pe = np.roll(ph, shift=(oz, oy, ox), axis=(0, 1, 2))
        sg = sig[pe]  # [z, y, x, 6]
        sx, sy, sz = (1.0 if ox else -1.0), (1.0 if oy else -1.0), (1.0 if oz else -1.0)
        g0[0] += sx * sg[..., 0] + sy * sg[..., 5] + sz * sg[..., 3]
        g0[1] += sx * sg[..., 5] + sy * sg[..., 1] + sz * sg[..., 4]
        g0[2] += sx * sg[..., 3] + sy * sg[..., 4] + sz * sg[..., 2]
    g0 = 0.25 * g0.reshape(3, -1).ravel()
    assert np.max(np.abs(g0 - g)) <= 1e-12 * np.max(np.abs(g))
    # and the start energy C + sum(u.Ku/2 + b.u) = C + sum(u.(g + b))/2
    u = o.affine_u()
    assert abs(o.C + 0.5 * u @ (g0 + o.b) - U) <= 1e-12 * abs(U)


@pytest.mark.parametrize("flag_m", [1, 0])
def test_laminate_with_isotropic_inclusion_layers(flag_m):
    """Laminates that include the inclusion phase (isotropic, from E1 and nu1)
    and, for flag_m = 0, the isotropic (Voigt-Reuss-Hill) matrix phases: the
    closed form holds for any stiffness per layer, so these pin the phase
    tables of both material modes."""
    import analytic as AN

    rng = np.random.default_rng(90 + flag_m)
    shape, axis, ng = (5, 6, 14), 2, 3
    layers = rng.integers(1, ng + 2, size=shape[axis])  # grains 1..ng and the inclusion ng+1
    layers[:2] = [ng + 1, 1]
    pix = AN.laminate_pix(shape, layers, axis)
    rod = rng.normal(size=3 * ng)
    s = np.array([4e-4, 1e-3, -2e-4, 1e-4, 3e-4, -2e-4])
    p = O.Problem(*shape, ng + 1, flag_m=flag_m, c11=240e9, c12=150e9, c44=120e9, e1=380e9, nu1=0.27,
                  exx=s[0], eyy=s[1], ezz=s[2], exz=s[3], eyz=s[4], exy=s[5], tol=1e-10, criterion=1)
    r = O.run(p, pix, rod)
    cm = O.Oracle(p, pix, rod).femat().cmod_array()
    w, sig, _ = AN.laminate_exact(cm, layers, AN.engineering(s), axis)
    assert r["exit_reason"] == 0
    assert abs(r["utot"] - w * p.ns) <= 1e-12 * w * p.ns
    assert _rel(r["strav"], sig) < 1e-12


def test_laminate_effective_stiffness_matches_six_oracle_solves():
    """tests/analytic.py's exact 6x6 laminate stiffness (used against the batch
    engine on the GPU) equals the oracle's <sigma> over the six unit load cases
    and is symmetric positive definite."""
    import analytic as AN

    rng = np.random.default_rng(140)
    shape, axis, ng = (5, 13, 4), 1, 3
    layers = rng.integers(1, ng + 1, size=shape[axis])
    pix = AN.laminate_pix(shape, layers, axis)
    rod = rng.normal(size=3 * ng)
    cols = []
    for lc in range(6):
        s = np.zeros(6)
        s[lc] = 1e-3 if lc < 3 else 0.5e-3
        p = O.Problem(*shape, ng + 1, c11=240e9, c12=150e9, c44=100e9, exx=s[0], eyy=s[1], ezz=s[2], exz=s[3],
                      eyz=s[4], exy=s[5], tol=1e-10, criterion=1)
        cols.append(O.run(p, pix, rod)["strav"] / 1e-3)
    ceff = np.stack(cols, axis=1)
    cm = O.rotate_stiffness(rod, 240e9, 150e9, 100e9)
    exact = AN.laminate_ceff(cm, layers, axis)
    assert np.abs(ceff - exact).max() <= 1e-10 * np.abs(exact).max()
    assert np.abs(exact - exact.T).max() <= 1e-12 * np.abs(exact).max()
    assert np.linalg.eigvalsh(0.5 * (exact + exact.T)).min() > 0
