"""Independent numpy/scipy restatement of the reference's voxel-FE system.

TEST INFRASTRUCTURE ONLY (cross-checks the C oracle; never used by the
product).  It shares no code with oracle/e3d_oracle.c and uses different
formulations on purpose:

- element stiffness by 2x2x2 Gauss quadrature (the reference uses 3x3x3
  Simpson, src/elas3dxtal_pcg.f90:713-805; both are exact for this integrand);
- the global stiffness as an explicitly assembled scipy sparse matrix over the
  periodic grid (the reference applies a 27-point stencil node by node,
  :1176-1321);
- b and C from the expansion of U(u) = 1/2 sum_e (u_e + delta_e)^T K_e
  (u_e + delta_e) (the reference enumerates faces, edges and the corner,
  :815-1100);
- the Bond-rotated stiffness rebuilt from the 4th-order tensor rotation
  (used to check the reference's xz/yz slot ordering).
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp

# reference local node order (src/elas3dxtal_pcg.f90:639)
LO = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]])
VOIGT = [(0, 0), (1, 1), (2, 2), (0, 2), (1, 2), (0, 1)]  # xx yy zz xz yz xy (reference order)


def bmatrix(x, y, z):
    """6 x 24 strain-displacement matrix at local point (x,y,z), columns (node a, dof c)."""
    B = np.zeros((6, 24))
    for a, (ox, oy, oz) in enumerate(LO):
        fx = (x if ox else 1 - x)
        fy = (y if oy else 1 - y)
        fz = (z if oz else 1 - z)
        dx = (1 if ox else -1) * fy * fz
        dy = (1 if oy else -1) * fx * fz
        dz = (1 if oz else -1) * fx * fy
        B[0, 3 * a + 0] = dx
        B[1, 3 * a + 1] = dy
        B[2, 3 * a + 2] = dz
        B[3, 3 * a + 0] = dz
        B[3, 3 * a + 2] = dx
        B[4, 3 * a + 1] = dz
        B[4, 3 * a + 2] = dy
        B[5, 3 * a + 0] = dy
        B[5, 3 * a + 1] = dx
    return B


def element_stiffness(C6: np.ndarray) -> np.ndarray:
    """24x24 K_e = int B^T C B over the unit cube, 2x2x2 Gauss."""
    g = 0.5 / np.sqrt(3.0)
    pts = [0.5 - g, 0.5 + g]
    K = np.zeros((24, 24))
    for x in pts:
        for y in pts:
            for z in pts:
                B = bmatrix(x, y, z)
                K += 0.125 * B.T @ C6 @ B
    return K


def cubic_voigt(c11, c12, c44):
    C = np.zeros((6, 6))
    C[:3, :3] = c12
    for i in range(3):
        C[i, i] = c11
    C[3, 3] = C[4, 4] = C[5, 5] = c44
    return C


def rodrigues_to_Q(r):
    r = np.asarray(r, float)
    rr = r @ r
    K = np.array([[0, -r[2], r[1]], [r[2], 0, -r[0]], [-r[1], r[0], 0]])
    return ((1 - rr) * np.eye(3) + 2 * np.outer(r, r) + 2 * K) / (1 + rr)


def tensor_from_voigt(C6):
    T = np.zeros((3, 3, 3, 3))
    for I, (i, j) in enumerate(VOIGT):
        for J, (k, l) in enumerate(VOIGT):
            for (a, b) in {(i, j), (j, i)}:
                for (c, d) in {(k, l), (l, k)}:
                    T[a, b, c, d] = C6[I, J]
    return T


def voigt_from_tensor(T):
    C6 = np.zeros((6, 6))
    for I, (i, j) in enumerate(VOIGT):
        for J, (k, l) in enumerate(VOIGT):
            C6[I, J] = T[i, j, k, l]
    return C6


def rotate_voigt(C6, Q):
    """True rotation C'_ijkl = Q_ia Q_jb Q_kc Q_ld C_abcd."""
    T = tensor_from_voigt(C6)
    return voigt_from_tensor(np.einsum("ia,jb,kc,ld,abcd->ijkl", Q, Q, Q, Q, T))


SWAP45 = np.eye(6)[[0, 1, 2, 4, 3, 5]]


def reference_rotated(C6, r):
    """The stiffness the reference applies: P R(Q^T)[C] P with P swapping the xz
    and yz Voigt slots (its Bond matrix mixes (..,xz,yz,..) rows with
    (..,yz,xz,..) columns, src/elas3dxtal_pcg.f90:2577-2621)."""
    Q = rodrigues_to_Q(r)
    return SWAP45 @ rotate_voigt(C6, Q.T) @ SWAP45


def cmod_table(nphase, flag_m, c11, c12, c44, rod, e1=0.0, nu1=0.0):
    cm = np.zeros((nphase, 6, 6))
    ck = np.zeros((6, 6))
    ck[:3, :3] = 1.0
    cmu = np.zeros((6, 6))
    cmu[:3, :3] = -2.0 / 3.0
    for i in range(3):
        cmu[i, i] = 4.0 / 3.0
    cmu[3, 3] = cmu[4, 4] = cmu[5, 5] = 1.0
    K1 = e1 / 3.0 / (1.0 - 2.0 * nu1)
    G1 = e1 / 2.0 / (1.0 + nu1)
    if flag_m == 1:
        Cc = cubic_voigt(c11, c12, c44)
        for p in range(nphase - 1):
            cm[p] = reference_rotated(Cc, rod[3 * p:3 * p + 3])
    else:
        K0 = (c11 + 2 * c12) / 3.0
        G0 = (c11 - c12 + 3 * c44) / 5.0
        E0 = 9 * K0 * G0 / (3 * K0 + G0)
        nu0 = (3 * K0 - 2 * G0) / (2 * (3 * K0 + G0))
        for p in range(nphase - 1):
            cm[p] = E0 / 3 / (1 - 2 * nu0) * ck + E0 / 2 / (1 + nu0) * cmu
    cm[nphase - 1] = K1 * ck + G1 * cmu
    return cm


class SparseModel:
    """Globally assembled periodic stiffness; DOF index = c*ns + m (SoA)."""

    def __init__(self, nx, ny, nz, pix, cmod, strain):
        self.nx, self.ny, self.nz = nx, ny, nz
        ns = nx * ny * nz
        self.ns = ns
        pix = np.asarray(pix).reshape(-1)
        Ke = np.array([element_stiffness(c) for c in cmod])  # [p, 24, 24]
        self.Ke = Ke
        i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
        i, j, k = i.ravel(order="F"), j.ravel(order="F"), k.ravel(order="F")
        m = i + nx * (j + ny * k)
        order = np.argsort(m)
        i, j, k = i[order], j[order], k[order]
        nodes = np.stack([((i + ox) % nx) + nx * (((j + oy) % ny) + ny * ((k + oz) % nz))
                          for (ox, oy, oz) in LO], axis=1)  # [ns, 8]
        dofs = np.concatenate([nodes[:, a:a + 1] + ns * c for a in range(8) for c in range(3)], axis=1)
        ph = pix - 1
        rows = np.repeat(dofs, 24, axis=1).ravel()
        cols = np.tile(dofs, (1, 24)).ravel()
        vals = Ke[ph].reshape(ns, 576).ravel()
        self.K = sp.csr_matrix((vals, (rows, cols)), shape=(3 * ns, 3 * ns))
        # jumps: element with lower corner on a high face, local node offset 1 along it
        E = np.array([[strain[0], strain[5], strain[3]], [strain[5], strain[1], strain[4]],
                      [strain[3], strain[4], strain[2]]])
        wrap = np.stack([(i == nx - 1), (j == ny - 1), (k == nz - 1)], axis=1)
        nvec = np.array([nx, ny, nz], float)
        delta = np.zeros((ns, 24))
        for a, o in enumerate(LO):
            for c in range(3):
                delta[:, 3 * a + c] = ((wrap * o) * E[c] * nvec).sum(axis=1)
        Kd = np.einsum("eij,ej->ei", Ke[ph], delta)
        self.b = np.zeros(3 * ns)
        np.add.at(self.b, dofs.ravel(), Kd.ravel())
        self.C = 0.5 * float(np.einsum("ei,ei->", delta, Kd))
        self.E = E

    def apply(self, x):
        return self.K @ x

    def energy(self, u):
        Ku = self.K @ u
        return Ku + self.b, self.C + 0.5 * u @ Ku + self.b @ u

    def affine(self):
        ns, nx, ny = self.ns, self.nx, self.ny
        m = np.arange(ns)
        x, y, z = m % nx, (m // nx) % ny, m // (nx * ny)
        E = self.E
        return np.concatenate([x * E[0, 0] + y * E[0, 1] + z * E[0, 2],
                               x * E[1, 0] + y * E[1, 1] + z * E[1, 2],
                               x * E[2, 0] + y * E[2, 1] + z * E[2, 2]])

    def block_jacobi(self):
        ns = self.ns
        D = self.K.diagonal()
        out = np.zeros((ns, 3, 3))
        Kc = self.K.tocsr()
        for c in range(3):
            for d in range(3):
                out[:, c, d] = np.asarray(Kc[c * ns + np.arange(ns), d * ns + np.arange(ns)]).ravel()
        inv = np.zeros_like(out)
        det = np.linalg.det(out)
        ok = np.abs(det) >= 1e-14
        inv[ok] = np.linalg.inv(out[ok])
        del D
        return inv

    def pcg(self, tol=1e-8, maxit=10000, criterion=0, reset=True, plain=False):
        """The reference's PCG (src/elas3dxtal_pcg.f90:1527-2012) in numpy.
        plain=True: the unpreconditioned CG of the serial and cg variants
        (applications/sec3_1/serial/n_100x100x100/elas3dxtal_serial.f90:898-1052):
        z = g, so gg = g.g and h starts as g."""
        ns = self.ns
        u = self.affine()
        g, _ = self.energy(u)
        gg0 = g @ g
        Mi = None if plain else self.block_jacobi()

        def prec(v):
            if plain:
                return v.copy()
            V = v.reshape(3, ns).T
            return np.einsum("mij,mj->mi", Mi, V).T.ravel()

        z = prec(g)
        gg = z @ g
        h = z.copy()
        den = gg if criterion == 1 else gg0
        prev = np.sqrt(gg / den)
        tolf = float(np.float32(tol))
        L = 0
        for L in range(1, maxit + 1):
            Ah = self.K @ h
            hAh = h @ Ah
            if abs(hAh) < 1e-14:
                break
            lam = gg / hAh
            u -= lam * h
            g -= lam * Ah
            z = prec(g)
            last = gg
            gg = z @ g
            rel = np.sqrt(gg / den)
            if reset and rel > 10 * prev and L > 1:
                h = z.copy()
            else:
                h = z + (gg / last) * h
            prev = rel
            if rel < tolf:
                break
        return u, L
