"""Closed-form solutions that pin the solvers without the oracle.

A laminate -- planes of voxels normal to one axis, each plane one grain -- has
an exact periodic solution: every layer carries a uniform strain, equal to the
imposed one in the in-plane components, while the three components that act on
the layer plane (normal strain and the two shears through it) adjust so that
the traction on the plane is the same in every layer and the fluctuation
averages to zero.  The displacement is then affine in each voxel layer and
continuous across them, so the trilinear hexahedra of the reference
(src/elas3dxtal_pcg.f90:599-809, femat) represent it exactly, and the discrete
minimiser IS this field: the energy, <sigma> and <eps> of a converged solve
equal the closed form to rounding, for any stiffness per layer (rotated cubic
crystals included).

Conventions as in the reference: strains in the order xx, yy, zz, xz, yz, xy
with engineering shears (the tensor inputs exz, eyz, exy doubled), stress =
cmod . strain, energy = 1/2 strain . cmod . strain per voxel of unit volume.
"""
import numpy as np

# strain / stress slots acting on a plane normal to x, y, z
PLANE_SLOTS = {0: (0, 3, 5), 1: (1, 4, 5), 2: (2, 3, 4)}


def laminate_pix(shape, layer_phase, axis):
    """1-based phase ids (x fastest) of a laminate whose layer l along `axis`
    is phase layer_phase[l]."""
    nx, ny, nz = shape
    assert len(layer_phase) == shape[axis]
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    idx = (i, j, k)[axis]
    return np.asarray(layer_phase)[idx].transpose(2, 1, 0).ravel().astype(np.int32)


def engineering(tensor_strain):
    """(exx, eyy, ezz, exz, eyz, exy) tensor components -> engineering strain."""
    return np.asarray(tensor_strain, float) * np.array([1, 1, 1, 2, 2, 2])


def laminate_exact(cmods, layer_phase, eng_strain, axis):
    """(energy density, <sigma>, per-layer strains) of the laminate under the
    mean engineering strain `eng_strain`; cmods[ph] is phase ph+1's 6x6."""
    T = list(PLANE_SLOTS[axis])
    E = np.asarray(eng_strain, float)
    Cs = [np.asarray(cmods[ph - 1], float) for ph in layer_phase]
    f = 1.0 / len(Cs)
    # traction t on the layer plane: sum_l f (C_TT^-1 (t - C_T: E)) = 0
    A = np.zeros((3, 3))
    rhs = np.zeros(3)
    for C in Cs:
        Ki = np.linalg.inv(C[np.ix_(T, T)])
        A += f * Ki
        rhs += f * Ki @ (C[T, :] @ E)
    t = np.linalg.solve(A, rhs)
    w, sig, strains = 0.0, np.zeros(6), []
    for C in Cs:
        e = E.copy()
        e[T] += np.linalg.solve(C[np.ix_(T, T)], t - C[T, :] @ E)
        w += f * 0.5 * e @ C @ e
        sig += f * C @ e
        strains.append(e)
    return w, sig, np.array(strains)


def laminate_ceff(cmods, layer_phase, axis):
    """Exact 6x6 effective stiffness of the laminate (columns: unit
    engineering strains)."""
    return np.stack([laminate_exact(cmods, layer_phase, np.eye(6)[c], axis)[1] for c in range(6)], axis=1)
