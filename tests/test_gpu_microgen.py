"""GPU microstructure generator (e3d_micro_*_device): the same phase maps and
orientations as the host generator, bit for bit, and device-side upload into a
solver handle (e3d_upload_device) equivalent to the host upload."""
import numpy as np
import pytest

import elas3d_xtal_gb300 as e3d

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

CASES = [
    (40, 37, 42, 30, 0.0, 1),
    (33, 30, 35, 200, 0.5, 2),   # Laguerre weights
    (64, 61, 66, 64, 0.0, 3),
    (12, 9, 14, 5, 0.0, 4),      # fewer than three seed cells per direction: every seed searched
    (50, 47, 52, 7, 0.3, 5),
    (96, 96, 96, 1000, 0.0, 6),
]


@pytest.mark.parametrize("nx,ny,nz,ng,sigma,seed", CASES)
def test_device_generator_matches_host(nx, ny, nz, ng, sigma, seed):
    pix, rod = e3d.micro_grains(nx, ny, nz, ng, seed, laguerre_sigma=sigma)
    n_sph = e3d.micro_spherical_pores(pix, nx, ny, nz, 0.02, ng + 1, seed + 10)
    n_ell = e3d.micro_ellipsoidal_pores(pix, nx, ny, nz, 0.04, ng + 1, seed + 20)
    d = torch.empty(nx * ny * nz, dtype=torch.int32, device="cuda")
    rod_d = e3d.micro_grains_device(d, nx, ny, nz, ng, seed, laguerre_sigma=sigma)
    grains_only = d.cpu().numpy().copy()
    m_sph = e3d.micro_spherical_pores_device(d, nx, ny, nz, 0.02, ng + 1, seed + 10)
    m_ell = e3d.micro_ellipsoidal_pores_device(d, nx, ny, nz, 0.04, ng + 1, seed + 20)
    assert np.array_equal(rod_d, rod)
    assert (n_sph, n_ell) == (m_sph, m_ell)
    assert np.array_equal(d.cpu().numpy(), pix)
    ref, _ = e3d.micro_grains(nx, ny, nz, ng, seed, laguerre_sigma=sigma)
    assert np.array_equal(grains_only, ref)


def test_upload_device_solves_like_upload():
    n, ng = 24, 12
    pix, rod = e3d.micro_grains(n, n, n, ng, 3)
    e3d.micro_spherical_pores(pix, n, n, n, 0.02, ng + 1, 4, log_mu=np.log(1.5))
    d = torch.from_numpy(pix).cuda()
    p = e3d.Problem(n, n, n, ng + 1, c11=240e9, c12=150e9, c44=90e9)
    with e3d.Elas3D(p) as a, e3d.Elas3D(p) as b:
        ra = a.upload(pix, rod).run()
        rb = b.upload_device(d, rod).run()
        assert ra["iterations"] == rb["iterations"] and ra["utot"] == rb["utot"]
        assert np.array_equal(a.get_u(), b.get_u())


def test_upload_device_rejects_out_of_range_phase():
    n = 8
    p = e3d.Problem(n, n, n, 3)
    d = torch.ones(n ** 3, dtype=torch.int32, device="cuda")
    d[17] = 4  # nphase + 1
    with e3d.Elas3D(p) as g:
        with pytest.raises(e3d.E3DError):
            g.upload_device(d, np.zeros(6))
        d[17] = 2
        g.upload_device(d, np.zeros(6))  # the handle stays usable
