"""Coarse grid of the learned closure, on the CPU: restriction keeps the
lab-frame sums, prolongation inverts it, coarsened velocities keep face
fluxes and the divergence, and the schedule maps onto coarse steps."""
import numpy as np
import pytest
import torch

from initializator_gb300 import coarse as cg
from initializator_gb300 import geometry


def lab_sum(f, k, d):
    nz, ny, nx = f[0].shape
    z, y, x = np.meshgrid(*[(np.arange(n) + 0.5) * dd for n, dd in zip((nz, ny, nx), d[::-1])], indexing="ij")
    ph = np.exp(-1j * (k[0] * x + k[1] * y + k[2] * z))
    return (ph * (f[0].numpy() + 1j * f[1].numpy())).sum(), f[2].numpy().sum()


@pytest.mark.parametrize("k", [(0.0, 0.0, 0.0), (3e5, -2e5, 1e5), (0.0, 0.0, 2.5e6)])
def test_restriction_keeps_lab_sums(k):
    rng = np.random.default_rng(0)
    f = [torch.tensor(rng.standard_normal((6, 4, 8))) for _ in range(3)]
    k = np.array(k)
    dxf = (1e-6, 1.3e-6, 0.8e-6)
    c = cg.restrict(f, k, dxf)
    sf, zf = lab_sum(f, k, dxf)
    sc, zc = lab_sum(c, k, tuple(2 * d for d in dxf))
    assert abs(sf - 8 * sc) <= 1e-12 * abs(sf) + 1e-12
    assert abs(zf - 8 * zc) <= 1e-12


def test_prolong_inverts_restrict():
    rng = np.random.default_rng(1)
    c = [torch.tensor(rng.standard_normal((3, 2, 4))) for _ in range(3)]
    k = np.array([1e5, 4e5, -3e5])
    dxf = (1e-6,) * 3
    back = cg.restrict(cg.prolong(c, k, dxf, np.ones((6, 4, 8))), k, dxf)
    for a, b in zip(c, back):
        assert float((a - b).abs().max()) < 1e-14
    # partly solid cells: fine solid voxels are zero, the coarse value is kept
    mask = (rng.random((6, 4, 8)) > 0.5).astype(np.uint8)
    mask[0:2, 0:2, 0:2] = 0
    fp = cg.prolong(c, k, dxf, mask)
    assert float(fp[0][torch.as_tensor(mask) == 0].abs().max()) == 0.0
    back = cg.restrict(fp, k, dxf)
    _, phi, _ = cg.coarsen_geometry(mask, None)
    for a, b in zip(c, back):
        assert float((a - b)[torch.as_tensor(phi) > 0].abs().max()) < 1e-14
        assert float(b[0, 0, 0]) == 0.0


def test_coarsened_geometry_and_flux():
    mask = geometry.sphere_pack((8, 10, 12), 2.0, 0.3, seed=3)
    vel = geometry.curl_velocity(mask, 1.5, 1e-3, seed=4)
    mc, phi, (vx, vy, vz) = cg.coarsen_geometry(mask, vel)
    assert mc.shape == (4, 5, 6) and vx.shape == (4, 5, 7) and vy.shape == (4, 6, 6) and vz.shape == (5, 5, 6)
    assert np.array_equal(mc, (phi > 0).astype(np.uint8))
    assert abs(phi.mean() - mask.mean()) < 1e-15
    # flux through each coarse face = (2 dx)^2 * mean of its 4 fine faces = dx^2 * sum
    assert np.allclose(4 * vx[1, 2, 3], vel[0][2:4, 4:6, 6].sum())
    # net outflow of a coarse cell = the summed net outflow of its 8 fine cells
    def outflow(vx, vy, vz):
        return (vx[:, :, 1:] - vx[:, :, :-1]) + (vy[:, 1:, :] - vy[:, :-1, :]) + (vz[1:] - vz[:-1])
    fine = outflow(*vel).reshape(4, 2, 5, 2, 6, 2).sum(axis=(1, 3, 5))
    assert np.allclose(4 * outflow(vx, vy, vz), fine, rtol=0, atol=1e-18)
    with pytest.raises(ValueError):
        cg.coarsen_geometry(np.ones((3, 4, 4), np.uint8), None)


def test_schedule_maps_to_coarse_steps():
    wave = np.arange(24, dtype=np.float64).reshape(8, 3)
    wc = cg.coarse_waveform(wave, 2)
    g, dt = 2.675e8, 1e-5
    assert np.allclose(cg.kvec(wc, g, 4 * dt, 2), cg.kvec(wave, g, dt, 8), rtol=1e-14)
    assert cg.coarse_pulses([(7, 2, 3.14, (1, 0, 0))]) == [(1, 2, 3.14, (1, 0, 0))]
    with pytest.raises(ValueError):
        cg.coarse_pulses([(6, 2, 3.14, (1, 0, 0))])


def test_pore_average_restriction_keeps_weighted_lab_sums():
    rng = np.random.default_rng(2)
    mask = (rng.random((6, 4, 8)) > 0.4).astype(np.uint8)
    f = [torch.tensor(rng.standard_normal((6, 4, 8)) * mask) for _ in range(3)]
    k = np.array([3e5, -2e5, 1e5])
    dxf = (1e-6,) * 3
    c = cg.restrict(f, k, dxf, mask)
    _, phi, _ = cg.coarsen_geometry(mask, None)
    a = cg.lab_sums(f, k, dxf)
    b = 8 * cg.lab_sums(c, k, (2e-6,) * 3, phi)
    assert np.abs(a - b).max() <= 1e-12 * np.abs(a).max()
    back = cg.restrict(cg.prolong(c, k, dxf, mask, pore_average=True), k, dxf, mask)
    for x, y in zip(c, back):
        assert float((x - y).abs().max()) < 1e-14
