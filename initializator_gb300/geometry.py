"""Seeded synthetic pore geometries and flow fields.

The reference ships no geometry (its Poro.dat / Vx/Vy/Vz.dat are absent), so
every workload here is generated from a seed. All generators run on any torch
device (CPU for small cases, the GPU for the 1024x1024x768 case) and return
numpy arrays in this package's layouts: ``mask[k, j, i]`` (uint8, 1 = pore),
face velocities ``vx[k, j, 0..nx]``, ``vy[k, 0..ny, i]``, ``vz[0..nz, j, i]``.
"""
from __future__ import annotations

import math

import numpy as np
import torch


def sphere_pack(shape, radius: float, solid_fraction: float, seed: int, device="cpu") -> np.ndarray:
    """Overlapping solid spheres with uniform centres, added until the solid
    fraction reaches ``solid_fraction``. shape = (nz, ny, nx)."""
    nz, ny, nx = shape
    g = torch.Generator(device="cpu").manual_seed(seed)
    solid = torch.zeros(shape, dtype=torch.bool, device=device)
    target = solid_fraction * solid.numel()
    count = 0
    r = float(radius)
    ri = int(math.ceil(r))
    while count < target:
        c = torch.rand(3, generator=g, dtype=torch.float64) * torch.tensor([nz, ny, nx], dtype=torch.float64)
        cz, cy, cx = (float(v) for v in c)
        z0, z1 = max(0, int(cz) - ri - 1), min(nz, int(cz) + ri + 2)
        y0, y1 = max(0, int(cy) - ri - 1), min(ny, int(cy) + ri + 2)
        x0, x1 = max(0, int(cx) - ri - 1), min(nx, int(cx) + ri + 2)
        zz = torch.arange(z0, z1, device=device, dtype=torch.float64).view(-1, 1, 1) + 0.5 - cz
        yy = torch.arange(y0, y1, device=device, dtype=torch.float64).view(1, -1, 1) + 0.5 - cy
        xx = torch.arange(x0, x1, device=device, dtype=torch.float64).view(1, 1, -1) + 0.5 - cx
        ball = (zz * zz + yy * yy + xx * xx) <= r * r
        sub = solid[z0:z1, y0:y1, x0:x1]
        count += int((ball & ~sub).sum())
        sub |= ball
    return (~solid).to(torch.uint8).cpu().numpy()


def _smooth_noise(shape, sigma: float, gen: torch.Generator, device) -> torch.Tensor:
    """White noise convolved with a periodic Gaussian of std ``sigma`` voxels (via FFT)."""
    noise = torch.randn(shape, generator=gen, dtype=torch.float32, device="cpu").to(device)
    spec = torch.fft.rfftn(noise)
    freqs = [torch.fft.fftfreq(n, device=device) for n in shape[:-1]] + [torch.fft.rfftfreq(shape[-1], device=device)]
    k2 = torch.zeros(spec.shape, dtype=torch.float32, device=device)
    for ax, f in enumerate(freqs):
        view = [1] * len(shape)
        view[ax] = -1
        k2 = k2 + (f.view(view) ** 2).float()
    spec = spec * torch.exp(-2.0 * (math.pi ** 2) * (sigma ** 2) * k2)
    out = torch.fft.irfftn(spec, s=shape)
    return out / out.std()


def gaussian_random_field(shape, sigma: float, porosity: float, seed: int, device="cpu") -> np.ndarray:
    """Thresholded Gaussian random field with pore fraction ``porosity``."""
    g = torch.Generator(device="cpu").manual_seed(seed)
    field = _smooth_noise(tuple(shape), sigma, g, device)
    flat = field.flatten()
    n = flat.numel()
    sample = flat if n <= 16_000_000 else flat[torch.randint(0, n, (16_000_000,), generator=g).to(device)]
    thr = torch.quantile(sample.float(), porosity)
    return (field <= thr).to(torch.uint8).cpu().numpy()


def curl_velocity(mask: np.ndarray, sigma: float, vmax: float, seed: int, device="cpu"):
    """Face velocities from the curl of a Gaussian-smoothed vector potential.

    The potential lives on cell edges of the staggered grid, so the face
    fluxes are discretely divergence-free; faces touching solid and faces on
    the domain boundary are then set to zero and the field is scaled so that
    the largest face speed is ``vmax``."""
    nz, ny, nx = mask.shape
    g = torch.Generator(device="cpu").manual_seed(seed)
    ax = _smooth_noise((nz + 1, ny + 1, nx + 1), sigma, g, device)
    ay = _smooth_noise((nz + 1, ny + 1, nx + 1), sigma, g, device)
    az = _smooth_noise((nz + 1, ny + 1, nx + 1), sigma, g, device)
    # v = curl A with A_x on x-edges (k, j corners), etc.
    vx = (az[:nz, 1:, :] - az[:nz, :ny, :]) - (ay[1:, :ny, :] - ay[:nz, :ny, :])      # (nz, ny, nx+1)
    vy = (ax[1:, :, :nx] - ax[:nz, :, :nx]) - (az[:nz, :, 1:] - az[:nz, :, :nx])      # (nz, ny+1, nx)
    vz = (ay[:, :ny, 1:] - ay[:, :ny, :nx]) - (ax[:, 1:, :nx] - ax[:, :ny, :nx])      # (nz+1, ny, nx)
    pore = torch.from_numpy(mask).to(device).bool()
    ox = torch.zeros((nz, ny, nx + 1), dtype=torch.bool, device=device)
    ox[:, :, 1:nx] = pore[:, :, 1:] & pore[:, :, :-1]
    oy = torch.zeros((nz, ny + 1, nx), dtype=torch.bool, device=device)
    oy[:, 1:ny, :] = pore[:, 1:, :] & pore[:, :-1, :]
    oz = torch.zeros((nz + 1, ny, nx), dtype=torch.bool, device=device)
    oz[1:nz, :, :] = pore[1:, :, :] & pore[:-1, :, :]
    vx = torch.where(ox, vx, torch.zeros_like(vx))
    vy = torch.where(oy, vy, torch.zeros_like(vy))
    vz = torch.where(oz, vz, torch.zeros_like(vz))
    m = max(float(vx.abs().max()), float(vy.abs().max()), float(vz.abs().max()), 1e-30)
    s = vmax / m
    return tuple((v.double() * s).cpu().numpy() for v in (vx, vy, vz))


def stable_dt(dx: float, d: float) -> float:
    """dt = 0.9 * dx^2 / (6 D): the explicit diffusion step used by every workload."""
    return 0.9 * dx * dx / (6.0 * d)
