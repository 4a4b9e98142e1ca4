"""Factor-2 coarse grid for the learned closure: coarse geometry, and the
restriction / prolongation of a KSPACE field between the fine and the coarse
grid.

A KSPACE field stores the transverse magnetization in the frame of the wave
vector k of its step: m(r) = exp(+i k.r) M_lab(r), with r the voxel centre
((i + 0.5) dx, ...), the same convention as the solver's lab-frame M(t). The
coarse field holds fine-cell averages, so (coarse sums) x 8 = (fine sums) in
the lab frame, exactly, when a coarse field is the restriction of a fine one.

Pure torch / numpy: everything here runs on the CPU as well as on the GPU.
"""
from __future__ import annotations

import itertools

import numpy as np


def coarsen_geometry(mask, vel):
    """(mask [nz][ny][nx], face velocities) -> (coarse mask, porosity, coarse
    face velocities). A coarse voxel is pore when any of its 8 fine voxels is
    (no magnetization is dropped); its porosity is the pore fraction; a coarse
    face velocity is the mean of the 4 fine faces it covers (the flux through
    the coarse face is kept)."""
    nz, ny, nx = mask.shape
    if nz % 2 or ny % 2 or nx % 2:
        raise ValueError("coarsening needs even grid sizes")
    m = np.asarray(mask, dtype=np.float64).reshape(nz // 2, 2, ny // 2, 2, nx // 2, 2)
    phi = m.mean(axis=(1, 3, 5))
    mask_c = (phi > 0).astype(np.uint8)
    if vel is None:
        vel = (np.zeros((nz, ny, nx + 1)), np.zeros((nz, ny + 1, nx)), np.zeros((nz + 1, ny, nx)))
    vx, vy, vz = (np.asarray(v, dtype=np.float64) for v in vel)
    vxc = vx[:, :, ::2].reshape(nz // 2, 2, ny // 2, 2, nx // 2 + 1).mean(axis=(1, 3))
    vyc = vy[:, ::2, :].reshape(nz // 2, 2, ny // 2 + 1, nx // 2, 2).mean(axis=(1, 4))
    vzc = vz[::2, :, :].reshape(nz // 2 + 1, ny // 2, 2, nx // 2, 2).mean(axis=(2, 4))
    return mask_c, phi, tuple(np.ascontiguousarray(v) for v in (vxc, vyc, vzc))


def sub_phases(k, dxf):
    """exp(-i k.(r_f - r_c)) for the 8 fine cells of a coarse cell, as a
    (2, 2, 2, 2) array [dz][dy][dx][re, im]; r_f - r_c = (d - 1/2) * dx_f per axis."""
    out = np.zeros((2, 2, 2, 2))
    for a, b, c in itertools.product(range(2), range(2), range(2)):
        ang = k[0] * (c - 0.5) * dxf[0] + k[1] * (b - 0.5) * dxf[1] + k[2] * (a - 0.5) * dxf[2]
        out[a, b, c] = (np.cos(ang), -np.sin(ang))
    return out


def _blocks(t):
    nz, ny, nx = t.shape[-3:]
    lead = t.shape[:-3]
    v = t.reshape(lead + (nz // 2, 2, ny // 2, 2, nx // 2, 2))
    n = len(lead)
    return v.permute(*range(n), n, n + 2, n + 4, n + 1, n + 3, n + 5)  # [..., Z, Y, X, dz, dy, dx]


def restrict(f, k, dxf, mask_f=None):
    """Fine field (three tensors [..., nz, ny, nx]: Re, Im in the frame of k,
    and Mz) -> coarse field in the same frame: the mean of the 8 fine cells'
    lab-frame values, re-expressed at the coarse cell centre. With mask_f the
    mean is over the cell's fine pore voxels instead (the pore average; zero
    where a coarse cell holds no pore)."""
    import torch
    ph = torch.as_tensor(sub_phases(k, dxf), dtype=f[0].dtype, device=f[0].device)
    cr, ci = ph[..., 0], ph[..., 1]
    mr, mi = _blocks(f[0]), _blocks(f[1])
    re = (cr * mr - ci * mi).mean(dim=(-3, -2, -1))
    im = (cr * mi + ci * mr).mean(dim=(-3, -2, -1))
    mz = _blocks(f[2]).mean(dim=(-3, -2, -1))
    out = [re, im, mz]
    if mask_f is not None:
        mk = torch.as_tensor(np.asarray(mask_f), device=f[0].device).to(f[0].dtype)
        npore = _blocks(mk).sum(dim=(-3, -2, -1))
        scale = torch.where(npore > 0, 8.0 / npore.clamp(min=1), torch.zeros_like(npore))
        out = [t * scale for t in out]
    return [t.contiguous() for t in out]


def prolong(c, k, dxf, mask_f, pore_average=False):
    """Coarse field -> fine field: each coarse value (a cell average, divided
    by the pore fraction of its cell; or, with pore_average, a pore average as
    it is) is copied into the cell's fine pore voxels with the restriction's
    phase undone; fine solid voxels get 0. restrict(prolong(c)) == c on every
    coarse cell that holds pore (with the same pore_average / mask_f choice)."""
    import torch
    ph = torch.as_tensor(sub_phases(k, dxf), dtype=c[0].dtype, device=c[0].device)
    cr, ci = ph[..., 0], -ph[..., 1]
    Z, Y, X = c[0].shape
    mk = torch.as_tensor(np.asarray(mask_f), device=c[0].device).to(c[0].dtype)
    if not pore_average:
        npore = _blocks(mk).sum(dim=(-3, -2, -1))
        scale = torch.where(npore > 0, 8.0 / npore.clamp(min=1), torch.zeros_like(npore))
        c = [t * scale for t in c]

    def spread(t):
        return t[:, :, :, None, None, None].expand(Z, Y, X, 2, 2, 2)

    def unblock(t):
        return t.permute(0, 3, 1, 4, 2, 5).reshape(2 * Z, 2 * Y, 2 * X)

    re_c, im_c = spread(c[0]), spread(c[1])
    re = cr * re_c - ci * im_c
    im = cr * im_c + ci * re_c
    return [unblock(re) * mk, unblock(im) * mk, unblock(spread(c[2])) * mk]


def coarse_waveform(wave, n_coarse):
    """Per-step gradients of the fine solve -> per coarse step (4 fine steps):
    the mean, so that the coarse k after n steps equals the fine k after 4n."""
    w = np.asarray(wave, dtype=np.float64)[:4 * n_coarse]
    return w.reshape(n_coarse, 4, 3).mean(axis=1)


def coarse_pulses(pulses):
    """RF pulses of the fine solve -> the coarse solve. A pulse applied after
    fine step s lands after coarse step (s - 3) / 4, which needs s = 3 mod 4."""
    out = []
    for step, flag, param, axis in pulses:
        if step % 4 != 3:
            raise ValueError(f"fine pulse step {step} is not at the end of a coarse step (3 mod 4)")
        out.append(((step - 3) // 4, flag, param, axis))
    return out


def kvec(wave, gamma, dt, n):
    """KSPACE wave vector after n steps of a waveform, accumulated in FP64 in
    the solver's order (k += gamma * g * dt per step)."""
    k = np.zeros(3)
    w = np.asarray(wave, dtype=np.float64)
    for s in range(n):
        k = k + gamma * w[s] * dt
    return k


def lab_sums(field, k, d, weight=None):
    """Lab-frame sums of a KSPACE field (three tensors [nz][ny][nx]) whose
    transverse part is in the frame of k: sum of w * exp(-i k.r) m, r the voxel
    centres ((i + 0.5) d); w = 1 or a per-voxel weight. Returns (x, y, z), FP64."""
    import torch
    nz, ny, nx = field[0].shape
    dev = field[0].device
    ax = [torch.exp(-1j * torch.as_tensor(k[a] * (np.arange(n) + 0.5) * d[a], device=dev))
          for a, n in ((0, nx), (1, ny), (2, nz))]
    ph = ax[2][:, None, None] * ax[1][None, :, None] * ax[0][None, None, :]
    m = field[0].double() + 1j * field[1].double()
    w = 1.0 if weight is None else torch.as_tensor(weight, device=dev, dtype=torch.float64)
    s = (w * ph * m).sum()
    return np.array([float(s.real), float(s.imag), float((w * field[2].double()).sum())])
