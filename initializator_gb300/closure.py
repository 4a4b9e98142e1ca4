"""Learned closure: a 4-layer 3-D CNN (16 channels, 3x3x3, GELU) that corrects
a 2x-coarse, 4x-time-step solve toward the fine solve. Its convolutions, data
and weight gradients and optimizer run on the library's own kernels
(bt_conv3d on tcgen05 tensor cores, bt_conv3d_weight_grad, bt_adamw); torch
only provides device buffers and streams.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import BtError, Conv3dArgs, lib

CH = 16
TAPS = 27


def _ptr(t):
    return ctypes.c_void_p(0 if t is None else t.data_ptr())


class PaddedRows:
    """Channels-last BF16 rows of a zero-padded grid (see include/bt.h)."""

    def __init__(self, nb, nz, ny, nx):
        self.nb, self.nz, self.ny, self.nx = nb, nz, ny, nx
        self.margin = int(lib().bt_conv3d_margin(nx, ny))
        self.rows = nb * (nz + 2) * (ny + 2) * (nx + 2)
        self.total = self.rows + 2 * self.margin

    def empty(self, device):
        import torch
        return torch.zeros((self.total, CH), dtype=torch.bfloat16, device=device)

    def pack(self, a, device):
        """a: (nb, nz, ny, nx, C<=16) array or tensor -> padded BF16 rows."""
        import torch
        t = torch.as_tensor(a, device=device, dtype=torch.float32)
        full = torch.zeros((self.nb, self.nz + 2, self.ny + 2, self.nx + 2, CH), device=device)
        full[:, 1:-1, 1:-1, 1:-1, :t.shape[-1]] = t
        out = self.empty(device)
        out[self.margin:self.margin + self.rows] = full.reshape(-1, CH).to(torch.bfloat16)
        return out

    def unpack(self, rows, fp32_rows=False):
        """padded rows (BF16 with margins, or FP32 without) -> (nb, nz, ny, nx, 16) float tensor"""
        r = rows if fp32_rows else rows[self.margin:self.margin + self.rows]
        full = r.float().reshape(self.nb, self.nz + 2, self.ny + 2, self.nx + 2, CH)
        return full[:, 1:-1, 1:-1, 1:-1, :]


def conv3d(layout: PaddedRows, x, wpack, mode, bias=None, out=None, pre=None, outf=None, status=None, stream=None):
    import torch
    a = Conv3dArgs()
    a.nb, a.nx, a.ny, a.nz = layout.nb, layout.nx, layout.ny, layout.nz
    a.mode = mode
    a.x, a.wpack = x.data_ptr(), wpack.data_ptr()
    a.bias = 0 if bias is None else bias.data_ptr()
    a.out = 0 if out is None else out.data_ptr()
    a.pre = 0 if pre is None else pre.data_ptr()
    a.outf = 0 if outf is None else outf.data_ptr()
    a.status = 0 if status is None else status.data_ptr()
    s = torch.cuda.current_stream().cuda_stream if stream is None else stream
    rc = lib().bt_conv3d(ctypes.byref(a), ctypes.c_void_p(s))
    if rc:
        raise BtError(rc, "bt_conv3d")


def pack_weights(w):
    """w: (27, 16, 16) FP32 CUDA tensor -> (forward, data-gradient) packed BF16 blocks."""
    import torch
    fwd = torch.zeros(TAPS * 512, dtype=torch.uint8, device=w.device)
    dg = torch.zeros(TAPS * 512, dtype=torch.uint8, device=w.device)
    rc = lib().bt_conv3d_pack_weights(_ptr(w.contiguous()), _ptr(fwd), _ptr(dg),
                                      ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    if rc:
        raise BtError(rc, "bt_conv3d_pack_weights")
    return fwd, dg


def weight_grad(layout: PaddedRows, x, dz, scratch=None):
    import torch
    n = int(lib().bt_conv3d_wgrad_scratch(layout.nb, layout.nx, layout.ny, layout.nz))
    if scratch is None or scratch.numel() < n:
        scratch = torch.empty(n, dtype=torch.float32, device=x.device)
    grad = torch.empty((TAPS + 1, CH, CH), dtype=torch.float32, device=x.device)
    rc = lib().bt_conv3d_weight_grad(_ptr(x), _ptr(dz), layout.nb, layout.nx, layout.ny, layout.nz, _ptr(scratch),
                                     _ptr(grad), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    if rc:
        raise BtError(rc, "bt_conv3d_weight_grad")
    return grad[:TAPS], grad[TAPS, 0], scratch
