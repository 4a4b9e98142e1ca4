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


class Net:
    """4 conv layers, 16 -> 16 channels, GELU after the first three. FP32
    master parameters in one flat buffer (for AdamW), packed BF16 copies for
    the kernels. The last layer starts at zero, so an untrained net leaves the
    coarse solve unchanged."""

    NW = 4 * TAPS * CH * CH
    NP = NW + 4 * CH

    def __init__(self, device="cuda", seed=0, scale=1.0, zero_last=True):
        import torch
        g = torch.Generator(device="cpu").manual_seed(seed)
        self.device = device
        self.flat = torch.zeros(self.NP, dtype=torch.float32)
        w = self.flat[:self.NW].view(4, TAPS, CH, CH)
        for i in range(4):
            w[i] = torch.randn((TAPS, CH, CH), generator=g) * (scale / np.sqrt(TAPS * CH))
        if zero_last:
            w[3].zero_()
        self.flat = self.flat.to(device)
        self.grad = torch.zeros_like(self.flat)
        self.m = torch.zeros_like(self.flat)
        self.v = torch.zeros_like(self.flat)
        self.step_count = 0
        self.status = torch.zeros(1, dtype=torch.int32, device=device)
        self.repack()

    def w(self, i):
        return self.flat[:self.NW].view(4, TAPS, CH, CH)[i]

    def b(self, i):
        return self.flat[self.NW:].view(4, CH)[i]

    def repack(self):
        self.packed = [pack_weights(self.w(i)) for i in range(4)]

    def forward(self, layout: PaddedRows, x):
        """x: BF16 padded rows -> FP32 output rows (16 channels), with the
        activations and pre-activations kept for backward."""
        import torch
        acts, pres = [x], []
        a = x
        for i in range(3):
            out = layout.empty(self.device)
            pre = torch.empty((layout.rows, CH), dtype=torch.float32, device=self.device)
            conv3d(layout, a, self.packed[i][0], 0, bias=self.b(i), out=out, pre=pre, status=self.status)
            acts.append(out)
            pres.append(pre)
            a = out
        y = torch.empty((layout.rows, CH), dtype=torch.float32, device=self.device)
        conv3d(layout, a, self.packed[3][0], 1, bias=self.b(3), outf=y, status=self.status)
        self._cache = (acts, pres)
        return y

    def backward(self, layout: PaddedRows, dy):
        """dy: FP32 rows (zero on the halo) = dL/dy. Fills self.grad."""
        acts, pres = self._cache
        g = layout.empty(self.device)
        g[layout.margin:layout.margin + layout.rows] = dy.to(g.dtype)
        gw = self.grad[:self.NW].view(4, TAPS, CH, CH)
        gb = self.grad[self.NW:].view(4, CH)
        scratch = None
        for i in range(3, -1, -1):
            gwi, gbi, scratch = weight_grad(layout, acts[i], g, scratch)
            gw[i] = gwi
            gb[i] = gbi
            if i > 0:
                nxt = layout.empty(self.device)
                conv3d(layout, g, self.packed[i][1], 2, out=nxt, pre=pres[i - 1], status=self.status)
                g = nxt

    def adamw(self, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8, weight_decay=0.01):
        import torch
        self.step_count += 1
        rc = lib().bt_adamw(_ptr(self.flat), _ptr(self.grad), _ptr(self.m), _ptr(self.v), self.NP,
                            ctypes.c_float(lr), ctypes.c_float(beta1), ctypes.c_float(beta2), ctypes.c_float(eps),
                            ctypes.c_float(weight_decay), self.step_count,
                            ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        if rc:
            raise BtError(rc, "bt_adamw")
        self.repack()

    def check_status(self):
        if int(self.status.item()) != 0:
            raise BtError(-6, "a bounded wait in the convolution kernel gave up")

    def state_dict(self):
        return {"flat": self.flat.detach().cpu().numpy()}

    def load_state_dict(self, d):
        import torch
        self.flat.copy_(torch.as_tensor(d["flat"], device=self.device))
        self.repack()
