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




# ---------------------------------------------------------------------------
# The closure applied to a solve: fine cases, training pairs, training, rollout
# ---------------------------------------------------------------------------

class Case:
    """A seeded fine KSPACE problem: geometry, flow, a PGSE waveform with its
    180-degree pulse, physics parameters; M_xy = 1 on pore voxels at t = 0."""

    def __init__(self, mask, vel, wave, pulses, kw):
        self.mask, self.vel, self.wave, self.pulses, self.kw = mask, vel, np.asarray(wave), list(pulses), dict(kw)
        self.shape = mask.shape

    @classmethod
    def pgse(cls, shape, seed, kind="sphere", g_amp=0.1, n_coarse=88, axis=(0.0, 0.0, 1.0), device="cpu"):
        """delta = 2 ms, Delta = 20 ms, D = 2.3e-9, rho = 10 um/s, flow up to
        1 mm/s, dx = 1 um; 'sphere' = overlapping spheres (r = 6, 35% solid),
        'grf' = thresholded Gaussian random field (sigma = 3, porosity 0.4)."""
        import math

        from . import GAMMA_PROTON, geometry, kspace_waveform_pgse
        if kind == "sphere":
            mask = geometry.sphere_pack(shape, 6.0, 0.35, seed=seed, device=device)
        elif kind == "grf":
            mask = geometry.gaussian_random_field(shape, 3.0, 0.4, seed=seed, device=device)
        else:
            raise ValueError(kind)
        vel = geometry.curl_velocity(mask, 3.0, 1.0e-3, seed=seed + 1, device=device)
        dt = geometry.stable_dt(1e-6, 2.3e-9)
        n_fine = 4 * n_coarse
        wave = kspace_waveform_pgse(n_fine, dt, g_amp, 2e-3, 20e-3, axis=axis)
        s_rf = 4 * int(math.ceil(10e-3 / dt / 4)) - 1
        kw = dict(dx=1e-6, dt=dt, d_pore=2.3e-9, t1=2.5, t2=2.0, rho1=1e-5, rho2=1e-5, p_eq=1.0, velocity=1,
                  diffusion=1, gamma=GAMMA_PROTON)
        return cls(mask, vel, wave, [(s_rf, 2, math.pi, (1.0, 0.0, 0.0))], kw)

    def k_at(self, step):
        from .coarse import kvec
        return kvec(self.wave, self.kw["gamma"], self.kw["dt"], step)

    def solver(self, precision=None, state=True):
        """A fine handle with geometry, schedule and (state=True) the initial field."""
        from . import BT_F32, BT_SCHEME_KSPACE, Solver, make_config
        s = Solver(make_config(self.shape, precision=BT_F32 if precision is None else precision,
                               scheme=BT_SCHEME_KSPACE, **self.kw))
        s.upload_geometry(self.mask, self.vel)
        s.set_schedule(self.pulses, grad_wave=self.wave)
        if state:
            st0 = np.zeros((3,) + self.shape)
            st0[0] = self.mask
            s.set_state(st0)
        return s

    def reference_mt(self, n_coarse, precision=None):
        """M(t) of the fine solve (FP64 unless given) after every 4th fine step."""
        from . import BT_F64
        s = self.solver(BT_F64 if precision is None else precision)
        mt = s.run(4 * n_coarse)[3::4]
        s.close()
        return mt


class CoarseCase:
    """The factor-2 coarse counterpart of a Case: 2 dx, 4 dt, coarsened
    geometry, step-averaged waveform, pulses moved to coarse steps; plus the
    closure's static input channels on the coarse grid."""

    def __init__(self, case: Case, n_coarse, device="cuda", pore_average=False):
        import torch

        from . import coarse as cg
        self.case, self.n = case, n_coarse
        # pore_average: a coarse cell holds the mean over its fine pore voxels
        # (a uniform pore field stays uniform on the coarse grid); M(t) then
        # weights each cell by its porosity. Otherwise the mean over all 8.
        self.pore_average = pore_average
        self.mask, self.phi, self.vel = cg.coarsen_geometry(case.mask, case.vel)
        self.shape = self.mask.shape
        self.wave = cg.coarse_waveform(case.wave, n_coarse)
        self.pulses = cg.coarse_pulses(case.pulses)
        self.kw = dict(case.kw)
        self.kw["dx"] = 2 * case.kw["dx"]
        self.kw["dt"] = 4 * case.kw["dt"]
        self.dxf = (case.kw["dx"],) * 3
        c = self.kw["dt"] / self.kw["dx"]
        vx, vy, vz = self.vel
        u = 0.5 * (vx[:, :, 1:] + vx[:, :, :-1]) * c
        v = 0.5 * (vy[:, 1:, :] + vy[:, :-1, :]) * c
        w = 0.5 * (vz[1:] + vz[:-1]) * c
        self.static = torch.as_tensor(np.stack([self.phi, u, v, w], axis=-1), dtype=torch.float32, device=device)
        self.pore = torch.as_tensor(self.mask, dtype=torch.float32, device=device)
        self.device = device

    def solver(self):
        from . import BT_F32, BT_SCHEME_KSPACE, Solver, make_config
        s = Solver(make_config(self.shape, precision=BT_F32, scheme=BT_SCHEME_KSPACE, **self.kw))
        s.upload_geometry(self.mask, self.vel)
        s.set_schedule(self.pulses, grad_wave=self.wave)
        return s

    def initial(self):
        """The restriction of the fine initial field (M_x = 1 in pore)."""
        st = np.zeros((3,) + self.shape)
        st[0] = self.mask if self.pore_average else self.phi
        return st

    def restrict(self, field, fine_step):
        from . import coarse as cg
        return cg.restrict(field, self.case.k_at(fine_step), self.dxf,
                           self.case.mask if self.pore_average else None)

    def prolong(self, field, fine_step):
        from . import coarse as cg
        return cg.prolong(field, self.case.k_at(fine_step), self.dxf, self.case.mask, self.pore_average)

    def mt(self, solver, n_done):
        """Lab-frame M(t) of a coarse handle after n_done coarse steps, in fine units."""
        from . import coarse as cg
        from .coarse import kvec
        k = kvec(self.wave, self.kw["gamma"], self.kw["dt"], n_done)
        w = self.phi if self.pore_average else None
        return 8.0 * cg.lab_sums(solver.field_views(), k, (self.kw["dx"],) * 3, w)

    def kfeat(self, n):
        """k x dx_c at the start and at the end of coarse step n (6 numbers):
        the k-frame discretization error of the step depends on them."""
        from .coarse import kvec
        g, dt = self.kw["gamma"], self.kw["dt"]
        k0 = kvec(self.wave, g, dt, n)
        k1 = k0 + g * self.wave[min(n, len(self.wave) - 1)] * dt
        return np.concatenate([k0, k1]) * self.kw["dx"]

    def features(self, field, n):
        """field: 3 coarse tensors after coarse step n -> (nz, ny, nx, 13)
        network input: field, porosity, velocity (cells per step), k x dx_c."""
        import torch
        kf = torch.as_tensor(self.kfeat(n), dtype=torch.float32, device=self.device)
        kb = kf.expand(tuple(self.shape) + (6,))
        return torch.cat([torch.stack([f.float() for f in field], dim=-1), self.static, kb], dim=-1)


def _write_views(solver, field):
    """Copy three tensors into a handle's field, ordered on the handle's stream."""
    import torch
    hs = solver.torch_stream()
    hs.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(hs):
        for v, f in zip(solver.field_views(), field):
            v.copy_(f)
    hs.synchronize()  # the sources may be freed once this returns


def make_pairs(cc: CoarseCase):
    """Training pairs from the fine solver's own trajectory: for each coarse
    step n, the restriction of the fine field at fine step 4n is advanced one
    coarse step (pred) and compared with the restriction at fine step 4n + 4
    (target). Returns a list of (pred (Z,Y,X,3), residual target (Z,Y,X,3), n)."""
    import torch

    case = cc.case
    fine = case.solver()
    crs = cc.solver()
    crs.set_state(np.zeros((3,) + cc.shape))
    pairs = []
    src = cc.restrict(fine.field_views(), 0)
    for n in range(cc.n):
        crs.set_step(n)
        _write_views(crs, src)
        crs.run(1)
        pred = torch.stack([v.clone() for v in crs.field_views()], dim=-1)
        fine.run(4)
        src = cc.restrict(fine.field_views(), 4 * n + 4)
        torch.cuda.synchronize()
        tgt = torch.stack(src, dim=-1)
        pairs.append((pred, (tgt - pred) * cc.pore[..., None], n))
    fine.close()
    crs.close()
    return pairs


def _head(y, m, sg, sh):
    """Net output (..., 16) and coarse field (..., 3) -> correction (..., 3):
    a complex gain on M_xy (channels 0, 1), a gain and an offset on M_z
    (channels 2, 3). The update is linear in M, so is the correction."""
    import torch
    t = torch.tanh(y[..., :4])  # bounded: |gain| <= sg per step, so a rollout cannot blow up
    gr, gi, gz, hz = t[..., 0] * sg, t[..., 1] * sg, t[..., 2] * sg, t[..., 3] * sh
    return torch.stack([gr * m[..., 0] - gi * m[..., 1], gr * m[..., 1] + gi * m[..., 0], gz * m[..., 2] + hz], -1)


def _global_gain(y, pore, sg):
    """Net output (B, ..., 16) -> one complex gain per sample: sg times the
    mean over pore voxels of channels 0 + i 1."""
    p = pore[..., 0] if pore.dim() == y.dim() else pore
    dims = tuple(range(1, y.dim() - 1))
    n = p.sum(dim=dims).clamp(min=1.0)
    gr = (y[..., 0] * p).sum(dim=dims) / n * sg
    gi = (y[..., 1] * p).sum(dim=dims) / n * sg
    return gr, gi


def make_rollout_pairs(cc: CoarseCase):
    """Trajectory targets for the global head: along a plain coarse rollout,
    the field after each step n (what the net sees in a rollout) and the
    lab-frame sums M (after the step) and R = (fine increment of M(t) over the
    step) - (coarse increment): the per-step rate error of the rollout itself.
    A one-step target from a restricted fine state instead carries that
    state's projection residual, which a self-consistent rollout pays once,
    not every step."""
    import torch
    case = cc.case
    mf = case.reference_mt(cc.n, precision=0)  # fine M(t) after fine steps 4, 8, ...
    crs = cc.solver()
    crs.set_state(cc.initial())
    prev_c = cc.mt(crs, 0)
    prev_f = prev_c.copy()  # the restriction keeps the lab-frame sums
    # steps at and next to an RF pulse: both increments are large and their
    # difference is dominated by where within the step the pulse acts; they
    # are left out of the targets
    near_pulse = {p[0] + o for p in cc.pulses for o in (-1, 0, 1)}
    pairs = []
    for n in range(cc.n):
        crs.run(1)
        mc = cc.mt(crs, n + 1)
        r = (mf[n] - prev_f) - (mc - prev_c)
        if n not in near_pulse:
            pred = torch.stack([v.clone() for v in crs.field_views()], dim=-1)
            pairs.append((pred, None, n, (mc[0], mc[1], r[0], r[1])))
        prev_c, prev_f = mc, mf[n]
    torch.cuda.synchronize()
    crs.close()
    return pairs


class Closure:
    """The trained net and the scales of its head. head "voxel": `apply` adds
    a per-voxel correction (complex gain on M_xy, gain and offset on M_z) on
    coarse pore voxels. head "global": the net's gain channels are averaged
    over the pore voxels into one complex gain per step that multiplies the
    whole transverse field (a correction of the step's decay and phase rate,
    with no per-voxel structure)."""

    def __init__(self, net: Net, sg=1.0, sh=1.0, head="voxel"):
        self.net, self.sg, self.sh, self.head = net, float(sg), float(sh), head
        self._lay = None

    def apply(self, solver, cc: CoarseCase, n):
        import torch
        with torch.cuda.stream(solver.torch_stream()):
            views = solver.field_views()
            if self._lay is None or (self._lay.nz, self._lay.ny, self._lay.nx) != cc.shape:
                self._lay = PaddedRows(1, *cc.shape)
            m = torch.stack([v.float() for v in views], dim=-1)
            x = self._lay.pack(cc.features(views, n)[None], self.net.device)
            y = self._lay.unpack(self.net.forward(self._lay, x), fp32_rows=True)[0]
            if self.head == "global":
                gr, gi = _global_gain(y[None], cc.pore[None], self.sg)
                mr, mi = m[..., 0].clone(), m[..., 1].clone()
                views[0].add_(gr[0] * mr - gi[0] * mi)
                views[1].add_(gr[0] * mi + gi[0] * mr)
                return
            dm = _head(y, m, self.sg, self.sh) * cc.pore[..., None]
            for c in range(3):
                views[c].add_(dm[..., c])


def _pair_sums(cc: CoarseCase, pair):
    """Lab-frame transverse sums of a pair: M of the predicted field and R of
    the residual target (a global gain g closes the step when g M = R)."""
    from . import coarse as cg
    pred, res, n = pair
    k = cg.kvec(cc.wave, cc.kw["gamma"], cc.kw["dt"], n + 1)
    d = (cc.kw["dx"],) * 3
    w = cc.phi if cc.pore_average else None
    R = cg.lab_sums([res[..., c] for c in range(3)], k, d, w)
    M = cg.lab_sums([pred[..., c] for c in range(3)], k, d, w)
    return M[0], M[1], R[0], R[1]


def _train_global(samples, allp, iters, batch, lr, lr_end, rng, net, log_every):
    """Training of the global head (see train)."""
    import math

    import torch
    shape = samples[0][0].shape
    lay = PaddedRows(batch, *shape)
    dy = torch.zeros((lay.rows, CH), dtype=torch.float32, device=net.device)
    dyv = dy.view(batch, shape[0] + 2, shape[1] + 2, shape[2] + 2, CH)
    losses = []
    sh = 1.0
    # per pair the lab-frame sums M (prediction) and R (residual); the loss
    # |g M - R|^2 stays well conditioned where the signal is dephased
    # (M near 0), unlike a fit of g to R / M
    mr = torch.tensor([p[3] if len(p) > 3 else _pair_sums(cc, p) for cc, p in allp], dtype=torch.float64,
                      device=net.device)
    rms_m = float(mr[:, :2].pow(2).sum(dim=1).mean().sqrt()) or 1.0
    rms_r = float(mr[:, 2:].pow(2).sum(dim=1).mean().sqrt()) or 1.0
    sgg = rms_r / rms_m
    mr = (mr / torch.tensor([rms_m, rms_m, rms_r, rms_r], dtype=torch.float64, device=net.device)).float()
    for it in range(iters):
        idx = rng.integers(0, len(allp), size=batch)
        x = torch.stack([allp[i][0].features([allp[i][1][0][..., c] for c in range(3)], allp[i][1][2])
                         for i in idx])
        pore = torch.stack([allp[i][0].pore for i in idx])
        y = lay.unpack(net.forward(lay, lay.pack(x, net.device)), fp32_rows=True).detach().requires_grad_(True)
        gr, gi = _global_gain(y, pore, 1.0)  # g / sgg
        t = mr[torch.as_tensor(idx, device=net.device)]
        er = gr * t[:, 0] - gi * t[:, 1] - t[:, 2]
        ei = gr * t[:, 1] + gi * t[:, 0] - t[:, 3]
        loss = (er ** 2 + ei ** 2).mean()
        loss.backward()
        losses.append(float(loss.detach()))
        if log_every and it % log_every == 0:
            print(f"closure train {it}: loss {float(loss.detach()):.4e}", flush=True)
        dyv[:, 1:-1, 1:-1, 1:-1, :] = y.grad
        net.backward(lay, dy)
        net.adamw(lr=lr_end + 0.5 * (lr - lr_end) * (1 + math.cos(math.pi * it / max(1, iters))))
    net.check_status()
    return Closure(net, sgg, sh, head="global"), losses


def train(samples, iters, batch=8, lr=2e-3, lr_end=1e-4, seed=0, net=None, vox_weight=1.0, sum_weight=0.1,
          log_every=0, head="voxel"):
    """AdamW on the closure net over the pairs of several coarse cases
    (samples: list of (CoarseCase, pairs)). Loss, in units of the targets'
    RMS sigma: vox_weight x the mean squared correction error over pore
    voxels, plus sum_weight x the squared per-sample sum of that error over
    the voxels divided by the voxel count (the part M(t) sees). Cosine learning rate
    from lr to lr_end. Returns the Closure and the loss history."""
    import math

    import torch
    rng = np.random.default_rng(seed)
    allp = [(cc, p) for cc, ps in samples for p in ps]
    if head == "global":
        return _train_global(samples, allp, iters, batch, lr, lr_end, rng, net or Net(seed=seed), log_every)
    res2 = torch.stack([(r[..., :2] ** 2).sum() for _, (_, r, _) in allp]).sum()
    m2 = torch.stack([(p[..., :2] ** 2).sum() for _, (p, _, _) in allp]).sum()
    npore = sum(float(cc.pore.sum()) for cc, _ in allp)
    sigma = float(torch.sqrt(torch.stack([(r ** 2).mean() for _, (_, r, _) in allp]).mean())) or 1.0
    sg = float(torch.sqrt(res2 / m2)) or 1.0
    sh = float(torch.sqrt(torch.stack([(r[..., 2] ** 2).sum() for _, (_, r, _) in allp]).sum() / npore)) or sigma
    net = net or Net(seed=seed)
    shape = samples[0][0].shape
    lay = PaddedRows(batch, *shape)
    dy = torch.zeros((lay.rows, CH), dtype=torch.float32, device=net.device)
    dyv = dy.view(batch, shape[0] + 2, shape[1] + 2, shape[2] + 2, CH)
    losses = []
    for it in range(iters):
        idx = rng.integers(0, len(allp), size=batch)
        m = torch.stack([allp[i][1][0] for i in idx])
        x = torch.stack([allp[i][0].features([allp[i][1][0][..., c] for c in range(3)], allp[i][1][2]) for i in idx])
        t = torch.stack([allp[i][1][1] for i in idx]) / sigma
        pore = torch.stack([allp[i][0].pore for i in idx])[..., None]
        y = lay.unpack(net.forward(lay, lay.pack(x, net.device)), fp32_rows=True).detach().requires_grad_(True)
        e = (_head(y, m, sg, sh) / sigma - t) * pore
        n = float(pore.sum())
        loss = vox_weight * (e ** 2).sum() / (3 * n) + sum_weight * (e.sum(dim=(1, 2, 3)) ** 2).sum() / (3 * n)
        loss.backward()
        losses.append(float(loss.detach()))
        if log_every and it % log_every == 0:
            print(f"closure train {it}: loss {float(loss.detach()):.4e}", flush=True)
        dyv[:, 1:-1, 1:-1, 1:-1, :] = y.grad
        net.backward(lay, dy)
        net.adamw(lr=lr_end + 0.5 * (lr - lr_end) * (1 + math.cos(math.pi * it / max(1, iters))))
    net.check_status()
    return Closure(net, sg, sh), losses


def rollout(cc: CoarseCase, closure: Closure = None, check_every=0, check_tol=2e-4):
    """Coarse solve of cc (corrected by the closure when given) from the
    restricted initial field. Returns (M(t) after each coarse step, x8 so it
    compares with the fine sums; the coarse step at which a periodic fine
    check fell back to the fine solver, or None).

    The check (every check_every coarse steps): the field is prolonged to the
    fine grid and advanced 4 fine steps; when the change of the lab-frame sums
    over the corrected coarse step differs from that of the 4 fine steps by
    more than check_tol x |M|, the run continues on the fine solver from there."""
    case = cc.case
    crs = cc.solver()
    crs.set_state(cc.initial())
    mt = np.zeros((cc.n, 3))
    fell_back, fine = None, None
    for n in range(cc.n):
        if fine is not None:
            mt[n] = fine.run(4)[-1]
            continue
        check = None
        if closure is not None and check_every and n > 0 and n % check_every == 0:
            check = case.solver(state=False)
            check.set_step(4 * n)
            _write_views(check, cc.prolong(crs.field_views(), 4 * n))
            before = check.measure()
            after_f = check.run(4)[-1]
        crs.run(1)
        if closure is not None:
            closure.apply(crs, cc, n)
        mt[n] = cc.mt(crs, n + 1)
        if check is not None:
            d = np.abs((mt[n] - before) - (after_f - before)).max()
            if d > check_tol * max(np.abs(before).max(), 1e-300):
                fell_back, fine = n, check
                mt[n] = after_f
                continue
            check.close()
    crs.close()
    if fine is not None:
        fine.close()
    return mt, fell_back


def mt_error(mt, ref):
    """max over t of |M_xy(t) - M_xy,ref(t)| / |M_xy,ref(0)| (lab frame)."""
    a = mt[:, 0] + 1j * mt[:, 1]
    b = ref[:, 0] + 1j * ref[:, 1]
    return float(np.max(np.abs(a - b)) / max(abs(b[0]), 1e-300))


def evaluate(shape=(64, 64, 64), n_coarse=88, n_train=8, iters=1500, g_test=0.2, seed=5, vox_weight=1.0,
             sum_weight=0.1, pore_average=False, head="voxel", targets="step", log=print):
    """The closure experiment: training pairs from n_train seeded fine PGSE
    cases (alternating sphere packs and Gaussian random fields, G uniform in
    0..0.3 T/m), training, then on two held-out cases (sphere, GRF) the M(t)
    error against the FP64 fine solve of the FP32 fine solve, the plain coarse
    solve and the corrected coarse solve (with and without the periodic fine
    check), and the time per coarse step of each. Returns a dict."""
    import time

    import torch
    t0 = time.time()
    rng = np.random.default_rng(seed)
    samples = []
    for i in range(n_train):
        kind = "sphere" if i % 2 == 0 else "grf"
        case = Case.pgse(shape, seed=100 + 7 * i, kind=kind, g_amp=float(rng.uniform(0, 0.3)), n_coarse=n_coarse,
                         device="cuda")
        cc = CoarseCase(case, n_coarse, pore_average=pore_average)
        samples.append((cc, make_rollout_pairs(cc) if targets == "rollout" else make_pairs(cc)))
    t_pairs = time.time() - t0
    t0 = time.time()
    clo, losses = train(samples, iters, vox_weight=vox_weight, sum_weight=sum_weight, head=head,
                        lr=5e-4 if head == "global" else 2e-3)
    torch.cuda.synchronize()
    t_train = time.time() - t0
    out = {"shape": list(shape), "coarse_steps": n_coarse, "train_cases": n_train, "iters": iters, "head": head, "targets": targets,
           "pairs_s": t_pairs, "train_s": t_train, "loss_first": losses[0],
           "loss_last": float(np.mean(losses[-50:])), "held_out": []}
    for kind, s in (("sphere", 900), ("grf", 901)):
        case = Case.pgse(shape, seed=s, kind=kind, g_amp=g_test, n_coarse=n_coarse, device="cuda")
        cc = CoarseCase(case, n_coarse, pore_average=pore_average)
        ref = case.reference_mt(n_coarse)
        t0 = time.time()
        f32 = case.reference_mt(n_coarse, precision=0)
        t_fine = time.time() - t0
        t0 = time.time()
        plain, _ = rollout(cc)
        t_plain = time.time() - t0
        t0 = time.time()
        corr, _ = rollout(cc, clo)
        t_corr = time.time() - t0
        chk, fb = rollout(cc, clo, check_every=22)
        row = {"case": kind, "G": g_test, "err_fine_f32": mt_error(f32, ref), "err_plain": mt_error(plain, ref),
               "err_closure": mt_error(corr, ref), "err_checked": mt_error(chk, ref), "fell_back_at": fb,
               "ms_per_coarse_step": {"fine_x4": 1e3 * t_fine / n_coarse, "plain": 1e3 * t_plain / n_coarse,
                                      "closure": 1e3 * t_corr / n_coarse}}
        out["held_out"].append(row)
        log(row)
    return out


if __name__ == "__main__":
    import argparse
    import json
    ap = argparse.ArgumentParser(description="train and evaluate the learned closure on seeded PGSE cases")
    ap.add_argument("--edge", type=int, default=64)
    ap.add_argument("--coarse-steps", type=int, default=88)
    ap.add_argument("--train-cases", type=int, default=8)
    ap.add_argument("--iters", type=int, default=1500)
    ap.add_argument("--pore-average", action="store_true")
    ap.add_argument("--head", default="voxel", choices=["voxel", "global"])
    ap.add_argument("--targets", default="step", choices=["step", "rollout"],
                    help="one-step targets from restricted fine states, or trajectory targets (global head)")
    a = ap.parse_args()
    res = evaluate((a.edge,) * 3, a.coarse_steps, a.train_cases, a.iters, pore_average=a.pore_average,
                   head=a.head, targets=a.targets)
    print(json.dumps(res))
