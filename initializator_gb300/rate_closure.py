"""Learned coarse relaxation closure.

The plain coarse solve (2 dx, 4 dt, coarse cell pore when any fine voxel is)
loses most of the pore surface, so its surface relaxation is too weak, and
the reference's advective upwind form leaks magnetisation on the averaged
coarse velocities; without a gradient these make its M(t) miss the fine one
by ~1e-2 of |M(0)| at 64^3. Here a 3-D CNN (4 layers of 3x3x3
convolutions, 16 channels, GELU: the library's tcgen05 kernels, BF16
operands, FP32 accumulation) reads a coarse sample's static geometry and flow
once and predicts, per coarse voxel, a correction of its relaxation rate.
The corrected coarse solve then runs on the library's own step kernel with
per-voxel rates (bt_upload_rates): the closure costs one network evaluation
per sample, nothing per step.

Training is a-posteriori, through the coarse rollout itself, against the fine
solver's own M(t), on gradient-free samples (the decay the rate correction
acts on): Gauss-Newton outer iterations run the corrected coarse solve of
every training sample, then inner iterations fit the network to the
rollout's linearised residual. The magnetisation a rate change dr(x) removes
at step m is dt dr(x) M(x, m); carried afterwards at the sum's own relative
rate, it moves the lab-frame sum after step n by
-S(n) sum_{m<=n} dt dr(x) M(x, m) / S(m). The network's parameters get the
gradient of the squared residual through that map, then the library's own
backward kernels and AdamW.

Under a PGSE gradient the coarse geometry adds an error of the other sign
(its pore space, a cell being pore when any fine voxel is, restricts the
diffusion less, so the echo attenuates more: ~1e-2 of |M(0)| at 0.2 T/m at
64^3), which this closure does not correct.
"""
from __future__ import annotations

import numpy as np

from . import closure as C
from . import coarse as cg

N_FEAT = 8


def solid_face_counts(mask):
    """Per voxel, the number of its six face neighbours inside the grid that
    are solid (the faces FillInDiffusinAndTime adds rho/d for); 0 in solid."""
    m = np.asarray(mask).astype(bool)
    s = ~m
    n = np.zeros(m.shape, dtype=np.int32)
    for ax in range(3):
        lo = [slice(None)] * 3
        hi = [slice(None)] * 3
        lo[ax] = slice(1, None)
        hi[ax] = slice(None, -1)
        n[tuple(lo)] += s[tuple(hi)]   # solid at -1 along ax
        n[tuple(hi)] += s[tuple(lo)]   # solid at +1 along ax
    return np.where(m, n, 0)


def _blocks(a):
    nz, ny, nx = a.shape
    return a.reshape(nz // 2, 2, ny // 2, 2, nx // 2, 2)


class RateCase:
    """A fine PGSE case (closure.Case) and its coarse counterpart with the
    closure's static input channels:
      0 pore fraction of the coarse cell
      1 solid faces of the coarse voxel (the plain coarse surface term), / 6
      2 mean solid faces of the cell's fine pore voxels, / 6
      3 coarse pore flag
      4-6 cell-centred coarse velocity, coarse cells per coarse step
      7 its magnitude."""

    def __init__(self, case: C.Case, n_coarse):
        self.case, self.n = case, n_coarse
        self.mask, self.phi, self.vel = cg.coarsen_geometry(case.mask, case.vel)
        self.shape = self.mask.shape
        kw = dict(case.kw)
        kw["dx"], kw["dt"] = 2 * case.kw["dx"], 4 * case.kw["dt"]
        self.kw = kw
        self.dxf = case.kw["dx"]
        self.wave = cg.coarse_waveform(case.wave, n_coarse)
        self.pulses = cg.coarse_pulses(case.pulses)
        self.count_c = solid_face_counts(self.mask).astype(np.float64)
        cf = solid_face_counts(case.mask).astype(np.float64)
        npore = _blocks(case.mask.astype(np.float64)).sum(axis=(1, 3, 5))
        self.count_f = np.where(npore > 0, _blocks(cf).sum(axis=(1, 3, 5)) / np.maximum(npore, 1), 0.0)
        vx, vy, vz = self.vel
        c = kw["dt"] / kw["dx"]
        u = 0.5 * (vx[:, :, :-1] + vx[:, :, 1:]) * c
        v = 0.5 * (vy[:, :-1, :] + vy[:, 1:, :]) * c
        w = 0.5 * (vz[:-1, :, :] + vz[1:, :, :]) * c
        pore = self.mask.astype(np.float64)
        feats = np.stack([self.phi, self.count_c / 6, self.count_f / 6, pore, u, v, w,
                          np.sqrt(u * u + v * v + w * w)], axis=-1).astype(np.float32)
        # in page-locked host memory, so that the network's input copy runs at
        # the copy engine's speed
        import torch
        self.features = torch.from_numpy(feats)
        if torch.cuda.is_available():
            self.features = self.features.pin_memory()
        # the surface rate unit: rho / dx_f per solid face of a fine voxel
        self.unit1 = case.kw["rho1"] / self.dxf
        self.unit2 = case.kw["rho2"] / self.dxf

    def rates(self, corr=None):
        """(t1, t2, diff) per coarse voxel for bt_upload_rates: bulk + plain
        coarse surface rate (rho / dx_c per coarse solid face) + the correction
        corr (in units of rho / dx_f; None = 0), the surface part kept >= 0
        and rounded onto at most 255 levels."""
        kw = self.kw
        r = self.dxf / kw["dx"]  # one coarse solid face, in units of rho / dx_f
        if corr is not None and not isinstance(corr, np.ndarray):
            return self._rates_device(corr, r)
        surf = self.count_c * r
        pore = self.mask > 0
        if corr is not None:
            surf = np.maximum(surf + corr, 0.0)
            # on a grid of r / k (k as large as keeps <= 255 levels up to the
            # sample's largest rate), so that the rates fit the FP32 fast
            # path's rate palette (256 pairs); the plain rates (multiples of
            # r) stay exactly as they are
            hi = float(surf[pore].max()) if pore.any() else 0.0
            k = max(1, int(254.0 * r / hi)) if hi > 0 else 1
            surf = (np.round(surf * (k / r)) / k) * r
        r1 = 1.0 / kw["t1"] + self.unit1 * surf
        r2 = 1.0 / kw["t2"] + self.unit2 * surf
        t1 = np.where(pore, 1.0 / r1, 1e50)
        t2 = np.where(pore, 1.0 / r2, 1e50)
        diff = np.where(pore, kw["d_pore"], 1e-50)
        return t1, t2, diff

    def palette_device(self, corr):
        """The corrected rates of rates() as a rate palette, formed on the GPU:
        the level entries' (t1, t2) (host arrays) and each voxel's level
        (uint8 CUDA tensor), the same per-voxel values as rates(corr)."""
        import torch
        kw = self.kw
        r = self.dxf / kw["dx"]
        dev = corr.device
        if getattr(self, "_dev", None) is None or self._dev[0] != dev:
            self._dev = (dev, torch.as_tensor(self.count_c, device=dev), torch.as_tensor(self.mask > 0, device=dev))
        _, count_c, pore = self._dev
        surf = torch.clamp(count_c * r + corr.double(), min=0.0)
        hi = float(torch.where(pore, surf, torch.zeros_like(surf)).max()) if bool(pore.any()) else 0.0
        k = max(1, int(254.0 * r / hi)) if hi > 0 else 1
        lev = torch.round(surf * (k / r))
        n = int(lev[pore].max()) + 1 if bool(pore.any()) else 1
        idx = torch.where(pore, lev, torch.zeros_like(lev)).to(torch.uint8).contiguous()
        s_e = (np.arange(n, dtype=np.float64) / k) * r
        t1 = 1.0 / (1.0 / kw["t1"] + self.unit1 * s_e)
        t2 = 1.0 / (1.0 / kw["t2"] + self.unit2 * s_e)
        return t1, t2, idx

    def _rates_device(self, corr, r):
        """rates() for a correction already on the GPU (a torch tensor): the
        same FP64 operations there, three host arrays back."""
        import torch
        kw = self.kw
        dev = corr.device
        if getattr(self, "_dev", None) is None or self._dev[0] != dev:
            self._dev = (dev, torch.as_tensor(self.count_c, device=dev), torch.as_tensor(self.mask > 0, device=dev))
        _, count_c, pore = self._dev
        surf = torch.clamp(count_c * r + corr.double(), min=0.0)
        hi = float(torch.where(pore, surf, torch.zeros_like(surf)).max()) if bool(pore.any()) else 0.0
        k = max(1, int(254.0 * r / hi)) if hi > 0 else 1
        surf = (torch.round(surf * (k / r)) / k) * r
        r1 = 1.0 / kw["t1"] + self.unit1 * surf
        r2 = 1.0 / kw["t2"] + self.unit2 * surf
        big = torch.full_like(surf, 1e50)
        t1 = torch.where(pore, 1.0 / r1, big)
        t2 = torch.where(pore, 1.0 / r2, big)
        diff = torch.where(pore, torch.full_like(surf, kw["d_pore"]), torch.full_like(surf, 1e-50))
        return t1.cpu().numpy(), t2.cpu().numpy(), diff.cpu().numpy()

    def initial(self):
        st = np.zeros((3,) + self.shape)
        st[0] = self.phi
        return st

    def solver(self, corr=None):
        """A coarse handle with the (corrected) rates and the initial field."""
        from . import BT_F32, BT_SCHEME_KSPACE, Solver, make_config
        s = Solver(make_config(self.shape, precision=BT_F32, scheme=BT_SCHEME_KSPACE, **self.kw))
        s.upload_geometry(self.mask, self.vel)
        on_device = corr is not None and not isinstance(corr, np.ndarray)
        if on_device:
            s.upload_rate_palette(*self.palette_device(corr))  # the same rates, formed on the GPU
        else:
            s.upload_rates(*self.rates(corr))
        s.set_schedule(self.pulses, grad_wave=self.wave)
        if on_device:
            # the same FP32 initial field, formed on the GPU
            import torch
            mx = torch.as_tensor(self.phi, dtype=torch.float32, device=corr.device).contiguous()
            s.set_state_device([mx, torch.zeros_like(mx), torch.zeros_like(mx)])
        else:
            s.set_state(self.initial())
        return s

    def lab_field(self, solver, n_done):
        """The coarse transverse field after n_done steps in the lab frame,
        complex (Z, Y, X) torch tensor (fine units: x 8)."""
        import torch
        k = cg.kvec(self.wave, self.kw["gamma"], self.kw["dt"], n_done)
        v = solver.field_views()
        nz, ny, nx = self.shape
        d = self.kw["dx"]
        dev = v[0].device
        ph = [torch.exp(-1j * torch.as_tensor(k[a] * (np.arange(n) + 0.5) * d, device=dev))
              for a, n in ((0, nx), (1, ny), (2, nz))]
        e = ph[2][:, None, None] * ph[1][None, :, None] * ph[0][None, None, :]
        return 8.0 * e * (v[0].double() + 1j * v[1].double())

    def rollout(self, corr=None, checkpoints=()):
        """The (corrected) coarse solve: M(t) after every coarse step (x 8, fine
        units) and, for each checkpoint step n, the sensitivity of the lab-frame
        transverse sum after step n to the correction (see sensitivity)."""
        s = self.solver(corr)
        mt = np.zeros((self.n, 3))
        sens = {}
        if not checkpoints:
            mt[:] = 8.0 * s.run(self.n)
            s.close()
            return mt, sens
        acc = None
        dt = self.kw["dt"]
        for m in range(self.n):
            mt[m] = 8.0 * s.run(1)[0]
            sm = complex(mt[m, 0], mt[m, 1])
            f = self.lab_field(s, m + 1)
            # magnetisation removed at step m by a rate change at x, carried
            # afterwards at the sum's own relative rate
            term = (dt * self.unit2 / sm) * f if abs(sm) > 0 else 0.0 * f
            acc = term if acc is None else acc + term
            if (m + 1) in checkpoints:
                sens[m + 1] = -sm * acc
        s.close()
        return mt, sens


class RateClosure:
    """The trained network and how it maps a sample to its rate correction."""

    def __init__(self, net: C.Net, scale=1.0):
        self.net, self.scale = net, float(scale)

    def save(self, path):
        np.savez(path, flat=self.net.flat.detach().cpu().numpy(), scale=np.array(self.scale))

    @classmethod
    def load(cls, path, device="cuda"):
        z = np.load(path)
        net = C.Net(device=device, zero_last=True)
        net.load_state_dict({"flat": z["flat"]})
        return cls(net, float(z["scale"]))

    def predict(self, rcs):
        """Corrections (units of rho / dx_f) for samples of one coarse shape:
        (nb, Z, Y, X) torch tensor, zero outside the pore."""
        import torch
        lay = C.PaddedRows(len(rcs), *rcs[0].shape)
        feats = [r.features for r in rcs]
        x = lay.pack(feats[0].unsqueeze(0) if len(feats) == 1 else torch.stack(feats), self.net.device)
        y = lay.unpack(self.net.forward(lay, x), fp32_rows=True)[..., 0]
        pore = torch.as_tensor(np.stack([r.mask for r in rcs]), device=y.device).float()
        return self.scale * y * pore, lay, x


def train(rcs, refs, outer=5, inner=120, lr=2e-3, lr_end=2e-4, seed=0, checkpoints=None, damp=1e-6, log=print):
    """A-posteriori training of the rate closure on samples rcs (RateCase, one
    coarse shape) against the fine M(t) refs ((n, 3) per sample, after every
    4th fine step). Returns (closure, loss history)."""
    import torch
    if checkpoints is None:
        n = rcs[0].n
        checkpoints = list(range(max(1, n // 8), n + 1, max(1, n // 8)))
    net = C.Net(seed=seed, zero_last=True)
    clo = RateClosure(net)
    dev = net.device
    s0 = [abs(r[0, 0] + 1j * r[0, 1]) for r in refs]
    pore = torch.as_tensor(np.stack([r.mask for r in rcs]), device=dev).float()
    losses = []
    total = outer * inner
    it = 0
    for o in range(outer):
        with torch.no_grad():
            corr0, lay, x = clo.predict(rcs)
        # rollouts with the current corrections: residuals and sensitivities
        res, sens = [], []
        for i, rc in enumerate(rcs):
            c = corr0[i].double().cpu().numpy()
            mt, sn = rc.rollout(c, checkpoints)
            e = [complex(mt[n - 1, 0] - refs[i][n - 1, 0], mt[n - 1, 1] - refs[i][n - 1, 1]) for n in checkpoints]
            res.append(torch.as_tensor(np.array(e), device=dev))
            sens.append(torch.stack([sn[n] for n in checkpoints]))
        rollout_err = float(np.mean([torch.abs(r).max().item() / s for r, s in zip(res, s0)]))
        for _ in range(inner):
            frac = it / max(total - 1, 1)
            rate = lr * (lr_end / lr) ** frac
            corr, lay, x = clo.predict(rcs)
            d = (corr - corr0).double()
            loss = 0.0
            dldc = torch.zeros_like(corr)
            for i in range(len(rcs)):
                e = res[i] + (sens[i] * d[i][None]).sum(dim=(1, 2, 3))
                loss += float((e.abs() ** 2).sum()) / s0[i] ** 2
                g = 2.0 * (e.conj()[:, None, None, None] * sens[i]).real.sum(dim=0) / s0[i] ** 2
                # damping of the Gauss-Newton step (a trust region around corr0)
                nv = float(pore[i].sum())
                loss += damp * float((d[i] ** 2).sum()) / nv
                g = g + 2.0 * damp * d[i] / nv
                dldc[i] = g.float()
            dy = torch.zeros((len(rcs),) + tuple(s + 2 for s in rcs[0].shape) + (C.CH,), device=dev)
            dy[:, 1:-1, 1:-1, 1:-1, 0] = clo.scale * dldc * pore
            net.backward(lay, dy.reshape(-1, C.CH))
            net.adamw(lr=rate, weight_decay=1e-4)
            losses.append(loss / len(rcs))
            it += 1
        net.check_status()
        if log:
            log({"outer": o, "rollout_err": rollout_err, "loss_lin": losses[-1]})
    return clo, losses


def mt_error(mt, ref):
    """max_t |M_xy(t) - M_xy,ref(t)| / |M_xy,ref(first)| (lab frame)."""
    return C.mt_error(mt, ref)


def _timed_run(s, nsteps):
    """M(t) of nsteps steps of handle s and the device time of the steps
    alone (CUDA events on the handle's stream)."""
    import torch
    st = s.torch_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    s.run_async(nsteps)
    e1.record(st)
    s.synchronize()
    return s.read_mt(nsteps), e0.elapsed_time(e1) / 1e3


def solve_checked(rc: RateCase, corr, check_every=50, check_tol=1e-3):
    """The corrected coarse solve with a periodic fine-step check, and the
    fine solver as its fallback: at every check_every-th coarse step the
    coarse field is prolonged to the fine grid (keeping its lab-frame sums)
    and advanced 4 fine steps on a fine FP32 handle beside the coarse step;
    when the two changes of the lab-frame sums differ by more than check_tol x
    |M|, the curve goes on from there on the fine solver. corr: the
    correction (None = the plain coarse solve). Returns (M(t) after each
    coarse step, fine units; the coarse step of the fallback or None)."""
    cs = rc.solver(corr)
    fine = None
    mt = np.zeros((rc.n, 3))
    fell = None
    n = 0
    try:
        while n < rc.n:
            if n > 0 and n % check_every == 0:
                if fine is None:
                    fine = rc.case.solver(state=False)
                fine.set_step(4 * n)
                C._write_views(fine, cg.prolong(cs.field_views(), rc.case.k_at(4 * n), (rc.dxf,) * 3, rc.case.mask))
                before = fine.measure()
                after_f = fine.run(4)[-1]
                mt[n] = 8.0 * cs.run(1)[0]
                d = np.abs((mt[n] - before) - (after_f - before)).max()
                if d > check_tol * max(np.abs(before).max(), 1e-300):
                    fell = n
                    mt[n] = after_f
                    if n + 1 < rc.n:
                        mt[n + 1:] = fine.run(4 * (rc.n - n - 1))[3::4]
                    break
                n += 1
                continue
            m = min(rc.n, (n // check_every + 1) * check_every) - n
            mt[n:n + m] = 8.0 * cs.run(m)
            n += m
    finally:
        cs.close()
        if fine is not None:
            fine.close()
    return mt, fell


def time_to_mt(rc: RateCase, clo: RateClosure, check_every=0):
    """Time to the M(t) curve of the sample once its geometry is known: the
    fine FP32 solve (handle, upload, 4 n fine steps) and the learned coarse
    solve (network, handle with per-voxel rates, n coarse steps); with
    check_every, also the learned solve with its periodic fine check
    (solve_checked). Returns {s_fine, s_learned: wall seconds of everything;
    s_fine_steps, s_learned_steps: device seconds of the steps (and the
    network); s_learned_checked, checked_fell_back_at, and the checked M(t)
    under _checked_mt}, fine M(t), learned M(t)."""
    import time

    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    s = rc.case.solver(0)
    fine, t_fs = _timed_run(s, 4 * rc.n)
    fine = fine[3::4]
    s.close()
    t_fine = time.perf_counter() - t0
    t0 = time.perf_counter()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    with torch.no_grad():
        corr, _, _ = clo.predict([rc])
    e1.record()
    torch.cuda.synchronize()
    t_net = e0.elapsed_time(e1) / 1e3
    cs = rc.solver(corr[0])
    mt, t_cs = _timed_run(cs, rc.n)
    cs.close()
    t_learned = time.perf_counter() - t0
    out = {"s_fine": t_fine, "s_learned": t_learned, "s_fine_steps": t_fs, "s_learned_steps": t_net + t_cs}
    if check_every:
        # the same with the periodic fine check (network, coarse handle, the
        # fine check handle and its 4-step checks)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        with torch.no_grad():
            corr, _, _ = clo.predict([rc])
        checked, fell = solve_checked(rc, corr[0], check_every=check_every)
        out.update({"s_learned_checked": time.perf_counter() - t0, "check_every": check_every,
                    "checked_fell_back_at": fell})
        out["_checked_mt"] = checked
    return out, fine, 8.0 * mt


def evaluate(shape=(64, 64, 64), n_coarse=88, n_train=8, outer=5, inner=120, g_test=0.2, seed=5, g_train=0.0,
             damp=1e-6, lr=2e-3, save=None, log=print):
    """Train on n_train seeded fine PGSE cases (sphere packs and GRFs
    alternately, G uniform in 0..0.3 T/m), then on held-out cases (one sphere
    pack, one GRF, at g_test) compare with the FP64 fine solve: the FP32 fine
    solve, the plain coarse solve and the corrected one, with their times."""
    import time

    import torch
    rng = np.random.default_rng(seed)
    rcs, refs = [], []
    t0 = time.time()
    for i in range(n_train):
        kind = "sphere" if i % 2 == 0 else "grf"
        g = float(rng.uniform(0, 0.3)) if g_train is None else g_train
        case = C.Case.pgse(shape, seed=100 + 7 * i, kind=kind, g_amp=g, n_coarse=n_coarse, device="cuda")
        rcs.append(RateCase(case, n_coarse))
        refs.append(case.reference_mt(n_coarse, precision=0))
    t_data = time.time() - t0
    t0 = time.time()
    clo, losses = train(rcs, refs, outer=outer, inner=inner, damp=damp, lr=lr, lr_end=0.1 * lr, log=log)
    torch.cuda.synchronize()
    t_train = time.time() - t0
    if save:
        clo.save(save)
    out = {"shape": list(shape), "coarse_steps": n_coarse, "train_cases": n_train, "outer": outer, "inner": inner,
           "data_s": t_data, "train_s": t_train, "loss_first": losses[0], "loss_last": losses[-1], "held_out": []}
    for kind, s, g in (("sphere", 900, 0.0), ("grf", 901, 0.0), ("sphere", 900, g_test), ("grf", 901, g_test)):
        case = C.Case.pgse(shape, seed=s, kind=kind, g_amp=g, n_coarse=n_coarse, device="cuda")
        rc = RateCase(case, n_coarse)
        ref = case.reference_mt(n_coarse)
        f32 = case.reference_mt(n_coarse, precision=0)
        plain, _ = rc.rollout(None)
        time_to_mt(rc, clo)  # warm-up: kernels loaded, graphs captured
        times, _, corr_mt = time_to_mt(rc, clo)
        row = {"case": kind, "G": g, "err_fine_f32": mt_error(f32, ref), "err_plain": mt_error(plain, ref),
               "err_closure": mt_error(corr_mt, ref), **times}
        out["held_out"].append(row)
        if log:
            log(row)
    return out


if __name__ == "__main__":
    import argparse
    import json
    ap = argparse.ArgumentParser(description="train and evaluate the learned coarse relaxation closure")
    ap.add_argument("--edge", type=int, default=64)
    ap.add_argument("--coarse-steps", type=int, default=88)
    ap.add_argument("--train-cases", type=int, default=8)
    ap.add_argument("--outer", type=int, default=5)
    ap.add_argument("--inner", type=int, default=120)
    ap.add_argument("--g-train", type=float, default=0.0, help="training gradient (T/m); < 0: uniform in 0..0.3")
    ap.add_argument("--damp", type=float, default=1e-6)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--save", default=None, help="write the trained weights to this .npz")
    a = ap.parse_args()
    print(json.dumps(evaluate((a.edge,) * 3, a.coarse_steps, a.train_cases, a.outer, a.inner,
                              g_train=None if a.g_train < 0 else a.g_train, damp=a.damp, lr=a.lr, save=a.save)))
