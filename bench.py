#!/usr/bin/env python
"""Throughput of the fused Bloch–Torrey step on GB300: voxel-steps/s and the
fraction of the HBM roofline it reaches.

Workload (one GPU): 256^3 sphere pack (radius 10 voxels, solid fraction 0.4),
face velocities from the curl of Gaussian-smoothed (sigma 4) vector noise,
zero on solid faces, max |v| = 1 mm/s, PGSE along z (G = 0.1 T/m, delta = 2 ms,
Delta = 20 ms, gamma = 2.675e8 rad/s/T) with a 180 degree refocusing pulse,
complex Mxy + Mz in FP32 (k-space exact-precession scheme), dx = 1 um,
D = 2.3e-9 m^2/s, T1 = 2.5 s, T2 = 2.0 s, rho = 10 um/s, dt = 0.9 dx^2/(6D).
Seeded synthetic inputs stand in for the reference's missing Poro/Vx/Vy/Vz.

One bench step = STEPS_PER_ITER (500) time steps of the whole field (one
M(t) sample per time step). Every time step streams ~620 MB through HBM, so
the working set exceeds the 129 MB L2 between timed iterations.

--impl reference times the reference's CPU update (the oracle port of
ExplicitSimple, FP64, all host threads) on a bounded sample of the same
workload. Multi-GPU runs are replicas (one independent field per GPU, no
data-path collective).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import re
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "voxel-steps/s/GB300 (%HBM roofline)"
UNIT = "voxel-steps/s"
SHAPE = (256, 256, 256)
STEPS_PER_ITER = 500
BYTES_PER_VOXEL_STEP = 37  # FP32: state read 12 + write 12 + face velocities 12 + geometry code 1
SEED = 20261203
WORKLOAD = "C2: 256^3 sphere pack r=10 phi_s=0.4, curl-noise flow 1 mm/s, PGSE z G=0.1 T/m d=2 ms D=20 ms, FP32 Mxy+Mz"


def rank_info():
    r = int(os.environ.get("RANK", "0"))
    w = int(os.environ.get("WORLD_SIZE", "1"))
    lr = int(os.environ.get("LOCAL_RANK", "0"))
    return r, w, lr


def max_over_ranks(x: float, device="cuda") -> float:
    """The largest x over all ranks (a replica job takes as long as its
    slowest rank); x itself without a process group."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(units_per_rank: float, world: int, seconds: float) -> float:
    """Whole-job throughput of N replicas: all ranks' units over the slowest rank's time."""
    return units_per_rank * world / seconds


def build_workload(device="cpu", seed=SEED):
    from initializator_gb300 import geometry
    mask = geometry.sphere_pack(SHAPE, 10.0, 0.4, seed=seed, device=device)
    vel = geometry.curl_velocity(mask, 4.0, 1.0e-3, seed=seed + 1, device=device)
    return mask, vel


QSHAPE = (256, 384, 384)   # C3a: 384 x 384 x 256
QBATCH = 32                 # gradient strengths, linspace(0, 0.3) T/m
QSTEPS_PER_ITER = 20


def run_qsweep(args, lr):
    """C3a: one 384x384x256 geometry (thresholded GRF, sigma 3, porosity 0.25),
    flow as C2, 32 PGSE gradient strengths advanced together: one launch per
    time step reads the shared geometry and velocity once per tile for all 32
    fields. Algorithmic bytes per voxel-step: 24 + 13 / 32."""
    import torch

    import initializator_gb300 as bt
    from initializator_gb300 import geometry
    dev = torch.device("cuda", lr)
    mask = geometry.gaussian_random_field(QSHAPE, 3.0, 0.25, seed=SEED + 7, device=dev)
    vel = geometry.curl_velocity(mask, 4.0, 1.0e-3, seed=SEED + 8, device=dev)
    S = QSTEPS_PER_ITER
    QB = args.qbatch
    total = (args.warmup + args.steps) * S + 64
    kw, wave, rf = physics(total)
    amps = np.linspace(0.0, 0.3, QB) / 0.1   # physics() builds the 0.1 T/m waveform
    waves = np.ascontiguousarray(wave[:, None, :] * amps[None, :, None])
    s = bt.Solver(bt.make_config(QSHAPE, precision=bt.BT_F32, scheme=bt.BT_SCHEME_KSPACE, batch=QB, **kw))
    s.upload_geometry(mask, vel)
    s.set_schedule(rf, grad_wave=waves)
    m = torch.from_numpy(mask).to(dev, torch.float32)
    st = [m.expand(QB, *QSHAPE).contiguous(), torch.zeros((QB,) + QSHAPE, device=dev),
          torch.zeros((QB,) + QSHAPE, device=dev)]
    s.set_state_device(st)
    del st, m
    zsplit = s.autotune(8)
    stream = torch.cuda.ExternalStream(s.stream_ptr)
    for _ in range(args.warmup):
        s.run_async(S)
    s.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        s.run_async(S)
    ev1.record(stream)
    s.synchronize()
    ms = ev0.elapsed_time(ev1)
    mt = s.read_mt(S)
    finite = bool(np.all(np.isfinite(mt)))
    s.close()
    nvox = int(np.prod(QSHAPE))
    vsteps = nvox * QB * S * args.steps
    per_launch = ms / 1e3 / (S * args.steps)
    bytes_launch = (24 * QB + 13) * nvox
    peak, peak_kind = hbm_peak()
    return {"workload": "C3a: 384x384x256 GRF sigma=3 porosity 0.25, flow 1 mm/s, 32 PGSE G in 0..0.3 T/m, FP32",
            "value": vsteps / (ms / 1e3), "unit": UNIT, "ms_per_time_step": per_launch * 1e3, "batch": QB,
            "tma_chunks": zsplit, "finite": finite,
            "roofline": {"bound": "hbm", "achieved": bytes_launch / per_launch / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": bytes_launch / per_launch / 1e9 / peak, "peak_kind": peak_kind,
                         "bytes_per_voxel_step": 24 + 13 / QB}}


RAGGED_N = 48               # C3b: 48 independent sphere packs
RAGGED_STEPS = 3000


def ragged_workload(seed=SEED + 11):
    """C3b: 48 sphere packs, each edge uniform in [48, 192] voxels, solid
    fraction uniform in [0.3, 0.5], sphere radius 6; no flow."""
    from initializator_gb300 import geometry
    rng = np.random.default_rng(seed)
    out = []
    for i in range(RAGGED_N):
        shape = tuple(int(e) for e in rng.integers(48, 193, size=3))
        out.append(geometry.sphere_pack(shape, 6.0, float(rng.uniform(0.3, 0.5)), seed=seed + 100 + i))
    return out


def run_ragged(args, lr):
    """C3b ragged batch: 48 independent samples of different sizes, PGSE as
    C2 (no flow), 3000 time steps each, advanced together by run_many (each
    handle's captured step graphs interleaved on its own stream) and, for
    comparison, one sample after another as a one-sample-per-process run
    would. Algorithmic bytes per voxel-step: 25."""
    import torch

    import initializator_gb300 as bt
    masks = ragged_workload()
    kw, wave, rf = physics(RAGGED_STEPS + 64)
    kw = dict(kw, velocity=0)
    solvers = []
    for m in masks:
        s = bt.Solver(bt.make_config(m.shape, precision=bt.BT_F32, scheme=bt.BT_SCHEME_KSPACE, **kw))
        s.upload_geometry(m)
        s.set_schedule(rf, grad_wave=wave)
        st0 = np.zeros((3,) + m.shape)
        st0[0] = m
        s.set_state(st0)
        solvers.append(s)
    nvox = sum(int(np.prod(m.shape)) for m in masks)
    # warm-up: graph capture and first touch (64 steps), then back to step 0
    bt.run_many(solvers, 64)
    for s in solvers:
        s.set_step(0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    mts = bt.run_many(solvers, RAGGED_STEPS)
    torch.cuda.synchronize()
    t_many = time.perf_counter() - t0
    finite = all(bool(np.all(np.isfinite(m))) for m in mts)
    # one sample after another, each with the chunking it would take alone
    # (run_many set the chunking for sharing the GPU); warm-up recaptures
    for s in solvers:
        s.set_zsplit(0)
        s.set_step(0)
        s.run(64)
        s.set_step(0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for s in solvers:
        s.run(RAGGED_STEPS)
    t_seq = time.perf_counter() - t0
    for s in solvers:
        s.close()
    peak, peak_kind = hbm_peak()
    v_many = nvox * RAGGED_STEPS / t_many
    return {"workload": "C3b: 48 sphere packs, edges U[48,192], phi_s U[0.3,0.5], PGSE z G=0.1 T/m, no flow, FP32, "
                        "3000 steps", "voxels": nvox, "value": v_many, "unit": UNIT,
            "seconds": t_many, "sequential_value": nvox * RAGGED_STEPS / t_seq, "sequential_seconds": t_seq,
            "finite": finite,
            "roofline": {"bound": "hbm", "achieved": v_many * 25 / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": v_many * 25 / 1e9 / peak, "peak_kind": peak_kind, "bytes_per_voxel_step": 25}}


C1_SHAPE = (64, 64, 64)
C1_STEPS = 2000


def run_c1(args, lr):
    """C1, the compatibility configuration: 64^3 sphere pack (r 6, solid
    0.35), no flow, no gradient, T1 2.5 s, T2 2.0 s, rho 10 um/s, the
    reference's update (ExplicitSimple) in FP64 (bit-identical to the
    reference's fields) and in FP32: 2000 time steps timed with CUDA events
    after a warm-up of 64 (one step per launch of the generic FP64 kernel,
    the fast path for FP32). Next to the reference's own CPU solve() at C1,
    2.76e7 voxel-steps/s on one core."""
    import torch

    import initializator_gb300 as bt
    from initializator_gb300 import geometry
    mask = geometry.sphere_pack(C1_SHAPE, 6.0, 0.35, seed=SEED + 31)
    kw = dict(dx=1e-6, dt=0.9 * (1e-6) ** 2 / (6 * 2.3e-9), d_pore=2.3e-9, t1=2.5, t2=2.0, rho1=1e-5, rho2=1e-5,
              p_eq=1.0, main_field=(1.0, 0.0, 0.0), velocity=0, diffusion=1)
    st0 = np.zeros((3,) + C1_SHAPE)
    st0[1] = mask  # Mxy = 1, Mz = 0 in the pores
    out = {}
    for name, prec in (("f64", bt.BT_F64), ("f32", bt.BT_F32)):
        with bt.Solver(bt.make_config(C1_SHAPE, precision=prec, **kw)) as s:
            s.upload_geometry(mask)
            s.set_state(st0)
            s.run(64)
            s.set_step(0)
            s.set_state(st0)
            stream = torch.cuda.ExternalStream(s.stream_ptr)
            ev0 = torch.cuda.Event(enable_timing=True)
            ev1 = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            ev0.record(stream)
            s.run_async(C1_STEPS)
            ev1.record(stream)
            s.synchronize()
            ms = ev0.elapsed_time(ev1)
            mt = s.read_mt(C1_STEPS)
        out[name] = {"value": int(np.prod(C1_SHAPE)) * C1_STEPS / (ms / 1e3), "us_per_step": 1e3 * ms / C1_STEPS,
                     "finite": bool(np.all(np.isfinite(mt)))}
    return {"workload": "C1: 64^3 sphere pack r=6 solid 0.35, no flow, no gradient, reference update (ExplicitSimple)",
            "unit": UNIT, "steps": C1_STEPS, **out,
            "reference_cpu_1core": 2.76e7}


C5_SHAPE = (768, 1024, 1024)  # C5: 1024 x 1024 x 768
C5_STEPS = 500
C5_ERR_STEPS = 200            # FP32-vs-FP64 horizon at C5 (the FP64 path runs ~4 G voxel-steps/s)
C2_ERR_STEPS = 5000           # the whole 5000-step C2 run
MT_ERR_TOL = 1e-4             # the plain form's FP32 M(t) bar


def mt_error_vs_f64(shape, mask, vel, kw, wave, rf, nsteps, device=None):
    """The benched FP32 kernel's M(t) against an FP64 run of the same solver
    (KSPACE scheme, same geometry, flow, waveform and pulses, same start:
    Mx = 1 in the pores): max over the nsteps steps of |M_FP32(t) - M_FP64(t)|
    (the 3-vector) divided by |M_FP64(0)|. The FP64 run is the generic kernel
    (pinned to the oracle's exact-rotation mode), the FP32 run the TMA fast
    path with the generic kernel on pulse steps, as in the timed region.
    Inputs on the host (numpy) or, with device set, the mask as a torch
    tensor on that device (the field is then set from device memory)."""
    import torch

    import initializator_gb300 as bt
    mts, secs = {}, {}
    for name, prec in (("f32", bt.BT_F32), ("f64", bt.BT_F64)):
        s = bt.Solver(bt.make_config(shape, precision=prec, scheme=bt.BT_SCHEME_KSPACE, **kw))
        try:
            s.upload_geometry(mask, vel)
            s.set_schedule(rf, grad_wave=wave[:nsteps + 1])
            dt = torch.float64 if prec == bt.BT_F64 else torch.float32
            m = torch.as_tensor(mask, device=device or "cuda").to(dt).contiguous()
            z = torch.zeros_like(m)
            s.set_state_device([m, z, z.clone()])
            del m, z
            m0 = s.measure()
            t0 = time.perf_counter()
            mt = s.run(nsteps)
            secs[name] = time.perf_counter() - t0
            mts[name] = (m0, mt)
        finally:
            s.close()
        torch.cuda.empty_cache()
    m0 = mts["f64"][0]
    d = np.linalg.norm(mts["f32"][1] - mts["f64"][1], axis=1)
    err = float(d.max() / np.linalg.norm(m0))
    return {"steps": nsteps, "value": err, "tol": MT_ERR_TOL, "pass": err <= MT_ERR_TOL,
            "definition": "max_t |M_f32(t) - M_f64(t)| / |M_f64(0)|, M = (Mx, My, Mz) lab-frame sums",
            "f64_seconds": secs["f64"], "f32_seconds": secs["f32"],
            "echo_f64": [float(v) for v in mts["f64"][1][-1]]}


def run_c5(args, lr):
    """C5, the largest single-GPU workload: 1024x1024x768 thresholded GRF
    (sigma 5, porosity 0.2), curl-noise flow up to 2 mm/s, PGSE along z with
    G = 0.2 T/m and the 180-degree refocusing pulse, KSPACE FP32: ~805 M
    voxels, ~40 GB resident. 500 time steps timed after 64 warm-up steps, with
    their own clock record; then the FP32-vs-FP64 M(t) error over the first
    C5_ERR_STEPS steps from the initial field."""
    import torch

    import initializator_gb300 as bt
    from initializator_gb300 import geometry
    dev = torch.device("cuda", lr)
    t0 = time.perf_counter()
    mask = geometry.gaussian_random_field(C5_SHAPE, 5.0, 0.2, seed=SEED + 21, device=dev)
    vel = geometry.curl_velocity(mask, 5.0, 2.0e-3, seed=SEED + 22, device=dev)
    gen_s = time.perf_counter() - t0
    dt = geometry.stable_dt(1e-6, 2.3e-9)
    total = 64 + C5_STEPS + 32
    wave = bt.kspace_waveform_pgse(total, dt, 0.2, 2e-3, 20e-3, axis=(0.0, 0.0, 1.0))
    rf = [(bt.pgse_refocus_step(dt, 20e-3), 2, math.pi, (1.0, 0.0, 0.0))]
    kw = dict(dx=1e-6, dt=dt, d_pore=2.3e-9, t1=2.5, t2=2.0, rho1=1e-5, rho2=1e-5, p_eq=1.0, velocity=1,
              diffusion=1, gamma=bt.GAMMA_PROTON)
    s = bt.Solver(bt.make_config(C5_SHAPE, precision=bt.BT_F32, scheme=bt.BT_SCHEME_KSPACE, **kw))
    s.upload_geometry(mask, vel)
    s.set_schedule(rf, grad_wave=wave)
    mx = torch.as_tensor(mask, device=dev).float().contiguous()
    zero = torch.zeros_like(mx)
    s.set_state_device([mx, zero, zero.clone()])
    del mx, zero
    zsplit = s.autotune(16)
    s.run(64)
    stream = torch.cuda.ExternalStream(s.stream_ptr)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    clocks = ClockSampler(lr)
    clocks.start()
    ev0.record(stream)
    s.run_async(C5_STEPS)
    ev1.record(stream)
    s.synchronize()
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1)
    mt = s.read_mt(C5_STEPS)
    s.close()
    torch.cuda.empty_cache()
    err = mt_error_vs_f64(C5_SHAPE, mask, vel, kw, wave, rf, C5_ERR_STEPS, device=dev)
    del vel
    nvox = int(np.prod(C5_SHAPE))
    per = ms / 1e3 / C5_STEPS
    peak, peak_kind = hbm_peak()
    return {"workload": "C5: 1024x1024x768 GRF sigma=5 porosity 0.2, curl-noise flow 2 mm/s, PGSE z G=0.2 T/m, "
                        "180-degree refocusing pulse, FP32",
            "voxels": nvox, "steps": C5_STEPS, "value": nvox / per, "unit": UNIT, "ms_per_time_step": per * 1e3,
            "tma_chunks": zsplit, "finite": bool(np.all(np.isfinite(mt))), "generate_s": gen_s, "clocks": clk,
            "mt_rel_err_vs_f64": err,
            "roofline": {"bound": "hbm", "achieved": BYTES_PER_VOXEL_STEP * nvox / per / 1e9, "peak": peak,
                         "unit": "GB/s", "frac": BYTES_PER_VOXEL_STEP * nvox / per / 1e9 / peak,
                         "peak_kind": peak_kind, "bytes_per_voxel_step": BYTES_PER_VOXEL_STEP}}


CPMG_ECHO = 10               # steps between the multi-echo leg's refocusing pulses
CPMG_G = 0.05                # T/m, its constant gradient along z


def cpmg_schedule(n):
    """The multi-echo leg's schedule over n steps: a constant gradient
    CPMG_G along z (with 16 spare steps), a 90-degree pulse about y at step 0
    and a 180-degree pulse about x at CPMG_ECHO / 2 and every CPMG_ECHO steps
    after it."""
    wave = np.zeros((n + 16, 3))
    wave[:, 2] = CPMG_G
    rf = [(0, 2, 0.5 * math.pi, (0.0, 1.0, 0.0))]
    rf += [(q, 2, math.pi, (1.0, 0.0, 0.0)) for q in range(CPMG_ECHO // 2, n, CPMG_ECHO)]
    return wave, rf


def run_cpmg(s, stream, st0, nvox, value_plain):
    """Multi-echo (CPMG) train on the C2 handle (same geometry, flow and
    z-chunking): a 90-degree pulse about y at step 0, then a 180-degree pulse
    about x every CPMG_ECHO steps, under a constant gradient along z; one
    warm-up iteration of STEPS_PER_ITER steps, then 2 x STEPS_PER_ITER timed
    steps (CUDA events). A step whose pulses are all fixed-angle stays on the
    fast path, so the train should run near the pulse-free rate; reported
    with its ratio to the C2 value. No 32-step window is pulse-free, so every
    step is its own launch (no CUDA graph)."""
    import torch
    S = STEPS_PER_ITER
    wave, rf = cpmg_schedule(3 * S)
    s.set_step(0)
    s.set_schedule(rf, grad_wave=wave)
    s.set_state(st0)
    s.run_async(S)
    s.synchronize()
    l0 = s.launches
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    s.run_async(2 * S)
    ev1.record(stream)
    s.synchronize()
    ms = ev0.elapsed_time(ev1)
    launches = s.launches - l0
    mt = s.read_mt(2 * S)
    v = nvox * 2 * S / (ms / 1e3)
    return {"workload": f"C2 handle, CPMG: 90y at step 0, 180x every {CPMG_ECHO} steps, G = {CPMG_G} T/m along z, "
                        f"{2 * S} timed steps", "value": v, "unit": UNIT, "ms_per_time_step": ms / (2 * S),
            "pulse_steps": sum(1 for q, *_ in rf if S <= q < 3 * S), "launches": launches,
            "vs_pulse_free": v / value_plain, "finite": bool(np.all(np.isfinite(mt)))}


def physics(total_steps):
    import initializator_gb300 as bt
    from initializator_gb300 import geometry
    dt = geometry.stable_dt(1e-6, 2.3e-9)
    wave = bt.kspace_waveform_pgse(total_steps, dt, 0.1, 2e-3, 20e-3, axis=(0.0, 0.0, 1.0))
    rf = [(bt.pgse_refocus_step(dt, 20e-3), 2, math.pi, (1.0, 0.0, 0.0))]
    kw = dict(dx=1e-6, dt=dt, d_pore=2.3e-9, t1=2.5, t2=2.0, rho1=1e-5, rho2=1e-5, p_eq=1.0, velocity=1,
              diffusion=1, gamma=bt.GAMMA_PROTON)
    return kw, wave, rf


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 100 ms."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.lines = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def hbm_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profiled_traffic():
    """DRAM bytes per launch of the step kernel from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "step_kernel_kspace_256.md")
    try:
        with open(p) as f:
            m = re.search(r"dram_bytes_per_launch:\s*([0-9.eE+]+)", f.read())
        return float(m.group(1)) if m else None
    except OSError:
        return None


def cpu_baseline(mask, vel, seconds=6.0):
    """The oracle (FP64 restatement of the reference's ExplicitSimple) on all
    host cores over a bounded sample of the workload."""
    import oracle
    kw, wave, _ = physics(64)
    threads = os.cpu_count() or 1
    p = oracle.make_params(SHAPE, dx=kw["dx"], dt=kw["dt"], main_field=(0.0, 0.0, 1.0), gamma=kw["gamma"],
                           d_pore=kw["d_pore"], t1=kw["t1"], t2=kw["t2"], rho1=kw["rho1"], rho2=kw["rho2"],
                           p_eq=1.0, vector_mult=1, velocity=1, diffusion=1)
    st0 = np.zeros((3,) + SHAPE)
    st0[0] = mask
    oracle.run(p, mask, st0, 1, vel=vel, grad_wave=wave[:1], threads=threads)
    one = oracle.last_loop_seconds()
    n = max(1, min(int(seconds / max(one, 1e-3)), 50))
    oracle.run(p, mask, st0, n, vel=vel, grad_wave=wave[:n], threads=threads)
    el = oracle.last_loop_seconds()
    nvox = int(np.prod(SHAPE))
    return {"value": nvox * n / el, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{n} time steps of the 256^3 workload, FP64, reference update (Euler cross product, "
                      f"PGSE waveform), OpenMP over z-planes, {el:.1f} s"}


B1_STEPS = {"c1": (2000, 100), "c2": (200, 10)}  # steps timed with ndPrint = nStep, and with ndPrint = 1


def _compat_workload(name):
    """The MacCormack FP64 comparison workloads: C1 (64^3 sphere pack r 6, solid
    0.35, no flow, no gradient) and C2 (the bench's 256^3 pack with its flow and
    a static z gradient of 0.1 T/m, cross-product precession), both with the
    reference's g and Mxy = 1 in the pores."""
    from initializator_gb300 import geometry
    dt = geometry.stable_dt(1e-6, 2.3e-9)
    kw = dict(dx=1e-6, dt=dt, d_pore=2.3e-9, t1=2.5, t2=2.0, rho1=1e-5, rho2=1e-5, p_eq=1.0, diffusion=1)
    if name == "c1":
        mask = geometry.sphere_pack(C1_SHAPE, 6.0, 0.35, seed=SEED + 31)
        vel = None
        kw.update(main_field=(1.0, 0.0, 0.0), grad=(0.0, 0.0, 0.0), vector_mult=0, velocity=0)
    else:
        mask, vel = build_workload("cpu")
        kw.update(main_field=(0.0, 0.0, 1.0), grad=(0.0, 0.0, 0.1), vector_mult=1, velocity=1)
    st0 = np.zeros((3,) + mask.shape)
    st0[0] = mask
    return mask, vel, kw, st0


def reference_gpu_baseline():
    """The reference's own CUDA path at one rank: its MacCormack kernels and
    BC kernels (compiled from its sources, nvcc's default flags as its own
    build) driven as solve_gpu drives them (oracle/ref_gpu.cpp), FP64, at C1
    and C2; timed with ndPrint = nStep (kernels, boundary launches and
    device copies only) and ndPrint = 1 (plus three full-field device-to-host
    copies and the host sums every step). Host wall clock of the loop."""
    import torch

    import oracle
    if not torch.cuda.is_available():
        return {"unavailable": "no GPU on this host"}
    if oracle.ref_gpu_cubin(fmad=True) is None:
        return {"unavailable": "the reference's kernels were not compiled into oracle/_ref (its sources are read "
                               "only where BT_REFERENCE_DIR names them)"}
    out = {"kind": "the reference's CUDA kernels (src/NmrRelaxationSolveKernels.cu, unmodified, nvcc default "
                   "flags), one rank, host loop of solve_gpu restated; FP64 MacCormack", "unit": UNIT}
    for name in ("c1", "c2"):
        mask, vel, kw, st0 = _compat_workload(name)
        p = oracle.make_params(mask.shape, **kw)
        nvox = int(mask.size)
        n_fast, n_slow = B1_STEPS[name]
        with oracle.RefGpu(p, mask, st0, vel=vel, fmad=True) as r:
            r.run(10, 10)  # warm-up: module load, first launches
            _, t_fast = r.run(n_fast, n_fast)
            _, t_slow = r.run(n_slow, 1)
        out[name] = {"grid": list(mask.shape), "ndprint_nstep": {"steps": n_fast, "seconds": t_fast,
                                                                "value": nvox * n_fast / t_fast},
                     "ndprint_1": {"steps": n_slow, "seconds": t_slow, "value": nvox * n_slow / t_slow}}
    return out


def run_compat(args, lr):
    """Our own MacCormack FP64 path (the drop-in solve_gpu's default) on the
    workloads the reference's CUDA path is timed on (B1): steps on the device,
    M(t) every step, CUDA events on the handle's stream."""
    import torch

    import initializator_gb300 as bt
    out = {"scheme": "MacCormack FP64 (the reference's GPU scheme, bit-identical to its kernels)", "unit": UNIT}
    for name in ("c1", "c2"):
        mask, vel, kw, st0 = _compat_workload(name)
        n = B1_STEPS[name][0]
        with bt.Solver(bt.make_config(mask.shape, precision=bt.BT_F64, scheme=bt.BT_SCHEME_MACCORMACK, **kw)) as s:
            s.upload_geometry(mask, vel)
            s.set_state(st0)
            s.run(64)
            stream = torch.cuda.ExternalStream(s.stream_ptr)
            ev0 = torch.cuda.Event(enable_timing=True)
            ev1 = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            ev0.record(stream)
            s.run_async(n)
            ev1.record(stream)
            s.synchronize()
            ms = ev0.elapsed_time(ev1)
            mt = s.read_mt(n)
        out[name] = {"grid": list(mask.shape), "steps": n, "value": mask.size * n / (ms / 1e3),
                     "us_per_step": 1e3 * ms / n, "finite": bool(np.all(np.isfinite(mt)))}
    return out


LEARNED_WEIGHTS = os.path.join(ROOT, "initializator_gb300", "data", "rate_closure_g0.npz")
LEARNED_CHECK_EVERY = 50  # coarse steps between the learned solve's fine checks (checked timing)
LEARNED_CASES = [((64, 64, 64), 250, "sphere", 900, 0.0), ((64, 64, 64), 250, "grf", 901, 0.0),
                 ((256, 256, 256), 250, "sphere", 902, 0.0), ((64, 64, 64), 250, "sphere", 900, 0.2)]


def run_learned(args, lr):
    """The learned coarse relaxation closure (initializator_gb300/rate_closure.py,
    weights trained by `python -m initializator_gb300.rate_closure --save`):
    on held-out seeded cases drawn like its training samples (sphere packs r 6
    with 35 % solid, Gaussian random fields, flow 1 mm/s, rho 10 um/s), the
    M(t) error against the FP64 fine solve of the fine FP32 solve, the plain
    coarse solve (2 dx, 4 dt) and the learned one, and the time to the M(t)
    curve of the fine FP32 solve and of the learned one (network + coarse
    solve). Without a gradient (what it was trained on) and, for the record,
    under PGSE at 0.2 T/m, where the coarse geometry's diffusion error is
    not corrected."""
    import torch

    from initializator_gb300 import closure as C
    from initializator_gb300 import rate_closure as R
    if not os.path.exists(LEARNED_WEIGHTS):
        return {"unavailable": "no trained weights at initializator_gb300/data/rate_closure_g0.npz"}
    clo = R.RateClosure.load(LEARNED_WEIGHTS, device=f"cuda:{lr}")
    rows = []
    for shape, n_coarse, kind, seed, g in LEARNED_CASES:
        case = C.Case.pgse(shape, seed=seed, kind=kind, g_amp=g, n_coarse=n_coarse, device=f"cuda:{lr}")
        rc = R.RateCase(case, n_coarse)
        ref = case.reference_mt(n_coarse)
        plain, _ = rc.rollout(None)
        R.time_to_mt(rc, clo, check_every=LEARNED_CHECK_EVERY)  # warm-up
        t, fine, learned = R.time_to_mt(rc, clo, check_every=LEARNED_CHECK_EVERY)
        checked = t.pop("_checked_mt")
        rows.append({"grid": list(shape), "fine_steps": 4 * n_coarse, "geometry": kind, "seed": seed, "G": g,
                     "err_fine_f32": R.mt_error(fine, ref), "err_plain_coarse": R.mt_error(plain, ref),
                     "err_learned": R.mt_error(learned, ref), "err_learned_checked": R.mt_error(checked, ref), **t,
                     "speedup": t["s_fine"] / t["s_learned"],
                     "speedup_checked": t["s_fine"] / t["s_learned_checked"],
                     "speedup_steps": t["s_fine_steps"] / t["s_learned_steps"]})
        del case, rc
        torch.cuda.empty_cache()
    return {"definition": "err = max_t |M_xy(t) - M_xy,FP64 fine(t)| / |M_xy(first)|; time to M(t) after the "
                          "geometry is known (handle, upload, steps; the learned form adds the network); "
                          "*_steps: device time of the steps (and the network) alone; *_checked: the learned "
                          "solve with a fine check (prolong, 4 fine steps, compare) every 50 coarse steps and "
                          "the fine solver as fallback",
            "weights": os.path.relpath(LEARNED_WEIGHTS, ROOT), "cases": rows}


def run_reference(args):
    r, w, _ = rank_info()
    if r != 0:
        return
    mask, vel = build_workload("cpu")
    import oracle
    oracle.build()
    kw, wave, _ = physics(4096)
    threads = os.cpu_count() or 1
    p = oracle.make_params(SHAPE, dx=kw["dx"], dt=kw["dt"], main_field=(0.0, 0.0, 1.0), gamma=kw["gamma"],
                           d_pore=kw["d_pore"], t1=kw["t1"], t2=kw["t2"], rho1=kw["rho1"], rho2=kw["rho2"],
                           p_eq=1.0, vector_mult=1, velocity=1, diffusion=1)
    st = np.zeros((3,) + SHAPE)
    st[0] = mask
    per = 1  # time steps per bench step: a bounded sample keeps the run to minutes
    for i in range(args.warmup):
        st, _ = oracle.run(p, mask, st, per, vel=vel, grad_wave=wave[i * per:(i + 1) * per], threads=threads)
    el = 0.0  # stepping-loop time only (the oracle's per-call array set-up is not the reference's cost)
    for i in range(args.steps):
        j = args.warmup + i
        st, _ = oracle.run(p, mask, st, per, vel=vel, grad_wave=wave[j * per:(j + 1) * per], threads=threads)
        el += oracle.last_loop_seconds()
    nvox = int(np.prod(SHAPE))
    v = nvox * per * args.steps / el
    out = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "grid": list(SHAPE), "steps_per_iter": per, "seed": SEED,
                   "scheme": "the reference's update (ExplicitSimple: Euler cross-product precession), FP64",
                   "l2": "inputs larger than L2", "parallelism": "host threads",
                   "note": "reference CPU update via the oracle port (the reference sources are not on the GPU box); "
                           "the same workload (geometry, flow, gradient waveform) as the GPU arm, sampled one time "
                           "step per bench step"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{per} time step per bench step of the 256^3 workload, FP64, all host threads"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "reference_gpu": reference_gpu_baseline(),
    }
    print(json.dumps(out))


def run_ours(args):
    import torch

    import initializator_gb300 as bt
    from initializator_gb300 import build as bt_build
    r, w, lr = rank_info()
    torch.cuda.set_device(lr)
    if w > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    bt_build.build()
    S = STEPS_PER_ITER
    total = (args.warmup + args.steps) * S + (args.steps + 1) * S + 16
    mask, vel = build_workload(f"cuda:{lr}", seed=SEED + r)
    kw, wave, rf = physics(total)
    nvox = int(np.prod(SHAPE))
    if args.zsplit:
        os.environ["BT_TMA_ZSPLIT"] = str(args.zsplit)
    s = bt.Solver(bt.make_config(SHAPE, precision=bt.BT_F32, scheme=bt.BT_SCHEME_KSPACE, **kw))
    s.upload_geometry(mask, vel)
    s.set_schedule(rf, grad_wave=wave)
    st0 = np.zeros((3,) + SHAPE)
    st0[0] = mask
    s.set_state(st0)
    # the autotuner picks the z-chunking of the fast path (field and step
    # restored); reported as chunks per field
    tma_key = "tma_zsplit" if args.zsplit and not args.chunks else "tma_chunks"
    if args.chunks:
        s.set_chunks(args.chunks)
        zsplit = args.chunks
    else:
        zsplit = args.zsplit if args.zsplit else s.autotune(64)
    stream = torch.cuda.ExternalStream(s.stream_ptr)

    def barrier():
        torch.cuda.synchronize()
        if w > 1:
            import torch.distributed as dist
            dist.barrier()

    # ---- device-resident throughput (value) ----
    for _ in range(args.warmup):
        s.run_async(S)
    s.synchronize()
    barrier()
    clocks = ClockSampler(lr)
    clocks.start()
    l0 = s.launches
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        s.run_async(S)
    ev1.record(stream)
    s.synchronize()
    barrier()
    clk = clocks.stop()
    launches = s.launches - l0
    ms = ev0.elapsed_time(ev1)
    mt = s.read_mt(S)
    if not np.all(np.isfinite(mt)):
        raise RuntimeError("non-finite M(t)")
    ms = max_over_ranks(ms)
    value = job_value(nvox * S * args.steps, w, ms / 1e3)
    per_launch_s = ms / 1e3 / (args.steps * S)
    achieved = BYTES_PER_VOXEL_STEP * nvox / per_launch_s / 1e9
    peak, peak_kind = hbm_peak()

    if args.profile:
        s.close()
        print(json.dumps({"profile_run": True, "ms_per_step": ms / args.steps, "launches": launches,
                          tma_key: zsplit, "value": value, "frac": achieved / hbm_peak()[0]}))
        return None

    # ---- end to end through the C ABI with host buffers (e2e) ----
    host_state = np.ascontiguousarray(st0)
    s.set_step(0)
    s.set_state(host_state)
    s.run(S)
    barrier()
    # each bench step: the H2D of its input field (bt_set_state from host
    # memory), S time steps, the D2H of its S M(t) samples (bt_read_mt). The
    # next step's input is handed over while the GPU runs the current step:
    # bt_set_state converts it on the host cores at once and queues its copy
    # behind the running steps in the handle's stream order, and bt_read_mt
    # then waits for the steps (and that copy) before the next run is queued
    t0 = time.perf_counter()
    s.set_state(host_state)
    s.run_async(S)
    for i in range(args.steps):
        if i + 1 < args.steps:
            s.set_state(host_state)  # the next step's input
        s.read_mt(S)                 # this step's M(t)
        if i + 1 < args.steps:
            s.run_async(S)
    barrier()
    e2e_s = time.perf_counter() - t0
    e2e_s = max_over_ranks(e2e_s)
    e2e = job_value(nvox * S * args.steps, w, e2e_s)
    cpmg = None if args.no_cpmg else run_cpmg(s, stream, st0, nvox, value / w)  # this rank's pulse-free rate
    s.close()
    # the benched kernel's M(t) against an FP64 run of the same solver, over
    # the whole 5000-step C2 run (a separate waveform of that length)
    err_c2 = None
    if not args.no_f64_check:
        kw2, wave2, rf2 = physics(C2_ERR_STEPS + 64)
        err_c2 = mt_error_vs_f64(SHAPE, mask, vel, kw2, wave2, rf2, C2_ERR_STEPS)
    qsweep = None if args.no_qsweep else run_qsweep(args, lr)
    ragged = None if args.no_ragged else run_ragged(args, lr)
    c5 = None if args.no_c5 else run_c5(args, lr)
    c1 = run_c1(args, lr) if args.c1 else None
    compat = None if args.no_compat else run_compat(args, lr)
    learned = None if args.no_learned else run_learned(args, lr)

    out = None
    if r == 0:
        cpu = None if args.no_cpu_baseline else cpu_baseline(mask, vel)
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": w, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "grid": list(SHAPE), "steps_per_iter": S, "seed": SEED,
                       "scheme": "kspace (exact precession), FP64 M(t) and phase",
                       "l2": "inputs larger than L2 (~620 MB streamed per time step)",
                       "parallelism": f"replicas x{w}", tma_key: zsplit},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_kind": peak_kind,
                         "bytes_per_voxel_step": BYTES_PER_VOXEL_STEP, "traffic": profiled_traffic()},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": 3 * 4 * nvox,
                    "d2h_bytes_per_step": 3 * 8 * S},
            "gpu_launches": launches,
            "clocks": clk,
            "mt_rel_err_vs_f64": err_c2,
            "cpmg": cpmg,
            "qsweep": qsweep,
            "ragged": ragged,
            "c5": c5,
            "c1": c1,
            "compat_f64": compat,
            "learned": learned,
        }
        print(json.dumps(out))
    if w > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-qsweep", action="store_true", help="skip the batched 32-gradient q-sweep (C3a) leg")
    ap.add_argument("--no-cpmg", action="store_true",
                    help="skip the multi-echo train (a 180-degree pulse every 10 steps) on the C2 handle")
    ap.add_argument("--no-ragged", action="store_true", help="skip the 48-sample ragged batch (C3b) leg")
    ap.add_argument("--no-c5", action="store_true", help="skip the 1024x1024x768 (C5, ~100 GB with its FP64 check) leg")
    ap.add_argument("--no-learned", action="store_true",
                    help="skip the learned coarse closure leg (error and time to M(t) on held-out cases)")
    ap.add_argument("--no-compat", action="store_true",
                    help="skip the MacCormack FP64 (the reference's GPU scheme) leg at C1 and C2")
    ap.add_argument("--no-f64-check", action="store_true",
                    help="skip the FP32-vs-FP64 M(t) error over the 5000-step C2 run")
    ap.add_argument("--c1", action="store_true", help="add the 64^3 compatibility (C1, FP64 and FP32) leg")
    ap.add_argument("--zsplit", type=int, default=0, help="fixed z-chunks per tile column of the fast path (skips the autotuner)")
    ap.add_argument("--chunks", type=int, default=0,
                    help="fixed z-chunks per field of the fast path, spread over the tile columns (skips the autotuner)")
    ap.add_argument("--profile", action="store_true",
                    help="device-resident phase only (for ncu captures); prints no bench line")
    ap.add_argument("--profile-leg", default="c2", choices=["c2", "qsweep", "ragged"],
                    help="with --profile: the leg to run (C2's timed phase, the q-sweep or the ragged batch)")
    ap.add_argument("--qbatch", type=int, default=QBATCH,
                    help="q-sweep members (a smaller batch keeps an ncu capture to a few GB)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.profile and args.profile_leg != "c2":
        import torch
        torch.cuda.set_device(0)
        from initializator_gb300 import build as bt_build
        bt_build.build()
        leg = run_qsweep(args, 0) if args.profile_leg == "qsweep" else run_ragged(args, 0)
        print(json.dumps({"profile_run": True, "leg": args.profile_leg, "value": leg["value"],
                          "frac": leg["roofline"]["frac"]}))
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
