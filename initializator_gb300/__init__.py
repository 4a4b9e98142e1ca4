"""GB300-native Bloch–Torrey magnetization solver (drop-in for the reference's
``NmrRelaxationSolve`` stepper).

The compute path is ``_build/libbt.so`` (hand-written sm_103a CUDA behind the
C ABI of ``include/bt.h``); this module is a thin ctypes binding of that ABI
for tests, benchmarks and Python callers. There is no CPU fallback: when the
library is missing, :func:`lib` raises.
"""
from __future__ import annotations

import ctypes
import math
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "_build", "libbt.so")

BT_OK = 0
BT_F32, BT_F64 = 0, 1
BT_SCHEME_REFERENCE, BT_SCHEME_KSPACE, BT_SCHEME_MACCORMACK = 0, 1, 2
BT_BC_COPY, BT_BC_PERIODIC, BT_BC_ZERO = 0, 1, 2
GAMMA_REFERENCE = 4.78941714e7   # the reference's hard-coded g (cpp:807)
GAMMA_PROTON = 2.675e8            # rad/s/T


class BtError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"bt error {code}: {msg}")
        self.code = code


class Config(ctypes.Structure):
    """bt_config of include/bt.h."""
    _fields_ = [
        ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
        ("precision", ctypes.c_int), ("scheme", ctypes.c_int),
        ("vector_mult", ctypes.c_int), ("velocity", ctypes.c_int), ("diffusion", ctypes.c_int),
        ("buffer", ctypes.c_int * 3), ("batch", ctypes.c_int),
        ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dz", ctypes.c_double), ("dt", ctypes.c_double),
        ("main_field", ctypes.c_double * 3), ("gamma", ctypes.c_double), ("grad", ctypes.c_double * 3),
        ("d_pore", ctypes.c_double), ("t1", ctypes.c_double), ("t2", ctypes.c_double),
        ("rho1", ctypes.c_double), ("rho2", ctypes.c_double), ("p_eq", ctypes.c_double),
        ("boundary", ctypes.c_int * 3), ("reserved", ctypes.c_int),
    ]


class Pulse(ctypes.Structure):
    _fields_ = [("step", ctypes.c_longlong), ("flag", ctypes.c_int), ("reserved", ctypes.c_int),
                ("param", ctypes.c_double), ("axis", ctypes.c_double * 3)]


class SequenceParams(ctypes.Structure):
    _fields_ = [("n_sequence", ctypes.c_int), ("gpu_variant", ctypes.c_int), ("dt", ctypes.c_double),
                ("time1", ctypes.c_double), ("time2", ctypes.c_double), ("direction", ctypes.c_double * 3),
                ("gradient_pulse", ctypes.c_double), ("multiple_gradients", ctypes.c_double * 3)]


class Conv3dArgs(ctypes.Structure):
    """bt_conv3d_args of include/bt.h."""
    _fields_ = [("nb", ctypes.c_int), ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
                ("mode", ctypes.c_int), ("reserved", ctypes.c_int), ("x", ctypes.c_void_p),
                ("wpack", ctypes.c_void_p), ("bias", ctypes.c_void_p), ("out", ctypes.c_void_p),
                ("pre", ctypes.c_void_p), ("outf", ctypes.c_void_p), ("status", ctypes.c_void_p)]


# every symbol include/bt.h declares
EXPORTS = [
    "bt_create", "bt_destroy", "bt_last_error", "bt_upload_geometry", "bt_set_state", "bt_get_state",
    "bt_set_state_device", "bt_set_schedule", "bt_step_index", "bt_set_step", "bt_run", "bt_run_async",
    "bt_run_many", "bt_read_mt", "bt_synchronize", "bt_upload_rates", "bt_upload_rate_palette",
    "bt_set_phase_weights",
    "bt_read_mt_phases", "bt_stream", "bt_measure", "bt_launch_count", "bt_sequence_schedule",
    "bt_version", "bt_autotune", "bt_set_tma_split", "bt_set_tma_chunks", "bt_step_noalloc",
    "bt_conv3d_margin", "bt_conv3d", "bt_conv3d_weight_grad", "bt_conv3d_wgrad_scratch", "bt_conv3d_pack_weights",
    "bt_adamw", "bt_umma_selftest", "bt_field_device", "bt_set_wait_polls",
]

_lib = None


def lib():
    """Load libbt.so (build it first with initializator_gb300.build.build())."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: run `python -m initializator_gb300.build` "
                           "(the solver has no CPU fallback)")
    l = ctypes.CDLL(LIB_PATH)
    vp, dp, ll, i = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_longlong, ctypes.c_int
    sig = {
        "bt_create": ([ctypes.POINTER(Config), ctypes.POINTER(vp)], i),
        "bt_destroy": ([vp], i),
        "bt_last_error": ([vp], ctypes.c_char_p),
        "bt_upload_geometry": ([vp, vp, dp, dp, dp], i),
        "bt_set_state": ([vp, dp, dp, dp], i),
        "bt_get_state": ([vp, dp, dp, dp], i),
        "bt_set_state_device": ([vp, vp, vp, vp], i),
        "bt_set_schedule": ([vp, ctypes.POINTER(Pulse), i, dp, ll], i),
        "bt_step_index": ([vp], ll),
        "bt_set_step": ([vp, ll], i),
        "bt_run": ([vp, ll, dp], i),
        "bt_run_async": ([vp, ll], i),
        "bt_run_many": ([ctypes.POINTER(vp), i, ll], i),
        "bt_upload_rates": ([vp, dp, dp, dp], i),
        "bt_upload_rate_palette": ([vp, dp, dp, i, vp], i),
        "bt_set_phase_weights": ([vp, dp, dp], i),
        "bt_read_mt_phases": ([vp, dp, ll], i),
        "bt_read_mt": ([vp, dp, ll], i),
        "bt_synchronize": ([vp], i),
        "bt_stream": ([vp], vp),
        "bt_measure": ([vp, dp], i),
        "bt_launch_count": ([vp], ll),
        "bt_sequence_schedule": ([ctypes.POINTER(SequenceParams), ll, ctypes.POINTER(Pulse), i,
                                  ctypes.POINTER(ctypes.c_int)], i),
        "bt_version": ([], ctypes.c_char_p),
        "bt_autotune": ([vp, i, ctypes.POINTER(ctypes.c_int)], i),
        "bt_set_tma_split": ([vp, i], i),
        "bt_set_tma_chunks": ([vp, i], i),
        "bt_set_wait_polls": ([vp, ll], i),
        "bt_step_noalloc": ([ctypes.POINTER(Config), vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp], i),
        "bt_conv3d_margin": ([i, i], ll),
        "bt_conv3d": ([ctypes.POINTER(Conv3dArgs), vp], i),
        "bt_conv3d_weight_grad": ([vp, vp, i, i, i, i, vp, vp, vp], i),
        "bt_conv3d_wgrad_scratch": ([i, i, i, i], ll),
        "bt_conv3d_pack_weights": ([vp, vp, vp, vp], i),
        "bt_adamw": ([vp, vp, vp, vp, i, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                      ctypes.c_float, i, vp], i),
        "bt_umma_selftest": ([vp, vp, vp, vp, vp], i),
        "bt_field_device": ([vp, i, ctypes.POINTER(vp), ctypes.POINTER(vp), ctypes.POINTER(vp),
                             ctypes.POINTER(ctypes.c_int)], i),
    }
    for name, (args, res) in sig.items():
        fn = getattr(l, name)
        fn.argtypes = args
        fn.restype = res
    _lib = l
    return l


def _dp(a):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def make_config(shape, *, dx, dy=None, dz=None, dt, precision=BT_F32, scheme=BT_SCHEME_REFERENCE,
                main_field=(1.0, 0.0, 0.0), gamma=GAMMA_REFERENCE, grad=(0.0, 0.0, 0.0), d_pore=2.3e-9,
                t1=2.5, t2=2.0, rho1=0.0, rho2=0.0, p_eq=1.0, vector_mult=0, velocity=0, diffusion=1,
                buffer=(0, 0, 0), batch=1, boundary=(0, 0, 0)) -> Config:
    nz, ny, nx = shape
    c = Config()
    c.batch = batch
    c.nx, c.ny, c.nz = nx, ny, nz
    c.precision, c.scheme = precision, scheme
    c.vector_mult, c.velocity, c.diffusion = vector_mult, velocity, diffusion
    c.buffer[:] = list(buffer)
    c.dx = dx
    c.dy = dx if dy is None else dy
    c.dz = dx if dz is None else dz
    c.dt = dt
    c.main_field[:] = list(main_field)
    c.gamma = gamma
    c.grad[:] = list(grad)
    c.d_pore, c.t1, c.t2, c.rho1, c.rho2, c.p_eq = d_pore, t1, t2, rho1, rho2, p_eq
    c.boundary[:] = list(boundary)
    return c


def boundary_from_nb(nb):
    """bt_config.boundary for nBoundary1..6 of Nmr_data.dat: per axis (x: 1 and
    3, y: 2 and 4, z: 5 and 6) copy when both faces are 1, periodic when both
    are 3, zero otherwise (the reference's GPU path, cu:1321-1396)."""
    pairs = [(nb[0], nb[2]), (nb[1], nb[3]), (nb[4], nb[5])]
    return tuple(BT_BC_COPY if p == (1, 1) else BT_BC_PERIODIC if p == (3, 3) else BT_BC_ZERO for p in pairs)


def sequence_schedule(n_sequence, nsteps, *, dt, time1=0.0, time2=0.0, direction=(1.0, 0.0, 0.0),
                      gradient_pulse=0.0, multiple_gradients=(0.0, 0.0, 0.0), gpu_variant=True):
    """The reference's pulse schedule as a list of (step, flag, param, axis) (host only)."""
    sp = SequenceParams()
    sp.n_sequence, sp.gpu_variant, sp.dt, sp.time1, sp.time2 = n_sequence, int(gpu_variant), dt, time1, time2
    sp.direction[:] = list(direction)
    sp.gradient_pulse = gradient_pulse
    sp.multiple_gradients[:] = list(multiple_gradients)
    count = ctypes.c_int(0)
    rc = lib().bt_sequence_schedule(ctypes.byref(sp), nsteps, None, 0, ctypes.byref(count))
    if rc:
        raise BtError(rc, "bt_sequence_schedule")
    arr = (Pulse * max(1, count.value))()
    lib().bt_sequence_schedule(ctypes.byref(sp), nsteps, arr, count.value, ctypes.byref(count))
    return [(int(p.step), int(p.flag), float(p.param), tuple(p.axis)) for p in arr[: count.value]]


class Solver:
    """One bt_handle: the field, its geometry and its schedule on the current GPU."""

    def __init__(self, cfg: Config):
        self._l = lib()
        self.cfg = cfg
        h = ctypes.c_void_p()
        rc = self._l.bt_create(ctypes.byref(cfg), ctypes.byref(h))
        if rc:
            raise BtError(rc, "bt_create failed")
        self._h = h
        self.shape = (cfg.nz, cfg.ny, cfg.nx)
        self.batch = max(1, cfg.batch)

    def _check(self, rc, what):
        if rc:
            raise BtError(rc, f"{what}: {self._l.bt_last_error(self._h).decode()}")

    def close(self):
        if getattr(self, "_h", None):
            self._l.bt_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def upload_geometry(self, mask, vel=None):
        mask = np.ascontiguousarray(mask, dtype=np.uint8)
        assert mask.shape == self.shape
        if vel is None:
            self._check(self._l.bt_upload_geometry(self._h, mask.ctypes.data, None, None, None), "upload_geometry")
        else:
            vx, vy, vz = (np.ascontiguousarray(v, dtype=np.float64) for v in vel)
            nz, ny, nx = self.shape
            assert vx.shape == (nz, ny, nx + 1) and vy.shape == (nz, ny + 1, nx) and vz.shape == (nz + 1, ny, nx)
            self._check(self._l.bt_upload_geometry(self._h, mask.ctypes.data, _dp(vx), _dp(vy), _dp(vz)),
                        "upload_geometry")

    def upload_rates(self, t1=None, t2=None, diff=None):
        """Per-voxel T1, T2 (s) and D (m^2/s), dense (nz, ny, nx); None resets."""
        if t1 is None and t2 is None and diff is None:
            self._check(self._l.bt_upload_rates(self._h, None, None, None), "upload_rates")
            return
        arrs = [np.ascontiguousarray(a, dtype=np.float64).reshape(self.shape) for a in (t1, t2, diff)]
        self._check(self._l.bt_upload_rates(self._h, *(_dp(a) for a in arrs)), "upload_rates")

    def upload_rate_palette(self, t1, t2, idx):
        """Per-voxel rates as a palette: entries t1[e], t2[e] (s, at most 256)
        and idx, a (nz, ny, nx) uint8 CUDA tensor of each pore voxel's entry;
        the pore diffusivity is the configuration's (FP32 handles)."""
        import torch
        t1 = np.ascontiguousarray(t1, dtype=np.float64)
        t2 = np.ascontiguousarray(t2, dtype=np.float64)
        assert t1.shape == t2.shape and t1.ndim == 1
        assert idx.dtype == torch.uint8 and idx.is_cuda and tuple(idx.shape) == self.shape and idx.is_contiguous()
        hs = self.torch_stream()
        hs.wait_stream(torch.cuda.current_stream())
        self._check(self._l.bt_upload_rate_palette(self._h, _dp(t1), _dp(t2), int(t1.size),
                                                   ctypes.c_void_p(idx.data_ptr())), "upload_rate_palette")

    def set_phase_weights(self, c1=None, c2=None):
        """Two-component sums over c1 / c2 phase fractions, dense (nz, ny, nx); None switches off."""
        if c1 is None and c2 is None:
            self._check(self._l.bt_set_phase_weights(self._h, None, None), "set_phase_weights")
            return
        a, b = (np.ascontiguousarray(x, dtype=np.float64).reshape(self.shape) for x in (c1, c2))
        self._check(self._l.bt_set_phase_weights(self._h, _dp(a), _dp(b)), "set_phase_weights")

    def read_mt_phases(self, nsteps):
        """(nsteps, 6): {x1, y1, z1, x2, y2, z2} after each step of the last run."""
        out = np.zeros((max(1, nsteps), 6))
        self._check(self._l.bt_read_mt_phases(self._h, _dp(out), int(nsteps)), "read_mt_phases")
        return out[:nsteps]

    def set_state(self, state):
        """state: (3, nz, ny, nx), or (B, 3, nz, ny, nx) for a batch of B fields."""
        state = np.asarray(state, dtype=np.float64).reshape((self.batch, 3) + self.shape)
        st = [np.ascontiguousarray(state[:, c]) for c in range(3)]
        self._check(self._l.bt_set_state(self._h, _dp(st[0]), _dp(st[1]), _dp(st[2])), "set_state")

    def set_state_device(self, tensors):
        """tensors: three contiguous CUDA tensors of the handle's precision.
        The copy waits for the work torch has queued on its current stream and
        is complete on return, so the tensors may be reused or freed."""
        import torch
        hs = self.torch_stream()
        hs.wait_stream(torch.cuda.current_stream())
        self._check(self._l.bt_set_state_device(self._h, *(ctypes.c_void_p(t.data_ptr()) for t in tensors)),
                    "set_state_device")
        hs.synchronize()

    def get_state(self):
        comps = [np.zeros((self.batch,) + self.shape) for _ in range(3)]
        self._check(self._l.bt_get_state(self._h, _dp(comps[0]), _dp(comps[1]), _dp(comps[2])), "get_state")
        out = np.stack(comps, axis=1)
        return out[0] if self.batch == 1 else out

    def set_schedule(self, pulses=(), grad_wave=None):
        arr = (Pulse * max(1, len(pulses)))()
        for n, (step, flag, param, axis) in enumerate(pulses):
            arr[n].step, arr[n].flag, arr[n].param = int(step), int(flag), float(param)
            arr[n].axis[:] = [float(a) for a in axis]
        gw = None
        nwave = 0
        if grad_wave is not None:
            gw = np.ascontiguousarray(grad_wave, dtype=np.float64).reshape(-1, self.batch, 3)
            nwave = gw.shape[0]
        self._check(self._l.bt_set_schedule(self._h, arr, len(pulses), _dp(gw), nwave), "set_schedule")

    @property
    def step(self):
        return int(self._l.bt_step_index(self._h))

    def set_step(self, step):
        self._check(self._l.bt_set_step(self._h, int(step)), "set_step")

    def run(self, nsteps):
        """Advance nsteps; M(t) after each step: (nsteps, 3), or (nsteps, B, 3)."""
        mt = np.zeros((max(1, nsteps), self.batch, 3))
        self._check(self._l.bt_run(self._h, int(nsteps), _dp(mt)), "run")
        return mt[:nsteps, 0] if self.batch == 1 else mt[:nsteps]

    def run_async(self, nsteps):
        self._check(self._l.bt_run_async(self._h, int(nsteps)), "run_async")

    def read_mt(self, nsteps):
        mt = np.zeros((max(1, nsteps), self.batch, 3))
        self._check(self._l.bt_read_mt(self._h, _dp(mt), int(nsteps)), "read_mt")
        return mt[:nsteps, 0] if self.batch == 1 else mt[:nsteps]

    def synchronize(self):
        self._check(self._l.bt_synchronize(self._h), "synchronize")

    @property
    def stream_ptr(self):
        return self._l.bt_stream(self._h)

    def torch_stream(self):
        """The handle's own (non-blocking) CUDA stream as a torch stream: torch
        work on field_views() issued under it is ordered with the handle's
        launches without a host synchronisation."""
        import torch
        if getattr(self, "_ts", None) is None:
            self._ts = torch.cuda.ExternalStream(self.stream_ptr)
        return self._ts

    def measure(self):
        out = np.zeros((self.batch, 3))
        self._check(self._l.bt_measure(self._h, _dp(out)), "measure")
        return out[0] if self.batch == 1 else out

    def autotune(self, trial_steps=64):
        """Time the candidate z-chunkings of the FP32 fast path; returns the
        chosen number of chunks per field (see set_chunks)."""
        best = ctypes.c_int(0)
        self._check(self._l.bt_autotune(self._h, int(trial_steps), ctypes.byref(best)), "autotune")
        return best.value

    def set_zsplit(self, zsplit=0):
        """The FP32 fast path's z-chunks per column (0: the default for running
        alone; run_many sets them for sharing the GPU)."""
        self._check(self._l.bt_set_tma_split(self._h, int(zsplit)), "set_tma_split")

    def set_chunks(self, chunks=0):
        """The FP32 fast path's z-chunks per field in total, spread over the
        tile columns (they differ by at most one); 0: the default."""
        self._check(self._l.bt_set_tma_chunks(self._h, int(chunks)), "set_tma_chunks")

    def set_wait_polls(self, polls=-1):
        """Failure injection: the fast path's plane-ring waits give up after
        `polls` polls (0 = at once); -1 restores the default bound."""
        self._check(self._l.bt_set_wait_polls(self._h, int(polls)), "set_wait_polls")

    def field_views(self, member=0):
        """torch views (3 x [nz][ny][nx], strided by the pitch) of the current
        field on the device (k frame for KSPACE); valid until the next run."""
        import torch
        self.synchronize()  # the field is complete before other streams see it
        ptrs = [ctypes.c_void_p() for _ in range(3)]
        pitch = ctypes.c_int(0)
        self._check(self._l.bt_field_device(self._h, member, *[ctypes.byref(p) for p in ptrs], ctypes.byref(pitch)),
                    "field_device")
        dt = torch.float64 if self.cfg.precision == BT_F64 else torch.float32
        nz, ny, nx = self.shape
        esz = 8 if dt == torch.float64 else 4
        views = []
        for p in ptrs:
            flat = _cuda_tensor_from_ptr(p.value, nz * ny * pitch.value, dt)
            views.append(flat.view(nz, ny, pitch.value)[:, :, :nx])
        return views

    @property
    def launches(self):
        return int(self._l.bt_launch_count(self._h))


def run_many(solvers, nsteps):
    """Ragged batch: advance independent solvers (any grid sizes) by nsteps
    each, their launches interleaved on their own streams; returns each
    solver's M(t) ((nsteps, 3) per solver, or (nsteps, B, 3))."""
    solvers = list(solvers)
    arr = (ctypes.c_void_p * max(1, len(solvers)))(*[s._h.value for s in solvers])
    rc = lib().bt_run_many(arr, len(solvers), int(nsteps))
    if rc:
        msgs = "; ".join(s._l.bt_last_error(s._h).decode() for s in solvers if s._l.bt_last_error(s._h))
        raise BtError(rc, f"run_many: {msgs}")
    return [s.read_mt(nsteps) for s in solvers]


def _cuda_tensor_from_ptr(ptr, n, dtype):
    """A torch tensor over device memory owned by the library (no copy)."""
    import torch
    class _Wrap:
        pass
    w = _Wrap()
    typestr = {torch.float32: "<f4", torch.float64: "<f8"}[dtype]
    w.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr, "data": (ptr, False), "version": 3,
                                  "strides": None}
    return torch.as_tensor(w, device="cuda")


def kspace_waveform_pgse(nsteps, dt, g_amp, delta, Delta, axis=(0.0, 0.0, 1.0), ramp=0.0):
    """Per-step gradient (T/m) of a PGSE sequence: lobes of length delta at
    [0, delta) and [Delta, Delta + delta), both positive (a 180 pulse at Delta/2
    between them refocuses). With ramp > 0 each lobe is a trapezoid: a linear
    rise over `ramp` seconds, the plateau at g_amp, a linear fall over the
    last `ramp` seconds of the lobe (2 ramp <= delta). Step i covers
    [i*dt, (i+1)*dt); its value is the lobe's exact average over that interval,
    so k = gamma * sum(G dt) is exact at every step boundary."""
    if ramp < 0.0 or 2.0 * ramp > delta:
        raise ValueError("ramp must be in [0, delta / 2]")
    t0 = np.arange(nsteps) * dt
    t1 = t0 + dt
    ax = np.asarray(axis, dtype=np.float64)
    if ramp == 0.0:
        # rectangular lobes: each step's overlap with them, directly
        def overlap(a, b):
            return np.clip(np.minimum(t1, b) - np.maximum(t0, a), 0.0, None) / dt

        f = overlap(0.0, delta) + overlap(Delta, Delta + delta)
        return (f[:, None] * g_amp) * ax[None, :]

    def area(start, t):
        # integral of one unit-height lobe from its start to t
        tau = np.clip(t - start, 0.0, delta)
        e, p = ramp, delta - 2.0 * ramp
        up = np.minimum(tau, e)
        a = up * up / (2.0 * e)                               # the rise
        a += np.clip(tau - e, 0.0, p)                         # the plateau
        dn = np.clip(tau - e - p, 0.0, e)
        a += dn - dn * dn / (2.0 * e)                         # the fall
        return a

    f = (area(0.0, t1) - area(0.0, t0) + area(Delta, t1) - area(Delta, t0)) / dt
    return (f[:, None] * g_amp) * ax[None, :]


def pgse_refocus_step(dt, Delta):
    """Step after whose update the 180-degree pulse of a PGSE sequence is applied."""
    return max(0, int(math.ceil(Delta / 2.0 / dt)) - 1)
