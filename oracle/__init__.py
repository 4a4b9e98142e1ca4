"""ctypes binding of the oracle (FP64 CPU restatement of the reference's update).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
baseline legs of bench.py, where it is the checker or the reference being
timed. The product never imports it. ``build()`` compiles
``oracle/_build/libbt_oracle.so`` (gcc) and ``oracle/_build/libref_gpu.so``,
the harness that runs the reference's own CUDA kernels (:class:`RefGpu`) from
the cubins ``build_ref()`` compiles out of the reference sources (named by the
environment variable BT_REFERENCE_DIR; without it nothing is compiled from
them).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libbt_oracle.so")
REF_HARNESS = os.path.join(HERE, "_ref", "ref_harness")
REF_GPU_LIB = os.path.join(HERE, "_build", "libref_gpu.so")
# the reference's kernels as its own build makes them (nvcc's default
# -fmad=true) and without multiply-add contraction (bit-comparable to the
# oracle's and the library's FP64 arithmetic)
REF_CUBINS = {True: os.path.join(HERE, "_ref", "ref_kernels.cubin"),
              False: os.path.join(HERE, "_ref", "ref_kernels_nofma.cubin")}


class Params(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
        ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dz", ctypes.c_double), ("dt", ctypes.c_double),
        ("main_field", ctypes.c_double * 3), ("gamma", ctypes.c_double), ("grad", ctypes.c_double * 3),
        ("d_pore", ctypes.c_double), ("t1", ctypes.c_double), ("t2", ctypes.c_double),
        ("rho1", ctypes.c_double), ("rho2", ctypes.c_double), ("p_eq", ctypes.c_double),
        ("vector_mult", ctypes.c_int), ("velocity", ctypes.c_int), ("diffusion", ctypes.c_int),
        ("buffer", ctypes.c_int * 3), ("boundary", ctypes.c_int * 3),
    ]


class Pulse(ctypes.Structure):
    _fields_ = [("step", ctypes.c_longlong), ("flag", ctypes.c_int), ("pad", ctypes.c_int),
                ("param", ctypes.c_double), ("axis", ctypes.c_double * 3)]


_lib = None


def build(force: bool = False) -> str:
    if force or not (os.path.exists(LIB_PATH) and os.path.exists(REF_GPU_LIB)):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def reference_dir() -> str | None:
    """The reference's source directory (BT_REFERENCE_DIR), when given and present."""
    d = os.environ.get("BT_REFERENCE_DIR")
    return d if d and os.path.isdir(d) else None


def build_ref() -> str | None:
    """Compile the reference's CPU path into oracle/_ref/ref_harness and its GPU
    kernels into oracle/_ref/ref_kernels*.cubin (needs the reference sources,
    BT_REFERENCE_DIR); None without them."""
    ref = reference_dir()
    if ref is None:
        return None
    subprocess.run(["make", "-s", "-C", HERE, "ref", "ref-gpu", "REF=" + ref], check=True)
    return REF_HARNESS


def lib():
    global _lib
    if _lib is None:
        build()
        l = ctypes.CDLL(LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        l.bto_run_reference.argtypes = [ctypes.POINTER(Params), ctypes.c_void_p, dp, dp, dp, dp, dp, dp,
                                        ctypes.c_longlong, ctypes.POINTER(Pulse), ctypes.c_int, dp, dp, ctypes.c_int]
        l.bto_run_reference.restype = ctypes.c_int
        l.bto_run_fields.argtypes = [ctypes.POINTER(Params), ctypes.c_void_p, dp, dp, dp, dp, dp, dp,
                                     ctypes.c_longlong, ctypes.POINTER(Pulse), ctypes.c_int, dp, dp, dp, dp, dp, dp,
                                     dp, dp, ctypes.c_int]
        l.bto_run_fields.restype = ctypes.c_int
        l.bto_run_maccormack.argtypes = l.bto_run_fields.argtypes
        l.bto_run_maccormack.restype = ctypes.c_int
        l.bto_sums.argtypes = [ctypes.POINTER(Params), ctypes.c_void_p, dp, dp, dp, dp]
        l.bto_sums.restype = ctypes.c_longlong
        l.bto_rates.argtypes = [ctypes.POINTER(Params), ctypes.c_void_p, dp, dp]
        l.bto_gpu_inputs.argtypes = [ctypes.POINTER(Params), ctypes.c_void_p, dp, dp, dp, dp, dp, dp,
                                     ctypes.c_void_p, dp, dp, dp, dp, dp, dp]
        l.bto_gpu_inputs.restype = ctypes.c_int
        l.bto_last_loop_seconds.argtypes = []
        l.bto_last_loop_seconds.restype = ctypes.c_double
        _lib = l
    return _lib


def _dp(a):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def make_params(shape, *, dx, dy=None, dz=None, dt, main_field=(1.0, 0.0, 0.0), gamma=4.78941714e7,
                grad=(0.0, 0.0, 0.0), d_pore=2.3e-9, t1=2.5, t2=2.0, rho1=0.0, rho2=0.0, p_eq=1.0,
                vector_mult=0, velocity=0, diffusion=1, buffer=(0, 0, 0), boundary=(0, 0, 0)) -> Params:
    nz, ny, nx = shape
    p = Params()
    p.nx, p.ny, p.nz = nx, ny, nz
    p.dx = dx
    p.dy = dx if dy is None else dy
    p.dz = dx if dz is None else dz
    p.dt = dt
    p.main_field[:] = list(main_field)
    p.gamma = gamma
    p.grad[:] = list(grad)
    p.d_pore, p.t1, p.t2, p.rho1, p.rho2, p.p_eq = d_pore, t1, t2, rho1, rho2, p_eq
    p.vector_mult, p.velocity, p.diffusion = vector_mult, velocity, diffusion
    p.buffer[:] = list(buffer)
    p.boundary[:] = list(boundary)
    return p


def run(params: Params, mask, state, nsteps, vel=None, pulses=(), grad_wave=None, threads=0, fields=None,
        phases=None, maccormack=False):
    """Advance ``state`` (3, nz, ny, nx) float64 by nsteps; returns (state, mt[nsteps, 3]).

    fields = (t1, t2, diff): per-voxel coefficients replacing the uniform
    fluid's (dense (nz, ny, nx)). phases = (c1, c2): phase fractions; then the
    return value is (state, mt, mt6[nsteps, 6]) with the two-component sums.
    maccormack: the reference's GPU scheme (predictor-corrector) instead of
    ExplicitSimple."""
    mask = np.ascontiguousarray(mask, dtype=np.uint8)
    st = np.array(state, dtype=np.float64, copy=True)
    mx, my, mz = (np.ascontiguousarray(st[c]) for c in range(3))
    vx = vy = vz = None
    if vel is not None:
        vx, vy, vz = (np.ascontiguousarray(v, dtype=np.float64) for v in vel)
    parr = (Pulse * max(1, len(pulses)))()
    for n, (step, flag, param, axis) in enumerate(pulses):
        parr[n].step, parr[n].flag, parr[n].param = step, flag, param
        parr[n].axis[:] = list(axis)
    gw = None if grad_wave is None else np.ascontiguousarray(grad_wave, dtype=np.float64)
    mt = np.zeros((max(nsteps, 1), 3), dtype=np.float64)
    if fields is None and phases is None and not maccormack:
        rc = lib().bto_run_reference(ctypes.byref(params), mask.ctypes.data, _dp(vx), _dp(vy), _dp(vz),
                                     _dp(mx), _dp(my), _dp(mz), nsteps, parr, len(pulses), _dp(gw), _dp(mt), threads)
        if rc != 0:
            raise RuntimeError(f"oracle failed: {rc}")
        return np.stack([mx, my, mz]), mt[:nsteps]
    f = [None, None, None] if fields is None else [np.ascontiguousarray(a, dtype=np.float64) for a in fields]
    c = [None, None] if phases is None else [np.ascontiguousarray(a, dtype=np.float64) for a in phases]
    mt6 = None if phases is None else np.zeros((max(nsteps, 1), 6), dtype=np.float64)
    fn = lib().bto_run_maccormack if maccormack else lib().bto_run_fields
    rc = fn(ctypes.byref(params), mask.ctypes.data, _dp(vx), _dp(vy), _dp(vz),
                              _dp(mx), _dp(my), _dp(mz), nsteps, parr, len(pulses), _dp(gw),
                              _dp(f[0]), _dp(f[1]), _dp(f[2]), _dp(c[0]), _dp(c[1]), _dp(mt), _dp(mt6), threads)
    if rc != 0:
        raise RuntimeError(f"oracle failed: {rc}")
    if phases is None:
        return np.stack([mx, my, mz]), mt[:nsteps]
    return np.stack([mx, my, mz]), mt[:nsteps], mt6[:nsteps]


def last_loop_seconds() -> float:
    """Stepping-loop wall time of the last run() (array set-up excluded)."""
    return float(lib().bto_last_loop_seconds())


def sums(params: Params, mask, state):
    mask = np.ascontiguousarray(mask, dtype=np.uint8)
    mx, my, mz = (np.ascontiguousarray(state[c], dtype=np.float64) for c in range(3))
    out = np.zeros(3)
    n = lib().bto_sums(ctypes.byref(params), mask.ctypes.data, _dp(mx), _dp(my), _dp(mz), _dp(out))
    return out, int(n)


def rates(params: Params, mask):
    mask = np.ascontiguousarray(mask, dtype=np.uint8)
    t1 = np.zeros(mask.shape)
    t2 = np.zeros(mask.shape)
    lib().bto_rates(ctypes.byref(params), mask.ctypes.data, _dp(t1), _dp(t2))
    return t1, t2


# ---- the reference's own GPU kernels (libref_gpu.so + the cubins) ----

class RgParams(ctypes.Structure):
    _fields_ = [("ik", ctypes.c_int), ("jk", ctypes.c_int), ("kk", ctypes.c_int),
                ("dt", ctypes.c_double), ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dz", ctypes.c_double),
                ("vector_mult", ctypes.c_int), ("velocity", ctypes.c_int), ("diffusion", ctypes.c_int),
                ("p_eq", ctypes.c_double), ("nb", ctypes.c_int * 6), ("buffer", ctypes.c_int * 3)]


_rg = None


def _ref_gpu_lib():
    global _rg
    if _rg is None:
        build()
        l = ctypes.CDLL(REF_GPU_LIB)
        vp, dp = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)
        l.rg_create.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(RgParams), vp, dp, dp, dp, dp, dp, dp,
                                dp]
        l.rg_create.restype = vp
        l.rg_run.argtypes = [vp, ctypes.c_longlong, ctypes.c_longlong, dp, dp]
        l.rg_run.restype = ctypes.c_int
        l.rg_get.argtypes = [vp, dp]
        l.rg_get.restype = ctypes.c_int
        l.rg_destroy.argtypes = [vp]
        l.rg_last_error.restype = ctypes.c_char_p
        _rg = l
    return _rg


def ref_gpu_cubin(fmad: bool = False) -> str | None:
    """Path of the reference's compiled kernels, None when they were not built here."""
    p = REF_CUBINS[bool(fmad)]
    return p if os.path.exists(p) else None


def gpu_inputs(params: Params, mask, state, vel=None):
    """The ghosted arrays the reference's GPU path starts from (bto_gpu_inputs)."""
    nz, ny, nx = mask.shape
    num = (nx + 2) * (ny + 2) * (nz + 2)
    mask = np.ascontiguousarray(mask, dtype=np.uint8)
    st = np.asarray(state, dtype=np.float64)
    mx, my, mz = (np.ascontiguousarray(st[c]) for c in range(3))
    vx = vy = vz = None
    if vel is not None:
        vx, vy, vz = (np.ascontiguousarray(v, dtype=np.float64) for v in vel)
    out = {"act": np.zeros(num, dtype=np.uint8), "diff": np.zeros(num), "t1": np.zeros(num), "t2": np.zeros(num),
           "nf": np.zeros(3 * num), "vel": np.zeros(3 * num), "magn": np.zeros(3 * num)}
    rc = lib().bto_gpu_inputs(ctypes.byref(params), mask.ctypes.data, _dp(vx), _dp(vy), _dp(vz), _dp(mx), _dp(my),
                              _dp(mz), out["act"].ctypes.data, _dp(out["diff"]), _dp(out["t1"]), _dp(out["t2"]),
                              _dp(out["nf"]), _dp(out["vel"]), _dp(out["magn"]))
    if rc:
        raise RuntimeError(f"bto_gpu_inputs failed: {rc}")
    return out


class RefGpu:
    """The reference's own CUDA kernels (predictor, corrector, BC_*) driven as
    its solve_gpu loop drives them, on CUDA device `device` (see
    oracle/ref_gpu.cpp). nb: nBoundary1..6 of Nmr_data.dat. fmad: the cubin
    built as the reference builds it (True) or without multiply-add
    contraction (False, bit-comparable to FP64 restatements)."""

    def __init__(self, params: Params, mask, state, vel=None, nb=(1, 1, 1, 1, 1, 1), fmad=False, device=0):
        cubin = ref_gpu_cubin(fmad)
        if cubin is None:
            raise RuntimeError("the reference's GPU kernels were not built (oracle.build_ref with BT_REFERENCE_DIR)")
        self.shape = tuple(mask.shape)
        nz, ny, nx = self.shape
        self.num = (nx + 2) * (ny + 2) * (nz + 2)
        a = gpu_inputs(params, mask, state, vel)
        rp = RgParams()
        rp.ik, rp.jk, rp.kk = nx, ny, nz
        rp.dt, rp.dx, rp.dy, rp.dz = params.dt, params.dx, params.dy, params.dz
        rp.vector_mult, rp.velocity, rp.diffusion = params.vector_mult, params.velocity, params.diffusion
        rp.p_eq = params.p_eq
        rp.nb[:] = list(nb)
        rp.buffer[:] = list(params.buffer)
        mf = np.concatenate([np.full(self.num, float(params.main_field[c])) for c in range(3)])
        self._l = _ref_gpu_lib()
        self._h = self._l.rg_create(cubin.encode(), int(device), ctypes.byref(rp), a["act"].ctypes.data,
                                    _dp(a["diff"]), _dp(a["t1"]), _dp(a["t2"]), _dp(mf), _dp(a["nf"]),
                                    _dp(a["vel"]), _dp(a["magn"]))
        if not self._h:
            raise RuntimeError("rg_create: " + self._l.rg_last_error().decode())

    def run(self, nsteps, ndprint=1):
        """nsteps steps; returns (sums after every ndprint-th step (n, 3), loop wall seconds)."""
        n = (int(nsteps) + int(ndprint) - 1) // int(ndprint)
        mt = np.zeros((max(n, 1), 3))
        sec = ctypes.c_double(0.0)
        rc = self._l.rg_run(self._h, int(nsteps), int(ndprint), _dp(mt), ctypes.byref(sec))
        if rc:
            raise RuntimeError("rg_run: " + self._l.rg_last_error().decode())
        return mt[:n], sec.value

    def ghosted(self):
        out = np.zeros(3 * self.num)
        if self._l.rg_get(self._h, _dp(out)):
            raise RuntimeError("rg_get: " + self._l.rg_last_error().decode())
        nz, ny, nx = self.shape
        return out.reshape(3, nz + 2, ny + 2, nx + 2)

    def state(self):
        """The interior field, (3, nz, ny, nx)."""
        return np.ascontiguousarray(self.ghosted()[:, 1:-1, 1:-1, 1:-1])

    def close(self):
        if getattr(self, "_h", None):
            self._l.rg_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
