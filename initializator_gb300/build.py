"""Build the solver library ``initializator_gb300/_build/libbt.so`` for sm_103a.

Translation units are compiled in parallel with nvcc (one -gencode, no cmake):

* ``bt_step_f32.cu`` — FP32 step kernels (default -fmad=true)
* ``bt_step_tma64.cu`` — the FP32 fast path for 64-wide tiles (narrow grids)
* ``bt_step_tma_pal.cu`` — the FP32 fast path with per-voxel rates (rate palette)
* ``bt_step_f64.cu`` — FP64 step kernels, -fmad=false so that no
  multiply-add contraction changes the reference's rounding
* ``bt_api.cu``      — host runtime behind include/bt.h
* ``bt_noalloc.cu``   — the allocation-free single-step entry point
* ``bt_closure.cu``   — tcgen05 implicit-GEMM 3-D convolution of the learned closure
* ``bt_schedule.cpp`` — host replay of the reference's pulse schedules
* ``host/NmrRelaxationSolve.cpp`` + ``host/nmr_io.cpp`` — the drop-in C++ class
  (linked into the same library, and into the ``nmr_exe`` program)

Run ``python -m initializator_gb300.build`` or call :func:`build`.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libbt.so")
EXE = os.path.join(OUT, "nmr_exe")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]

UNITS = [
    ("bt_step_f32.cu", ARCH + ["--ptxas-options=-v"]),
    ("bt_step_tma64.cu", ARCH),
    ("bt_step_tma_pal.cu", ARCH),
    ("bt_step_tma_rf.cu", ARCH + ["--ptxas-options=-v"]),
    ("bt_step_f64.cu", ARCH + ["-fmad=false"]),
    ("bt_api.cu", ARCH),
    ("bt_noalloc.cu", ARCH),
    ("bt_closure.cu", ARCH),
    ("bt_schedule.cpp", []),
]
HOST_UNITS = [os.path.join("host", "NmrRelaxationSolve.cpp"), os.path.join("host", "nmr_io.cpp")]


def _newer(src_list, target):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in src_list)


def _deps(unit):
    # every unit depends on the shared headers
    hdrs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hdrs += [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    host = os.path.join(CSRC, "host")
    if os.path.isdir(host):
        hdrs += [os.path.join(host, f) for f in os.listdir(host) if f.endswith(".h")]
    return [os.path.join(CSRC, unit)] + hdrs


def _compile(unit, extra, verbose):
    src = os.path.join(CSRC, unit)
    obj = os.path.join(OUT, os.path.basename(unit) + ".o")
    if not _newer(_deps(unit), obj):
        return obj, ""
    if unit.endswith(".cu"):
        cmd = [NVCC] + COMMON + extra + ["-c", src, "-o", obj]
    else:
        cmd = [NVCC, "-x", "cu"] + COMMON + ARCH + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj, (r.stdout + r.stderr) if verbose else ""


def build(verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    units = list(UNITS)
    units += [(u, []) for u in HOST_UNITS if os.path.exists(os.path.join(CSRC, u))]
    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        results = list(ex.map(lambda u: _compile(u[0], u[1], verbose), units))
    objs = [o for o, _ in results]
    for _, log in results:
        if log:
            sys.stderr.write(log)
    if _newer(objs, LIB):
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    main = os.path.join(CSRC, "host", "main.cpp")
    if os.path.exists(main) and _newer([main, LIB], EXE):
        cmd = [NVCC, "-x", "cu"] + COMMON + ARCH + [main, "-o", EXE, "-L" + OUT, "-lbt",
                                                   "-Xlinker", "-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
