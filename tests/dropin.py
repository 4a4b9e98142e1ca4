"""Helpers for the drop-in NmrRelaxationSolve tests: case directories from
golden fixtures and the init() test driver."""
from __future__ import annotations

import dataclasses
import os
import subprocess

from helpers import load

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DRIVER_SRC = os.path.join(ROOT, "tests", "drivers", "describe_init.cpp")
DRIVER = os.path.join(ROOT, "initializator_gb300", "_build", "describe_init")


def write_case_dir(case, path, **overrides):
    """The fixture's reference input directory (data/*.dat) under path;
    overrides replace Nmr_data.dat parameters (NmrData field names)."""
    from initializator_gb300 import datfiles
    z = load(case)
    kw = {f.name: type(getattr(datfiles.NmrData(), f.name))(z["data_" + f.name].item())
          for f in dataclasses.fields(datfiles.NmrData)}
    kw.update(overrides)
    data = datfiles.NmrData(**kw)
    vel = (z["vx"], z["vy"], z["vz"]) if data.n_velocity == 1 else None
    surf = {}
    for key in datfiles.SURFREL_KEYS:
        if f"surf_{key}_x" in z:
            surf[key] = tuple(z[f"surf_{key}_{ax}"] for ax in "xyz")
    datfiles.write_case(path, data, z["mask"], vel=vel, grads=tuple(z["grads"]), surfrel=surf, n1=z.get("n1"))
    return z


def build_driver():
    from initializator_gb300 import build
    lib = build.build()
    if not os.path.exists(DRIVER) or os.path.getmtime(DRIVER) < max(os.path.getmtime(DRIVER_SRC),
                                                                    os.path.getmtime(lib)):
        subprocess.run(["g++", "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "initializator_gb300", "csrc", "host"),
                        "-I" + os.path.join(ROOT, "include"), DRIVER_SRC, "-o", DRIVER,
                        "-L" + os.path.dirname(lib), "-lbt", "-Wl,-rpath," + os.path.dirname(lib)], check=True)
    return DRIVER


def describe(path, fields_out=None):
    """What the drop-in's init() derived; with fields_out, also its per-voxel
    T1, T2, D, c1, c2 arrays (5 x N doubles) written to that file."""
    args = [build_driver(), path] + (["--fields", fields_out] if fields_out else [])
    out = subprocess.run(args, capture_output=True, text=True, check=True).stdout
    vals = {}
    for line in out.split("BEGIN-DESCRIBE\n", 1)[1].splitlines():
        k, *v = line.split()
        vals[k] = [float(x) for x in v]
    return vals
