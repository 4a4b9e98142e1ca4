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


def write_case_dir(case, path):
    """The fixture's reference input directory (data/*.dat) under path."""
    from initializator_gb300 import datfiles
    z = load(case)
    kw = {f.name: type(getattr(datfiles.NmrData(), f.name))(z["data_" + f.name].item())
          for f in dataclasses.fields(datfiles.NmrData)}
    data = datfiles.NmrData(**kw)
    vel = (z["vx"], z["vy"], z["vz"]) if data.n_velocity == 1 else None
    datfiles.write_case(path, data, z["mask"], vel=vel, grads=tuple(z["grads"]))
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


def describe(path):
    out = subprocess.run([build_driver(), path], capture_output=True, text=True, check=True).stdout
    vals = {}
    for line in out.split("BEGIN-DESCRIBE\n", 1)[1].splitlines():
        k, *v = line.split()
        vals[k] = [float(x) for x in v]
    return vals
