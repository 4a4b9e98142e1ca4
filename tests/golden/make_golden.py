"""Generate the golden fixtures that pin the oracle to the reference itself.

Each case writes a reference input directory in the exact ``data/*.dat``
formats, runs the reference's own CPU path (``oracle/_ref/ref_harness``, built
from the reference sources by ``oracle/Makefile``) and stores inputs and
outputs in ``tests/golden/<case>.npz``:

  mask, vx, vy, vz        geometry and face velocities (package layouts)
  state0                  initial field given to the harness (or the reference's
                          own initial field when the case uses init())
  mt                      (nsteps+1, 3) sums before every step and after the last
  state                   (3, nz, ny, nx) final field
  tau1, tau2, diff        per-voxel rates and diffusivity the reference formed
  dt, p_eq, direction     what the reference computed in init() (dt: the time step
                          the run used; dt_init / nstep_init: StepTime's own result)
  data_*                  every Nmr_data.dat parameter
  pulses                  (n, 6) explicit AddImpulse list, empty when the case
                          runs the reference's own Sequence()

Run from the repository root:  python tests/golden/make_golden.py
(needs the reference sources; the fixtures are committed, the script is how
they were made).
"""
from __future__ import annotations

import dataclasses
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from initializator_gb300 import datfiles, geometry  # noqa: E402

OUT = os.path.join(ROOT, "tests", "golden")
GAMMA_REF = 4.78941714e7


def run_case(name, data: datfiles.NmrData, mask, vel=None, grads=(2.0e-3,), nsteps=20, dt=None,
             state0=None, pulses=None):
    harness = oracle.build_ref()
    assert harness, "reference sources are needed to generate fixtures"
    with tempfile.TemporaryDirectory() as tmp:
        datfiles.write_case(tmp, data, mask, vel=vel, grads=grads)
        out = os.path.join(tmp, "out")
        os.makedirs(out)
        args = [harness, tmp, str(nsteps), repr(dt if dt else 0.0), out]
        if state0 is not None:
            p = os.path.join(tmp, "state.bin")
            np.ascontiguousarray(state0, dtype=np.float64).tofile(p)
            args.append(p)
        elif pulses is not None:
            args.append("-")
        if pulses is not None:
            p = os.path.join(tmp, "pulses.txt")
            with open(p, "w") as f:
                for row in pulses:
                    f.write("%d %d %r %r %r %r\n" % tuple(row))
            args.append(p)
        r = subprocess.run(args, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(r.stdout[-2000:] + r.stderr[-2000:])
        nz, ny, nx = mask.shape
        n = nx * ny * nz
        info = {}
        with open(os.path.join(out, "info.txt")) as f:
            for line in f:
                k, *v = line.split()
                info[k] = [float(x) for x in v]
        mt = np.fromfile(os.path.join(out, "mt.bin")).reshape(-1, 3)
        state = np.fromfile(os.path.join(out, "state.bin")).reshape(3, nz, ny, nx)
        rates = np.fromfile(os.path.join(out, "rates.bin")).reshape(2, nz, ny, nx)
        diff = np.fromfile(os.path.join(out, "diff.bin")).reshape(nz, ny, nx)
    if vel is None:
        vel = (np.zeros((nz, ny, nx + 1)), np.zeros((nz, ny + 1, nx)), np.zeros((nz + 1, ny, nx)))
    fx = {
        "mask": mask.astype(np.uint8), "vx": vel[0], "vy": vel[1], "vz": vel[2],
        "mt": mt, "state": state, "tau1": rates[0], "tau2": rates[1], "diff": diff,
        "dt": info["dTime"][0], "p_eq": info["pEq"][0], "direction": np.array(info["direction"]),
        "dt_init": info["dTimeInit"][0], "nstep_init": int(info["nStepInit"][0]),
        "gradient_pulse": info["gradientPulse"][0],
        "nsteps": nsteps, "grads": np.array(grads, dtype=np.float64),
        "pulses": np.array(pulses if pulses is not None else np.zeros((0, 6)), dtype=np.float64).reshape(-1, 6),
        "state0": (np.zeros((3, nz, ny, nx)) if state0 is None else state0),
        "state0_given": state0 is not None,
    }
    for fld in dataclasses.fields(datfiles.NmrData):
        fx["data_" + fld.name] = getattr(data, fld.name)
    np.savez_compressed(os.path.join(OUT, name + ".npz"), **fx)
    print(f"{name}: {mask.shape} steps={nsteps} dt={fx['dt']:.6e} final sums={mt[-1]}")


def main():
    dx = 1.0e-6
    d = 2.3e-9
    dt = geometry.stable_dt(dx, d)

    # 1. FID through the reference's init() and Sequence(): x-directed field,
    #    surface relaxation, no flow.
    mask = geometry.sphere_pack((8, 10, 12), radius=2.5, solid_fraction=0.3, seed=11)
    data = datfiles.NmrData(n_direction_field=1, n_sequence=0, dx=dx, dy=dx, dz=dx, d_water=d,
                            r1_water=2e-4, r2_water=3e-4, t1_water=0.05, t2_water=0.02, time2=1.0)
    run_case("fid", data, mask, nsteps=60, dt=dt)

    # 2. PFG (NSEQUENCE 2) with face velocities, static gradient cross product,
    #    z-directed field, pulses from the reference's own schedule.
    mask = geometry.sphere_pack((11, 9, 10), radius=2.0, solid_fraction=0.25, seed=12)
    vel = geometry.curl_velocity(mask, sigma=1.5, vmax=2e-3, seed=13)
    data = datfiles.NmrData(n_direction_field=3, n_sequence=2, n_velocity=1, n_vector_mult=1,
                            bx0=0.0, bz0=1.0, dx=dx, dy=dx, dz=dx, d_water=d, grad_x=0.01, grad_y=-0.02,
                            grad_z=0.03, vel_mult=1.0, r1_water=1e-4, r2_water=1.5e-4,
                            time1=5.3 * dt, time2=12.3 * dt)
    run_case("pfg_flow", data, mask, vel=vel, nsteps=40, dt=dt)

    # 3. Every AddImpulse flag, injected random initial field, automatic field
    #    direction (NDIRECT_FIELD 0), flow and cross product.
    mask = geometry.sphere_pack((7, 8, 9), radius=1.8, solid_fraction=0.3, seed=14)
    vel = geometry.curl_velocity(mask, sigma=1.2, vmax=3e-3, seed=15)
    rng = np.random.default_rng(16)
    state0 = rng.uniform(-1.0, 1.0, size=(3,) + mask.shape) * 1e-3
    data = datfiles.NmrData(n_direction_field=0, n_sequence=0, n_velocity=1, n_vector_mult=1,
                            bx0=0.3, by0=0.5, bz0=0.8, dx=dx, dy=1.2 * dx, dz=0.9 * dx, d_water=d,
                            grad_x=0.02, grad_y=-0.01, grad_z=0.03, vel_mult=0.5, r1_water=5e-5,
                            r2_water=7e-5, t1_water=0.3, t2_water=0.1)
    pulses = [
        (2, 1, 3.0e-3, 0.2, -0.4, 0.9),
        (5, 2, 0.7, 0.0, 0.6, 0.8),
        (9, 3, 1.0, 1e-9, 2e-9, -1e-9),
        (13, 4, 1.0, 0.01, 0.02, 0.03),
        (13, 2, np.pi, 1.0, 0.0, 0.0),
    ]
    run_case("pulses_explicit", data, mask, vel=vel, nsteps=20, dt=0.5 * dt, state0=state0, pulses=pulses)

    # 4. Oil phase (NFLUID 2), trimmed sums (buffers), y-directed field, CPMG
    #    (NSEQUENCE 1) from the reference's own schedule.
    mask = geometry.sphere_pack((9, 12, 10), radius=2.2, solid_fraction=0.3, seed=17)
    data = datfiles.NmrData(n_direction_field=2, n_sequence=1, n_fluid=2, bx0=0.0, by0=1.0, dx=dx, dy=dx,
                            dz=dx, d_oil=4e-10, r1_oil=3e-5, r2_oil=6e-5, t1_oil=0.2, t2_oil=0.05,
                            time1=3.3 * dt, buffer_x=1, buffer_y=2, buffer_z=1)
    run_case("cpmg_oil", data, mask, nsteps=30, dt=dt)


if __name__ == "__main__":
    main()
