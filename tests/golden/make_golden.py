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
  t1f, t2f                relTime.t1 / relTime.t2 as the reference stores them
  surf_<key>_<x|y|z>      SurfRel face relaxivities written to the input (if any)
  n1                      n1_init.dat values (NCOMP 2)
  mt6, conc               NCOMP 2: (nsteps+1, 6) sums X1 Y1 Z1 X2 Y2 Z2 and the
                          concentrations (2, nz, ny, nx)

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
             state0=None, pulses=None, surfrel=None, n1=None):
    harness = oracle.build_ref()
    assert harness, "reference sources are needed to generate fixtures"
    with tempfile.TemporaryDirectory() as tmp:
        datfiles.write_case(tmp, data, mask, vel=vel, grads=grads, surfrel=surfrel, n1=n1)
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
        times = np.fromfile(os.path.join(out, "times.bin")).reshape(2, nz, ny, nx)
        extra = {}
        if data.n_components == 2:
            extra["mt6"] = np.fromfile(os.path.join(out, "mt6.bin")).reshape(-1, 6)
            extra["conc"] = np.fromfile(os.path.join(out, "phases.bin")).reshape(2, nz, ny, nx)
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
        "t1f": times[0], "t2f": times[1],
    }
    fx.update(extra)
    for key, faces in (surfrel or {}).items():
        for ax, a in zip("xyz", faces):
            fx[f"surf_{key}_{ax}"] = a
    if n1 is not None:
        fx["n1"] = np.asarray(n1, dtype=np.float32)
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

    # 5. Face relaxivities from SurfRel*.dat (water, both T1 and T2 files),
    #    flow, cross product, z-directed field, PFG schedule.
    mask = geometry.sphere_pack((10, 9, 12), radius=2.2, solid_fraction=0.3, seed=18)
    vel = geometry.curl_velocity(mask, sigma=1.4, vmax=2e-3, seed=19)
    rng = np.random.default_rng(20)
    nz, ny, nx = mask.shape
    surf = {key: (rng.uniform(0.5e-4, 3e-4, (nz, ny, nx + 1)), rng.uniform(0.5e-4, 3e-4, (nz, ny + 1, nx)),
                  rng.uniform(0.5e-4, 3e-4, (nz + 1, ny, nx))) for key in ("1Water", "2Water")}
    data = datfiles.NmrData(n_direction_field=3, n_sequence=2, n_velocity=1, n_vector_mult=1, n_surf_rel_water=1,
                            bx0=0.0, bz0=1.0, dx=dx, dy=dx, dz=dx, d_water=d, grad_x=0.01, grad_y=0.02,
                            grad_z=-0.01, r1_water=1e-4, r2_water=2e-4, t1_water=0.4, t2_water=0.1,
                            time1=4.3 * dt, time2=11.3 * dt)
    run_case("surfrel", data, mask, vel=vel, nsteps=30, dt=dt, surfrel=surf)

    # 6. Two components (NCOMP 2): a smooth n1 field (some voxels in each pure
    #    phase, some mixed), oil face relaxivities from files, water constants,
    #    trimmed sums, x-directed field, FID.
    mask = geometry.sphere_pack((9, 10, 11), radius=2.0, solid_fraction=0.25, seed=21)
    nz, ny, nx = mask.shape
    g = np.random.default_rng(22)
    zz, yy, xx = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    n1 = 0.5 + 0.6 * np.sin(0.7 * xx + 0.3 * g.standard_normal()) * np.cos(0.5 * yy) * np.cos(0.4 * zz + 0.2)
    n1 = np.clip(n1, 0.0, 1.0).astype(np.float32)
    surf = {key: (g.uniform(1e-5, 8e-5, (nz, ny, nx + 1)), g.uniform(1e-5, 8e-5, (nz, ny + 1, nx)),
                  g.uniform(1e-5, 8e-5, (nz + 1, ny, nx))) for key in ("1Oil", "2Oil")}
    data = datfiles.NmrData(n_direction_field=1, n_sequence=0, n_components=2, n_surf_rel_oil=1, bx0=1.0, dx=dx,
                            dy=dx, dz=dx, d_water=d, d_oil=4e-10, r1_water=2e-4, r2_water=3e-4, t1_water=0.3,
                            t2_water=0.05, t1_oil=0.2, t2_oil=0.03, an1=1.0, an2=0.0, bn1=0.0, bn2=1.0,
                            buffer_x=1, buffer_y=0, buffer_z=1)
    run_case("two_phase", data, mask, nsteps=30, dt=dt, surfrel=surf, n1=n1)


if __name__ == "__main__":
    main()
