"""The oracle against the reference's own CPU path run live on generated cases
(the geometry and flow of the c1 and c2 presets of initializator_gb300.gen, on
small grids), where the reference's sources are available to build
oracle/_ref from (skipped elsewhere). Per-voxel fields bit-identical, as for
the golden fixtures; M(t) within 1e-12 relative (the oracle adds per-plane
partial sums, the reference keeps one running sum, and these grids are
larger than the fixtures')."""
import dataclasses
import os
import subprocess

import numpy as np
import pytest

from helpers import common, initial_state, pulses, rel_err, velocity


def _reference_run(case_dir, nsteps, shape):
    """The reference's solve() body (oracle/_ref/ref_harness) on case_dir with
    its own time step: (info, mt (nsteps+1, 3), final field (3, nz, ny, nx))."""
    import oracle
    out = os.path.join(case_dir, "out")
    os.makedirs(out)
    r = subprocess.run([oracle.build_ref(), case_dir, str(nsteps), "0", out], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    info = {}
    with open(os.path.join(out, "info.txt")) as f:
        for line in f:
            k, *v = line.split()
            info[k] = [float(x) for x in v]
    mt = np.fromfile(os.path.join(out, "mt.bin")).reshape(-1, 3)
    state = np.fromfile(os.path.join(out, "state.bin")).reshape((3,) + shape)
    return info, mt, state


@pytest.mark.parametrize("preset,shape,flow", [("c1", (20, 28, 36), 0.0), ("c2", (18, 24, 30), 1e-3)])
def test_oracle_matches_reference_on_generated_case(tmp_path, preset, shape, flow, oracle_lib):
    import oracle
    from initializator_gb300 import datfiles, gen
    if oracle.build_ref() is None:
        pytest.skip("the reference's sources are not on this machine")
    nz, ny, nx = shape
    spec = dict(gen.PRESETS[preset], shape=(nx, ny, nz), flow=flow)
    if spec["geometry"] == "spheres":
        spec["radius"] = 3.0
    mask, vel = gen.build_case(spec, seed=5)
    data = datfiles.NmrData(**dict(spec["data"], n_velocity=0 if vel is None else 1, n_sequence=0))
    grads = (2.0e-3,)
    datfiles.write_case(str(tmp_path), data, mask, vel=vel, grads=grads)
    nsteps = 30
    info, mt_ref, st_ref = _reference_run(str(tmp_path), nsteps, shape)

    # the same run through the oracle, with what the reference derived in init()
    z = {"data_" + f.name: getattr(data, f.name) for f in dataclasses.fields(datfiles.NmrData)}
    zero = (np.zeros((nz, ny, nx + 1)), np.zeros((nz, ny + 1, nx)), np.zeros((nz + 1, ny, nx)))
    vx, vy, vz = zero if vel is None else vel
    z.update(mask=mask, vx=vx, vy=vy, vz=vz, dt=info["dTime"][0], p_eq=info["pEq"][0],
             direction=np.array(info["direction"]), nsteps=nsteps, grads=np.array(grads),
             pulses=np.zeros((0, 6)), state0=np.zeros((3,) + shape), state0_given=False)
    p = oracle.make_params(shape, **common(z))
    st0 = initial_state(z)
    s0, _ = oracle.sums(p, mask, st0)
    st, mt = oracle.run(p, mask, st0, nsteps, vel=velocity(z), pulses=pulses(z))
    assert np.array_equal(st, st_ref), f"max abs diff {np.abs(st - st_ref).max()}"
    assert rel_err(np.vstack([s0[None], mt]), mt_ref) < 1e-12
