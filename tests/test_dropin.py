"""The drop-in NmrRelaxationSolve (C++, initializator_gb300/csrc/host).

CPU: init() reads the reference's data/*.dat files and derives the same time
step, step count, equilibrium magnetization, field direction and gradient as
the reference's own init() (golden fixtures record them): relative 1e-14,
step count exact.
GPU: nmr_exe runs the whole time loop; its CSV rows (6 significant digits, as
the reference prints them) match the oracle run with the same time step, the
reference's schedule and the reference's scheme of that path (solve_gpu:
MacCormack; solve: ExplicitSimple) to 5e-6 relative.
"""
import os
import subprocess

import numpy as np
import pytest

from dropin import describe, write_case_dir
from helpers import CASES, common, initial_state, rel_err, velocity


@pytest.mark.parametrize("case", CASES)
def test_init_matches_reference(case, tmp_path, btlib):
    z = write_case_dir(case, str(tmp_path))
    d = describe(str(tmp_path))
    assert abs(d["dTime"][0] / z["dt_init"] - 1) <= 1e-14
    assert int(d["nStep"][0]) == int(z["nstep_init"])
    assert abs(d["pEq"][0] / z["p_eq"] - 1) <= 1e-14
    assert np.allclose(d["direction"], z["direction"], rtol=1e-14, atol=0)
    assert d["gradientPulse"][0] == z["gradient_pulse"]


@pytest.mark.parametrize("case", ["surfrel", "two_phase"])
def test_init_fields_match_reference(case, tmp_path, btlib):
    """SurfRel*.dat and n1_init.dat read by the drop-in: its per-voxel T1, T2,
    D are the reference's relTime / diffusion arrays bit for bit, and its time
    step matches the reference's init()."""
    from test_fluid_golden import coeffs
    z = write_case_dir(case, str(tmp_path / "case"))
    out = str(tmp_path / "fields.bin")
    d = describe(str(tmp_path / "case"), fields_out=out)
    n = z["mask"].size
    f = np.fromfile(out).reshape(5, *z["mask"].shape)
    assert np.array_equal(f[0], z["t1f"]) and np.array_equal(f[1], z["t2f"]) and np.array_equal(f[2], z["diff"])
    _, (p1, p2), _ = coeffs(z)
    assert np.array_equal(f[3], p1) and np.array_equal(f[4], p2)
    assert abs(d["dTime"][0] / z["dt_init"] - 1) <= 1e-14
    assert int(d["nStep"][0]) == int(z["nstep_init"])
    assert n == f[0].size


def _read_csv(path):
    rows = []
    with open(path) as f:
        next(f)
        for line in f:
            rows.append([float(v) for v in line.split(";")])
    return np.array(rows)


def _phase_sums0(z, st0, p1, p2):
    """OutputX/Y/Z with two components (cpp:3324-3350) of a field."""
    bx, by, bz = int(z["data_buffer_x"]), int(z["data_buffer_y"]), int(z["data_buffer_z"])
    nz, ny, nx = z["mask"].shape
    sel = np.zeros(z["mask"].shape, bool)
    sel[bz:nz - bz, by:ny - by, bx:nx - bx] = True
    sel &= (z["mask"] == 1) & ((p1 > 0.8) | (p2 > 0.8))
    return np.array([(st0[c] * p1)[sel].sum() for c in range(3)] + [(st0[c] * p2)[sel].sum() for c in range(3)])


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["fid", "pfg_flow", "surfrel", "two_phase"])
@pytest.mark.parametrize("path", ["gpu", "cpu"])
def test_nmr_exe_end_to_end(case, path, tmp_path, btlib, oracle_lib):
    import initializator_gb300 as bt
    import oracle
    from initializator_gb300 import build
    from test_fluid_golden import coeffs
    z = write_case_dir(case, str(tmp_path))
    d = describe(str(tmp_path))
    env = dict(os.environ)
    if path == "cpu":
        env["BT_CPU_PATH"] = "1"
    r = subprocess.run([build.EXE, "1", "1", "1"], cwd=str(tmp_path), env=env, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    got = _read_csv(os.path.join(str(tmp_path), f"results_{path}.csv"))
    # the oracle with the drop-in's time step and the reference's schedule
    dt = d["dTime"][0]
    nstep = int(d["nStep"][0])
    kw = common(z)
    kw["dt"] = dt
    pl = bt.sequence_schedule(int(z["data_n_sequence"]), nstep + 1, dt=dt, time1=float(z["data_time1"]),
                              time2=float(z["data_time2"]), direction=tuple(z["direction"]),
                              gradient_pulse=float(z["gradient_pulse"]), gpu_variant=(path == "gpu"))
    p = oracle.make_params(z["mask"].shape, **kw)
    st0 = initial_state(z)
    two = int(z["data_n_components"]) == 2
    per_voxel = two or int(z["data_n_surf_rel_water"]) == 1 or int(z["data_n_surf_rel_oil"]) == 1
    _, (p1, p2), _ = coeffs(z)
    fields = (z["t1f"], z["t2f"], z["diff"]) if per_voxel else None
    # solve_gpu steps with the reference's GPU scheme (MacCormack), solve()
    # with its CPU scheme (ExplicitSimple)
    res = oracle.run(p, z["mask"], st0, nstep + 1, vel=velocity(z), pulses=pl, fields=fields,
                     phases=(p1, p2) if two else None, maccormack=(path == "gpu"))
    mt = res[2] if two else res[1]
    s0 = _phase_sums0(z, st0, p1, p2) if two else oracle.sums(p, z["mask"], st0)[0]
    nd = int(z["data_nd_print"])
    steps = np.arange(0, nstep + 1, nd)
    ref = mt[steps] if path == "gpu" else np.vstack([s0[None], mt])[steps]
    assert got.shape == (len(steps), 7 if two else 4)
    assert np.allclose(got[:, 0], steps * dt, rtol=5e-6)
    scale = np.abs(ref).max()
    assert np.abs(got[:, 1:] - ref).max() <= 5e-6 * scale
    if path == "gpu":
        final = _read_csv_noheader(os.path.join(str(tmp_path), "results_NMR", "results_grad_1_1_1.csv"))
        assert np.abs(final[1:] - mt[-1]).max() <= 5e-6 * scale


def _read_csv_noheader(path):
    with open(path) as f:
        return np.array([float(v) for v in f.readline().split(";")])


@pytest.mark.gpu
@pytest.mark.parametrize("nb", [(3, 3, 3, 3, 3, 3), (2, 1, 1, 1, 3, 3), (1, 3, 3, 1, 1, 1)])
@pytest.mark.parametrize("case", ["fid", "pfg_flow"])
def test_nmr_exe_boundaries(case, nb, tmp_path, btlib, oracle_lib):
    """solve_gpu with nBoundary1..6 other than 1: the drop-in maps them to the
    GPU path's ghost-layer kinds (copy / periodic / zero per pair); its CSV
    matches the oracle's MacCormack run with those kinds (which the GPU tests
    pin to the reference's own BC kernels) to 5e-6 relative. solve() (the CPU
    path) keeps copy layers, as the reference's CPU path does."""
    import initializator_gb300 as bt
    import oracle
    from initializator_gb300 import build
    ov = {f"nb{b + 1}": int(v) for b, v in enumerate(nb)}
    z = write_case_dir(case, str(tmp_path), **ov)
    d = describe(str(tmp_path))
    r = subprocess.run([build.EXE, "1", "1", "1"], cwd=str(tmp_path), capture_output=True, text=True)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    got = _read_csv(os.path.join(str(tmp_path), "results_gpu.csv"))
    dt = d["dTime"][0]
    nstep = int(d["nStep"][0])
    kw = common(z)
    kw["dt"] = dt
    pl = bt.sequence_schedule(int(z["data_n_sequence"]), nstep + 1, dt=dt, time1=float(z["data_time1"]),
                              time2=float(z["data_time2"]), direction=tuple(z["direction"]),
                              gradient_pulse=float(z["gradient_pulse"]), gpu_variant=True)
    p = oracle.make_params(z["mask"].shape, boundary=bt.boundary_from_nb(nb), **kw)
    _, mt = oracle.run(p, z["mask"], initial_state(z), nstep + 1, vel=velocity(z), pulses=pl, maccormack=True)
    nd = int(z["data_nd_print"])
    steps = np.arange(0, nstep + 1, nd)
    ref = mt[steps]
    assert got.shape == (len(steps), 4)
    assert np.abs(got[:, 1:] - ref).max() <= 5e-6 * np.abs(ref).max()
    # the same case with copy layers gives another curve: the kinds took effect
    p0 = oracle.make_params(z["mask"].shape, **kw)
    _, mt0 = oracle.run(p0, z["mask"], initial_state(z), nstep + 1, vel=velocity(z), pulses=pl, maccormack=True)
    assert np.abs(mt0[steps] - ref).max() > 1e-4 * np.abs(ref).max()
