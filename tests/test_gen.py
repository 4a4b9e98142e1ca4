"""The input-directory generator (python -m initializator_gb300.gen), on the CPU:
what it writes reads back through the reference-format readers as the seeded
generators' arrays (bit for bit: %.17g text for doubles), and the drop-in's
init() accepts the directory as the reference's would."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def run_gen(*args):
    out = subprocess.run([sys.executable, "-m", "initializator_gb300.gen", *args], cwd=ROOT, capture_output=True,
                         text=True)
    return out


def test_spheres_with_flow_round_trip(tmp_path):
    from initializator_gb300 import datfiles, geometry
    d = str(tmp_path / "case")
    out = run_gen(d, "--shape", "14", "12", "10", "--geometry", "spheres", "--radius", "2.5", "--solid-fraction",
                  "0.3", "--flow", "1e-3", "--seed", "3", "--set", "time2=1e-3", "--set", "n_sequence=9",
                  "--grad", "0.0", "0.05")
    assert out.returncode == 0, out.stderr
    summary = json.loads(out.stdout.strip().splitlines()[-1])
    assert summary["shape"] == [14, 12, 10] and summary["velocity"]
    data_dir = os.path.join(d, "data")
    assert datfiles.read_start(os.path.join(data_dir, "Nmr_start.dat")) == (14, 12, 10)
    mask = geometry.sphere_pack((10, 12, 14), 2.5, 0.3, seed=3)
    got = datfiles.read_poro(os.path.join(data_dir, "Poro.dat"), 14, 12, 10)
    assert np.array_equal(got, mask)
    assert abs(summary["porosity"] - mask.mean()) < 1e-12
    vel = geometry.curl_velocity(mask, 4.0, 1e-3, seed=4)
    for a, b in zip(datfiles.read_velocity(data_dir, 14, 12, 10), vel):
        assert np.array_equal(a, b)
    data = datfiles.read_data(os.path.join(data_dir, "Nmr_data.dat"))
    assert data.time2 == 1e-3 and data.n_sequence == 9 and data.n_velocity == 1


def test_presets_and_two_components(tmp_path):
    from initializator_gb300 import datfiles
    d = str(tmp_path / "c1")
    # the c1 preset's physics on a small grid
    out = run_gen(d, "--preset", "c1", "--shape", "16", "16", "16", "--seed", "1")
    assert out.returncode == 0, out.stderr
    data = datfiles.read_data(os.path.join(d, "data", "Nmr_data.dat"))
    assert data.n_velocity == 0 and data.r1_water == 1e-5 and data.d_water == 2.3e-9
    assert not os.path.exists(os.path.join(d, "data", "Vx.dat"))
    d2 = str(tmp_path / "two")
    out = run_gen(d2, "--shape", "8", "6", "5", "--geometry", "open", "--set", "n_components=2", "--n1", "0.7")
    assert out.returncode == 0, out.stderr
    n1 = datfiles.read_n1(os.path.join(d2, "data", "n1_init.dat"), 8, 6, 5)
    assert n1.shape == (5, 6, 8) and np.all(n1 == np.float32(0.7))


def test_surfrel_files(tmp_path):
    """Face relaxivity files for water: constant values with a seeded spread,
    read back in the package's face layout; nSurfRelWater switched on."""
    from initializator_gb300 import datfiles
    d = str(tmp_path / "s")
    out = run_gen(d, "--shape", "6", "5", "4", "--geometry", "open", "--surfrel-water", "1e-5", "2e-5",
                  "--surfrel-spread", "0.2", "--seed", "9")
    assert out.returncode == 0, out.stderr
    assert json.loads(out.stdout.strip().splitlines()[-1])["surfrel"] == ["1Water", "2Water"]
    data_dir = os.path.join(d, "data")
    data = datfiles.read_data(os.path.join(data_dir, "Nmr_data.dat"))
    assert data.n_surf_rel_water == 1 and data.n_surf_rel_oil == 0
    fx, fy, fz = datfiles.read_surfrel(data_dir, "2Water", 6, 5, 4)
    assert fx.shape == (4, 5, 7) and fy.shape == (4, 6, 6) and fz.shape == (5, 5, 6)
    for a in (fx, fy, fz):
        assert np.all(a >= 2e-5 * 0.8) and np.all(a <= 2e-5 * 1.2) and a.std() > 0
    assert not os.path.exists(os.path.join(data_dir, "SurfRel1OilX.dat"))


@pytest.mark.parametrize("args", [
    ["--shape", "4", "4", "4"],                                       # no geometry
    ["--shape", "4", "4", "4", "--geometry", "spheres"],              # no radius / solid fraction
    ["--shape", "4", "4", "4", "--geometry", "open", "--set", "bogus=1"],
    ["--shape", "4", "4", "4", "--geometry", "open", "--set", "n_components=2"],  # no n1
    ["--shape", "4", "4", "4", "--geometry", "open", "--set", "n_surf_rel_oil=1"],  # no oil relaxivities
])
def test_rejects_incomplete_cases(tmp_path, args):
    out = run_gen(str(tmp_path / "x"), *args)
    assert out.returncode != 0
    assert not os.path.exists(str(tmp_path / "x" / "data" / "Poro.dat"))


def test_dropin_init_reads_generated_case(tmp_path, btlib):
    """The drop-in NmrRelaxationSolve::init() (the reference's set-up and file
    readers) runs on a generated directory with flow and derives a positive
    time step and step count."""
    from dropin import describe
    d = str(tmp_path / "case")
    out = run_gen(d, "--shape", "12", "10", "8", "--geometry", "grf", "--sigma", "1.5", "--porosity", "0.5",
                  "--flow", "5e-4", "--seed", "2", "--set", "time2=2e-4")
    assert out.returncode == 0, out.stderr
    r = describe(d)
    assert r["dTime"][0] > 0 and int(r["nStep"][0]) >= 1
