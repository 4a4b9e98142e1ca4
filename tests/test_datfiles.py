"""The data/*.dat readers and writers (initializator_gb300.datfiles)."""
import numpy as np

from initializator_gb300 import datfiles, geometry


def test_data_roundtrip_and_first_match(tmp_path):
    d = datfiles.NmrData(n_sequence=9, dx=2.5e-6, time1=1.25e-3, cfl=0.01, cfl1=0.02, buffer_y=3)
    p = str(tmp_path / "Nmr_data.dat")
    datfiles.write_data(p, d)
    lines = open(p).read().splitlines()
    assert len(lines) == 61 and all("\t" in l for l in lines)
    assert datfiles.read_data(p) == d
    # the first comment containing a token wins: "CFL" also matches the CFL1 line
    lines[55], lines[56] = lines[56], lines[55]
    open(p, "w").write("\n".join(lines) + "\n")
    assert datfiles.read_data(p).cfl == 0.02


def test_poro_and_velocity_roundtrip(tmp_path):
    mask = geometry.sphere_pack((5, 6, 7), 1.5, 0.3, seed=1)
    vel = geometry.curl_velocity(mask, 1.0, 1e-3, seed=2)
    datfiles.write_case(str(tmp_path), datfiles.NmrData(), mask, vel=vel)
    d = str(tmp_path / "data")
    assert datfiles.read_start(d + "/Nmr_start.dat") == (7, 6, 5)
    assert np.array_equal(datfiles.read_poro(d + "/Poro.dat", 7, 6, 5), mask)
    for a, b in zip(datfiles.read_velocity(d, 7, 6, 5), vel):
        assert np.array_equal(a, b)


def test_curl_velocity_is_divergence_free_before_masking():
    mask = np.ones((6, 7, 8), np.uint8)
    vx, vy, vz = geometry.curl_velocity(mask, 1.5, 1.0, seed=3)
    div = (vx[:, :, 1:] - vx[:, :, :-1]) + (vy[:, 1:, :] - vy[:, :-1, :]) + (vz[1:] - vz[:-1])
    # interior cells (no boundary face zeroed) carry zero net flux
    # (the potential is FP32, so the cancellation holds to FP32 rounding)
    assert np.abs(div[1:-1, 1:-1, 1:-1]).max() < 1e-5 * np.abs(vx).max()
