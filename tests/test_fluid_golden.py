"""Per-voxel fluid coefficients (SurfRel*.dat face relaxivities, two-component
fluids) against the reference's own set-up and update (fixtures surfrel and
two_phase from tests/golden/make_golden.py, the reference's CPU path).

Bars: the host restatement of FillInConcentration / ReadSurfRel /
FillInDiffusinAndTime is bit-identical to the reference's arrays; the oracle
stepping with those per-voxel arrays is bit-identical per voxel, its M(t)
within 1e-13 (one-component sums) and 1e-12 (two-component sums)."""
import dataclasses

import numpy as np
import pytest

from helpers import common, initial_state, load, pulses, rel_err, velocity

FIELD_CASES = ["surfrel", "two_phase"]


def nmr_data(z):
    from initializator_gb300 import datfiles
    kw = {}
    for f in dataclasses.fields(datfiles.NmrData):
        v = z["data_" + f.name]
        kw[f.name] = int(v) if f.type in ("int", int) else float(v)
    return datfiles.NmrData(**kw)


def surf_files(z):
    out = {}
    for key in ("1Water", "2Water", "1Oil", "2Oil"):
        if f"surf_{key}_x" in z:
            out[key] = tuple(z[f"surf_{key}_{ax}"] for ax in "xyz")
    return out


def coeffs(z):
    from initializator_gb300 import fluid
    d = nmr_data(z)
    shape = z["mask"].shape
    c0, c1 = fluid.concentrations(d, shape, z.get("n1"))
    p1, p2 = fluid.phase_fractions(d, c0, c1)
    surf = fluid.surface_relaxivities(d, shape, surf_files(z))
    return (c0, c1), (p1, p2), fluid.coefficients(d, z["mask"], p1, p2, surf)


@pytest.mark.parametrize("case", FIELD_CASES)
def test_coefficients_bit_identical(case):
    z = load(case)
    conc, _, (t1, t2, dd) = coeffs(z)
    assert np.array_equal(t1, z["t1f"]) and np.array_equal(t2, z["t2f"])
    assert np.array_equal(dd, z["diff"])
    if "conc" in z:
        assert np.array_equal(conc[0], z["conc"][0]) and np.array_equal(conc[1], z["conc"][1])


@pytest.mark.parametrize("case", FIELD_CASES)
def test_oracle_with_fields_matches_reference(case, oracle_lib):
    import oracle
    z = load(case)
    _, (p1, p2), _ = coeffs(z)
    p = oracle.make_params(z["mask"].shape, **common(z))
    n = int(z["nsteps"])
    two = int(z["data_n_components"]) == 2
    res = oracle.run(p, z["mask"], initial_state(z), n, vel=velocity(z), pulses=pulses(z),
                     fields=(z["t1f"], z["t2f"], z["diff"]), phases=(p1, p2) if two else None)
    st = res[0]
    assert np.array_equal(st, z["state"]), f"max abs diff {np.abs(st - z['state']).max()}"
    if two:
        assert rel_err(res[2], z["mt6"][1:]) < 1e-12
    else:
        assert rel_err(res[1], z["mt"][1:]) < 1e-13


def test_surfrel_changes_the_answer(oracle_lib):
    """The face relaxivities matter: the uniform fluid's coefficients give a
    different field than the reference's SurfRel run."""
    import oracle
    z = load("surfrel")
    p = oracle.make_params(z["mask"].shape, **common(z))
    st, _ = oracle.run(p, z["mask"], initial_state(z), int(z["nsteps"]), vel=velocity(z), pulses=pulses(z))
    assert not np.array_equal(st, z["state"])
