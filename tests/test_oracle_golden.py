"""The oracle against the reference's own outputs (tests/golden, made by
tests/golden/make_golden.py from oracle/_ref, the reference's CPU path).

Bar: per-voxel fields bit-identical (the oracle keeps the reference's
operation order, -ffp-contract=off); M(t) within 1e-13 relative (the oracle
adds per-plane partial sums, the reference keeps one running sum)."""
import numpy as np
import pytest

from helpers import CASES, common, initial_state, load, pulses, rel_err, velocity

MT_TOL = 1e-13


@pytest.mark.parametrize("case", CASES)
def test_oracle_matches_reference(case, oracle_lib, btlib):
    import oracle
    z = load(case)
    p = oracle.make_params(z["mask"].shape, **common(z))
    st0 = initial_state(z)
    n = int(z["nsteps"])
    s0, _ = oracle.sums(p, z["mask"], st0)
    st, mt = oracle.run(p, z["mask"], st0, n, vel=velocity(z), pulses=pulses(z))
    assert np.array_equal(st, z["state"]), f"max abs diff {np.abs(st - z['state']).max()}"
    mt_all = np.vstack([s0[None], mt])
    assert rel_err(mt_all, z["mt"]) < MT_TOL


@pytest.mark.parametrize("case", CASES)
def test_oracle_rates_match_reference(case, oracle_lib):
    import oracle
    z = load(case)
    p = oracle.make_params(z["mask"].shape, **common(z))
    t1, t2 = oracle.rates(p, z["mask"])
    assert np.array_equal(t1, z["tau1"]) and np.array_equal(t2, z["tau2"])


def test_oracle_threads_deterministic(oracle_lib):
    import oracle
    z = load("pfg_flow")
    p = oracle.make_params(z["mask"].shape, **common(z))
    a = oracle.run(p, z["mask"], initial_state(z), 10, vel=velocity(z), threads=1)
    b = oracle.run(p, z["mask"], initial_state(z), 10, vel=velocity(z), threads=4)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_oracle_bulk_relaxation_known_answer(oracle_lib):
    """All-pore box, no diffusion gradients: forward Euler decay of a uniform
    transverse field is exactly (1 - dt/T2)^n, the longitudinal recovery
    p_eq + (m0 - p_eq)(1 - dt/T1)^n."""
    import oracle
    shape = (4, 5, 6)
    dt, t1, t2 = 1e-3, 0.05, 0.02
    p = oracle.make_params(shape, dx=1e-6, dt=dt, main_field=(0, 0, 1), t1=t1, t2=t2, p_eq=0.7)
    mask = np.ones(shape, np.uint8)
    st0 = np.zeros((3,) + shape)
    st0[0] = 1.0
    st, mt = oracle.run(p, mask, st0, 25)
    n = np.arange(1, 26)
    ex = 1.0 * (1 - dt / t2) ** n * mask.size
    ez = (0.7 + (0.0 - 0.7) * (1 - dt / t1) ** n) * mask.size
    assert np.allclose(mt[:, 0], ex, rtol=1e-12) and np.allclose(mt[:, 2], ez, rtol=1e-12)


def test_oracle_conservation_no_relaxation(oracle_lib):
    """Reflecting pore walls and domain faces: with no relaxation the total
    magnetization is conserved under diffusion and divergence-free flow is
    not needed for diffusion alone."""
    import oracle
    from initializator_gb300 import geometry
    shape = (10, 11, 12)
    mask = geometry.sphere_pack(shape, 2.0, 0.3, seed=3)
    p = oracle.make_params(shape, dx=1e-6, dt=geometry.stable_dt(1e-6, 2.3e-9), main_field=(0, 0, 1),
                           t1=1e30, t2=1e30)
    rng = np.random.default_rng(0)
    st0 = rng.uniform(0, 1, (3,) + shape) * mask
    s0, _ = oracle.sums(p, mask, st0)
    _, mt = oracle.run(p, mask, st0, 50)
    assert rel_err(mt[-1], s0) < 1e-12


def test_oracle_maccormack_relaxation_known_answer(oracle_lib):
    """MacCormack on bulk relaxation is Heun's method: per step the transverse
    field is multiplied by 1 - h + h^2/2 (h = dt/T2) and the longitudinal
    deviation from p_eq by the same with dt/T1."""
    import oracle
    shape = (4, 5, 6)
    dt, t1, t2, peq = 1e-3, 0.05, 0.02, 0.7
    p = oracle.make_params(shape, dx=1e-6, dt=dt, main_field=(0, 0, 1), t1=t1, t2=t2, p_eq=peq, diffusion=0)
    mask = np.ones(shape, np.uint8)
    st0 = np.zeros((3,) + shape)
    st0[0] = 1.0
    st, mt = oracle.run(p, mask, st0, 25, maccormack=True)
    n = np.arange(1, 26)
    h2, h1 = dt / t2, dt / t1
    assert np.allclose(mt[:, 0], (1 - h2 + h2 * h2 / 2) ** n * mask.size, rtol=1e-12)
    assert np.allclose(mt[:, 2], (peq + (0 - peq) * (1 - h1 + h1 * h1 / 2) ** n) * mask.size, rtol=1e-12)


def test_oracle_maccormack_transports_linear_profile(oracle_lib):
    """Uniform velocity along x, a field linear in x, no relaxation or
    diffusion: predictor and corrector differences are exact for a linear
    profile, so away from the domain faces one step moves it by u*dt."""
    import oracle
    shape = (3, 3, 16)
    dx, dt, u = 1e-6, 1e-4, 2e-3
    p = oracle.make_params(shape, dx=dx, dt=dt, main_field=(0, 0, 1), t1=1e30, t2=1e30, p_eq=0.0, diffusion=0,
                           velocity=1)
    mask = np.ones(shape, np.uint8)
    vx = np.full((3, 3, 17), u)
    vy = np.zeros((3, 4, 16))
    vz = np.zeros((4, 3, 16))
    x = np.arange(16.0)
    st0 = np.zeros((3,) + shape)
    st0[1] = 0.5 + 0.01 * x
    st, _ = oracle.run(p, mask, st0, 1, vel=(vx, vy, vz), maccormack=True)
    expect = 0.5 + 0.01 * x - u * dt / dx * 0.01
    assert np.allclose(st[1][:, :, 2:-2], expect[2:-2], rtol=0, atol=1e-15)
