"""The learned coarse relaxation closure on the GPU (initializator_gb300/rate_closure.py).

What the trained network gains over the method without it: on held-out seeds
(a sphere pack and a Gaussian random field not seen in training, with flow
and surface relaxation, no gradient), the coarse solve corrected by the
network misses the FP64 fine M(t) by less than half of what the plain coarse
solve misses (the committed weights, 32 training samples, over 1000 fine
steps: 3.55e-2 -> 2.3e-3 and 4.92e-2 -> 6.2e-3; here 4 training samples, 352
fine steps and a shorter training). Also:
an untrained network (zero last layer) leaves the coarse solve bit for bit
as it is, and the a-posteriori training lowers the training samples' own
rollout error.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPE = (64, 64, 64)
N_COARSE = 88


@pytest.fixture(scope="module")
def trained():
    from initializator_gb300 import closure as C
    from initializator_gb300 import rate_closure as R
    rcs, refs = [], []
    for i in range(4):
        case = C.Case.pgse(SHAPE, seed=100 + 7 * i, kind="sphere" if i % 2 == 0 else "grf", g_amp=0.0,
                           n_coarse=N_COARSE, device="cuda")
        rcs.append(R.RateCase(case, N_COARSE))
        refs.append(case.reference_mt(N_COARSE, precision=0))
    log = []
    clo, losses = R.train(rcs, refs, outer=4, inner=60, lr=1e-3, lr_end=1e-4, damp=1e-4, log=log.append)
    return R, C, clo, log


def test_untrained_network_leaves_the_coarse_solve(btlib):
    from initializator_gb300 import closure as C
    from initializator_gb300 import rate_closure as R
    case = C.Case.pgse((32, 32, 32), seed=3, kind="sphere", g_amp=0.1, n_coarse=24, device="cuda")
    rc = R.RateCase(case, 24)
    clo = R.RateClosure(C.Net(seed=1, zero_last=True))
    corr, _, _ = clo.predict([rc])
    assert float(corr.abs().max()) == 0.0
    plain, _ = rc.rollout(None)
    same, _ = rc.rollout(corr[0].double().cpu().numpy())
    assert np.array_equal(plain, same)


def test_training_lowers_the_rollout_error(trained, btlib):
    R, C, clo, log = trained
    assert log[-1]["rollout_err"] < 0.5 * log[0]["rollout_err"], log


@pytest.mark.parametrize("kind,seed", [("sphere", 900), ("grf", 901)])
def test_closure_beats_plain_coarse_on_held_out_seeds(trained, kind, seed, btlib):
    R, C, clo, _ = trained
    case = C.Case.pgse(SHAPE, seed=seed, kind=kind, g_amp=0.0, n_coarse=N_COARSE, device="cuda")
    rc = R.RateCase(case, N_COARSE)
    ref = case.reference_mt(N_COARSE)
    plain, _ = rc.rollout(None)
    corr, _, _ = clo.predict([rc])
    learned, _ = rc.rollout(corr[0].double().cpu().numpy())
    e_plain, e_learned = R.mt_error(plain, ref), R.mt_error(learned, ref)
    assert e_learned < 0.5 * e_plain, (e_learned, e_plain)


def test_palette_upload_equals_per_voxel_rates(trained, btlib):
    """The timed path hands the corrected rates over as a rate palette formed
    on the GPU; the rollout path as per-voxel host arrays. Same M(t), bit for
    bit."""
    R, C, clo, _ = trained
    case = C.Case.pgse((32, 32, 32), seed=77, kind="sphere", g_amp=0.0, n_coarse=24, device="cuda")
    rc = R.RateCase(case, 24)
    corr, _, _ = clo.predict([rc])
    mts = []
    for c in (corr[0].double().cpu().numpy(), corr[0]):
        s = rc.solver(c)
        mts.append(s.run(24))
        s.close()
    assert np.array_equal(mts[0], mts[1])


def test_fine_check_falls_back_on_a_broken_closure(trained, btlib):
    """The periodic fine check (prolong the coarse field, 4 fine steps,
    compare the change of the lab-frame sums): the trained closure passes
    every check; a broken correction (5 rho/dx_f more surface relaxation in
    every pore voxel) fails the first one, the curve goes on on the fine
    solver, and its error against the FP64 fine M(t) is less than half of the
    unchecked broken solve's."""
    import torch
    R, C, clo, _ = trained
    case = C.Case.pgse(SHAPE, seed=903, kind="sphere", g_amp=0.0, n_coarse=N_COARSE, device="cuda")
    rc = R.RateCase(case, N_COARSE)
    ref = case.reference_mt(N_COARSE)
    corr, _, _ = clo.predict([rc])
    good, fell = R.solve_checked(rc, corr[0], check_every=11)
    assert fell is None
    plain, _ = rc.rollout(None)
    assert R.mt_error(good, ref) < 0.5 * R.mt_error(plain, ref)
    broken = 5.0 * torch.as_tensor(rc.mask > 0, device=corr.device, dtype=torch.float32)
    bad, fell_bad = R.solve_checked(rc, broken, check_every=10 ** 9)
    assert fell_bad is None
    chk, fell = R.solve_checked(rc, broken, check_every=11)
    assert fell == 11
    assert R.mt_error(chk, ref) < 0.5 * R.mt_error(bad, ref), (R.mt_error(chk, ref), R.mt_error(bad, ref))
