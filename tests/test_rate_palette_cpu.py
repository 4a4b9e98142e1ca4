"""The learned closure's two hand-overs of its corrected rates (CPU only):
per-voxel host arrays (RateCase.rates, the rollout's path) and a rate palette
(RateCase.palette_device, the timed path: entries and a per-voxel level,
formed with torch) give every pore voxel the same T1 and T2 bit for bit, take
at most 255 levels, and leave the plain coarse rates (no correction) exactly
as they are."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def rc():
    from initializator_gb300 import closure as C
    from initializator_gb300 import rate_closure as R
    case = C.Case.pgse((32, 32, 32), seed=3, kind="sphere", g_amp=0.0, n_coarse=12, device="cpu")
    return R.RateCase(case, 12)


@pytest.mark.parametrize("scale", [0.0, 0.3, 2.5])
def test_palette_matches_per_voxel_rates(rc, scale):
    import torch
    rng = np.random.default_rng(int(scale * 10))
    # the network's correction is FP32; both paths widen it to FP64
    corr = torch.as_tensor(scale * rng.standard_normal(rc.shape) * (rc.mask > 0), dtype=torch.float32)
    e1, e2, idx = rc.palette_device(corr)
    t1, t2, diff = rc.rates(corr.double().numpy())
    pore = rc.mask > 0
    lev = idx.numpy().astype(np.int64)
    assert e1.size <= 255 and lev[pore].max() < e1.size
    assert np.array_equal(e1[lev][pore], t1[pore]) and np.array_equal(e2[lev][pore], t2[pore])
    assert np.all(diff[pore] == rc.kw["d_pore"])


def test_plain_rates_unchanged_by_rounding(rc):
    t1_plain, t2_plain, _ = rc.rates(None)
    t1_zero, t2_zero, _ = rc.rates(np.zeros(rc.shape))
    assert np.array_equal(t1_plain, t1_zero) and np.array_equal(t2_plain, t2_zero)
