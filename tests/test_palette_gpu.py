"""Per-voxel relaxation rates on the FP32 fast path (the rate palette).

When the uploaded per-voxel rates take at most 256 FP32 (dt/T1, dt/T2) pairs
over the pore voxels and the pore diffusivity is the configuration's, the
fast path reads each voxel's pair from a palette through a per-voxel index
(staged by TMA with the geometry code) instead of handing the run to the
generic kernel, which reads eight per-voxel fields. Bars (written here):
fields and M(t) within 1e-5 of the generic FP32 kernel (same update, another
FP32 operation order), on both schemes and both tile widths; rates with more
than 256 pairs, or a pore diffusivity that varies, stay on the generic kernel
(bit-identical to it). Which kernel ran is read from the launch count: a run
of fast steps adds closing launches (one per 32-step graph).
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-5


def rel_err(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _case(shape, seed, nclass, scheme):
    import initializator_gb300 as bt
    from initializator_gb300 import geometry
    mask = geometry.sphere_pack(shape, 3.0, 0.3, seed=seed)
    vel = geometry.curl_velocity(mask, 2.0, 1e-3, seed=seed + 1)
    rng = np.random.default_rng(seed)
    cls = rng.integers(0, nclass, shape)
    t1 = np.where(mask > 0, 0.05 + 0.01 * cls, 1e50)
    t2 = np.where(mask > 0, 0.02 + 0.004 * cls, 1e50)
    dt = geometry.stable_dt(1e-6, 2.3e-9)
    kw = dict(dx=1e-6, dt=dt, d_pore=2.3e-9, t1=2.5, t2=2.0, rho1=1e-5, rho2=1e-5, p_eq=1.0, velocity=1,
              diffusion=1)
    diff = np.where(mask > 0, kw["d_pore"], 1e-25)
    wave, rf = None, []
    if scheme == bt.BT_SCHEME_KSPACE:
        kw.update(gamma=bt.GAMMA_PROTON)
        wave = bt.kspace_waveform_pgse(96, dt, 0.1, 8 * dt, 48 * dt, axis=(0.0, 0.0, 1.0))
        rf = [(bt.pgse_refocus_step(dt, 48 * dt), 2, math.pi, (1.0, 0.0, 0.0))]
    else:
        kw.update(main_field=(0.2, 0.3, 0.9), grad=(0.02, -0.03, 0.05), vector_mult=1)
    st0 = np.zeros((3,) + shape)
    st0[0] = mask
    return mask, vel, st0, kw, (t1, t2, diff), wave, rf


def _run(shape, case, scheme, no_tma, monkeypatch, n=96):
    import initializator_gb300 as bt
    mask, vel, st0, kw, rates, wave, rf = case
    if no_tma:
        monkeypatch.setenv("BT_NO_TMA", "1")
    else:
        monkeypatch.delenv("BT_NO_TMA", raising=False)
    with bt.Solver(bt.make_config(shape, precision=bt.BT_F32, scheme=scheme, **kw)) as s:
        s.upload_geometry(mask, vel)
        s.upload_rates(*rates)
        s.set_schedule(rf, grad_wave=wave)
        s.set_state(st0)
        l0 = s.launches
        mt = s.run(n)
        return s.get_state(), mt, s.launches - l0


@pytest.mark.parametrize("scheme", [0, 1])
@pytest.mark.parametrize("shape", [(24, 20, 120), (20, 33, 40)])
def test_palette_fast_path_matches_generic(shape, scheme, btlib, monkeypatch):
    case = _case(shape, seed=17 + sum(shape), nclass=7, scheme=scheme)
    st_g, mt_g, n_g = _run(shape, case, scheme, True, monkeypatch)
    st_f, mt_f, n_f = _run(shape, case, scheme, False, monkeypatch)
    assert n_f > n_g, (n_g, n_f)  # the fast path ran (its closing launches)
    assert rel_err(st_f, st_g) <= TOL
    assert rel_err(mt_f, mt_g) <= TOL


def test_rates_beyond_the_palette_stay_generic(btlib, monkeypatch):
    shape = (16, 24, 40)
    scheme = 1
    case = _case(shape, seed=5, nclass=300, scheme=scheme)
    st_g, mt_g, n_g = _run(shape, case, scheme, True, monkeypatch)
    st_f, mt_f, n_f = _run(shape, case, scheme, False, monkeypatch)
    assert n_f == n_g
    assert np.array_equal(st_f, st_g) and np.array_equal(mt_f, mt_g)
    # a pore diffusivity that differs from the configuration's: generic too
    mask, vel, st0, kw, (t1, t2, diff), wave, rf = _case(shape, seed=6, nclass=3, scheme=scheme)
    diff = np.where(mask > 0, kw["d_pore"] * (1.0 + 0.1 * (np.arange(mask.size).reshape(shape) % 2)), 1e-25)
    case2 = (mask, vel, st0, kw, (t1, t2, diff), wave, rf)
    st_g, mt_g, n_g = _run(shape, case2, scheme, True, monkeypatch)
    st_f, mt_f, n_f = _run(shape, case2, scheme, False, monkeypatch)
    assert n_f == n_g
    assert np.array_equal(st_f, st_g)


def test_geometry_upload_drops_rates(btlib, monkeypatch):
    """A new geometry drops per-voxel rates (palette and per-voxel fields):
    the run then equals one with the configuration's uniform rates."""
    import initializator_gb300 as bt
    shape = (16, 24, 40)
    for nclass in (7, 300):
        mask, vel, st0, kw, rates, wave, rf = _case(shape, seed=9, nclass=nclass, scheme=0)
        mts = []
        for with_rates in (False, True):
            with bt.Solver(bt.make_config(shape, precision=bt.BT_F32, scheme=0, **kw)) as s:
                s.upload_geometry(mask, vel)
                if with_rates:
                    s.upload_rates(*rates)
                    s.upload_geometry(mask, vel)
                s.set_state(st0)
                mts.append(s.run(40))
        assert np.array_equal(mts[0], mts[1])


@pytest.mark.parametrize("scheme", [0, 1])
def test_palette_upload_matches_per_voxel_rates(scheme, btlib, monkeypatch):
    """bt_upload_rate_palette (entries + a device index) gives the same run,
    bit for bit, as bt_upload_rates with each voxel's entry spelled out; FP64
    handles refuse it."""
    import torch

    import initializator_gb300 as bt
    shape = (20, 33, 40)
    mask, vel, st0, kw, _, wave, rf = _case(shape, seed=23, nclass=5, scheme=scheme)
    rng = np.random.default_rng(4)
    cls = rng.integers(0, 9, shape)
    e1 = 0.04 + 0.013 * np.arange(9)
    e2 = 0.015 + 0.005 * np.arange(9)
    t1 = np.where(mask > 0, e1[cls], 1e50)
    t2 = np.where(mask > 0, e2[cls], 1e50)
    diff = np.where(mask > 0, kw["d_pore"], 1e-25)
    out = []
    for use_palette in (False, True):
        with bt.Solver(bt.make_config(shape, precision=bt.BT_F32, scheme=scheme, **kw)) as s:
            s.upload_geometry(mask, vel)
            if use_palette:
                s.upload_rate_palette(e1, e2, torch.as_tensor(cls.astype(np.uint8), device="cuda"))
            else:
                s.upload_rates(t1, t2, diff)
            s.set_schedule(rf, grad_wave=wave)
            s.set_state(st0)
            mt = s.run(64)
            out.append((s.get_state(), mt))
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    with bt.Solver(bt.make_config(shape, precision=bt.BT_F64, scheme=scheme, **kw)) as s:
        s.upload_geometry(mask, vel)
        with pytest.raises(bt.BtError):
            s.upload_rate_palette(e1, e2, torch.as_tensor(cls.astype(np.uint8), device="cuda"))


def test_new_entry_points_check_their_arguments(btlib):
    """bt_upload_rate_palette refuses 0 or more than 256 entries and a call
    before the geometry; bt_set_tma_chunks clamps any count to a valid
    chunking (fields bit-identical, M(t) within 1e-6: only the grouping of
    the FP32 sums changes)."""
    import torch

    import initializator_gb300 as bt
    shape = (16, 20, 40)
    mask, vel, st0, kw, _, wave, rf = _case(shape, seed=41, nclass=3, scheme=0)
    idx = torch.zeros(shape, dtype=torch.uint8, device="cuda")
    with bt.Solver(bt.make_config(shape, precision=bt.BT_F32, **kw)) as s:
        with pytest.raises(bt.BtError):
            s.upload_rate_palette([0.1], [0.05], idx)  # before the geometry
        s.upload_geometry(mask, vel)
        with pytest.raises(bt.BtError):
            s.upload_rate_palette(np.zeros(0), np.zeros(0), idx)
        with pytest.raises(bt.BtError):
            s.upload_rate_palette(np.full(257, 0.1), np.full(257, 0.05), idx)
        s.set_state(st0)
        ref = s.run(20)
        ref_st = s.get_state()
        for ch in (-5, 1, 10 ** 7):
            s.set_chunks(ch)
            s.set_state(st0)
            s.set_step(0)
            mt = s.run(20)
            assert np.array_equal(s.get_state(), ref_st)
            assert rel_err(mt, ref) <= 1e-6
