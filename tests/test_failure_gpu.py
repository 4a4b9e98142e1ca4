"""Failure detection on the GPU without a GPU fault.

The FP32 fast path bounds every mbarrier wait of its plane ring. A test hook
(bt_set_wait_polls) lowers that bound to zero polls, so every wait gives up at
once on a healthy copy: each CTA raises its failure flag, drains its own copies
in flight with the full bound, and exits; the run reports BT_E_TIMEOUT. After
the bound is restored the same handle, given its field again, runs exactly as
a fresh handle does. Nothing here faults, traps or hangs: the copies are
ordinary in-bounds copies that complete, only the waits stop polling early.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _case():
    import initializator_gb300 as bt
    from initializator_gb300 import geometry
    shape = (48, 24, 128)
    mask = geometry.sphere_pack(shape, 4.0, 0.3, seed=71)
    vel = geometry.curl_velocity(mask, 3.0, 1e-3, seed=72)
    dt = geometry.stable_dt(1e-6, 2.3e-9)
    n = 70
    wave = bt.kspace_waveform_pgse(n + 8, dt, 0.1, 10 * dt, 40 * dt, axis=(0.0, 0.0, 1.0))
    rf = [(bt.pgse_refocus_step(dt, 40 * dt), 2, math.pi, (1.0, 0.0, 0.0))]
    kw = dict(dx=1e-6, dt=dt, d_pore=2.3e-9, t1=2.5, t2=2.0, rho1=1e-5, rho2=1e-5, p_eq=1.0, velocity=1,
              diffusion=1, gamma=bt.GAMMA_PROTON)
    cfg = bt.make_config(shape, precision=bt.BT_F32, scheme=bt.BT_SCHEME_KSPACE, **kw)
    st0 = np.zeros((3,) + shape)
    st0[0] = mask
    return cfg, mask, vel, wave, rf, st0, n


def test_tma_wait_timeout_reports_and_recovers(btlib):
    import initializator_gb300 as bt
    cfg, mask, vel, wave, rf, st0, n = _case()
    with bt.Solver(cfg) as ref:
        ref.upload_geometry(mask, vel)
        ref.set_schedule(rf, grad_wave=wave)
        ref.set_state(st0)
        mt_ref = ref.run(n)
        st_ref = ref.get_state()
    with bt.Solver(cfg) as s:
        s.upload_geometry(mask, vel)
        s.set_schedule(rf, grad_wave=wave)
        s.set_state(st0)
        s.set_wait_polls(0)
        with pytest.raises(bt.BtError) as ei:
            s.run(n)
        assert ei.value.code == -6, str(ei.value)          # BT_E_TIMEOUT
        assert "bounded device wait" in str(ei.value)
        # the bound restored, the field given again: a normal run
        s.set_wait_polls(-1)
        s.set_step(0)
        s.set_state(st0)
        mt = s.run(n)
        st = s.get_state()
    assert np.array_equal(st, st_ref)
    assert np.array_equal(mt, mt_ref)


def test_tma_wait_timeout_twice_in_a_row(btlib):
    """Two failing runs back to back leave the device and the handle usable."""
    import initializator_gb300 as bt
    cfg, mask, vel, wave, rf, st0, n = _case()
    with bt.Solver(cfg) as s:
        s.upload_geometry(mask, vel)
        s.set_schedule(rf, grad_wave=wave)
        s.set_state(st0)
        s.set_wait_polls(0)
        for _ in range(2):
            s.set_step(0)
            with pytest.raises(bt.BtError) as ei:
                s.run(40)
            assert ei.value.code == -6
        s.set_wait_polls(-1)
        s.set_step(0)
        s.set_state(st0)
        mt = s.run(40)
    assert np.all(np.isfinite(mt))
