"""Ghost-layer kinds of the library (bt_config.boundary: copy, periodic,
zero per axis) against the oracle, on the GPU.

Bars (written here, checked below):
  REFERENCE and MACCORMACK schemes, FP64: fields bit-identical to the oracle's
      restatement (whose periodic and zero layers are pinned to the
      reference's BC_Inf_* / BC_Advanced_* kernels in test_ref_gpu.py),
      M(t) <= 1e-12 relative;
  KSPACE, FP64: <= 1e-10 against the oracle's lab-frame exact rotation (the
      k frame moves a periodic neighbour across the period by exp(-i k L));
  FP32 (REFERENCE and KSPACE): M(t) <= 1e-4 relative to FP64.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MODES = [(1, 1, 1), (2, 1, 0), (0, 2, 1), (1, 0, 2)]


def _case(shape=(18, 20, 40), seed=31):
    from initializator_gb300 import geometry
    mask = geometry.sphere_pack(shape, 3.0, 0.25, seed=seed)
    vel = geometry.curl_velocity(mask, 2.0, 1e-3, seed=seed + 1)
    st0 = np.zeros((3,) + shape)
    st0[0] = mask
    st0[1] = 0.3 * mask
    return mask, vel, st0


def _kw(**over):
    from initializator_gb300 import geometry
    kw = dict(dx=1e-6, dt=geometry.stable_dt(1e-6, 2.3e-9), main_field=(0.0, 0.0, 1.0), grad=(0.01, 0.0, 0.04),
              d_pore=2.3e-9, t1=0.5, t2=0.2, rho1=1e-5, rho2=1e-5, p_eq=1.0, vector_mult=1, velocity=1,
              diffusion=1)
    kw.update(over)
    return kw


def _rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("modes", MODES)
@pytest.mark.parametrize("scheme", ["reference", "maccormack"])
def test_f64_boundaries_match_oracle(modes, scheme, btlib, oracle_lib):
    import initializator_gb300 as bt
    import oracle
    mask, vel, st0 = _case()
    kw = _kw()
    pulses = [(7, 2, 0.5 * math.pi, (1.0, 0.0, 0.0))]
    n = 24
    mac = scheme == "maccormack"
    ref, ref_mt = oracle.run(oracle.make_params(mask.shape, boundary=modes, **kw), mask, st0, n, vel=vel,
                             pulses=pulses, maccormack=mac)
    sch = bt.BT_SCHEME_MACCORMACK if mac else bt.BT_SCHEME_REFERENCE
    with bt.Solver(bt.make_config(mask.shape, precision=bt.BT_F64, scheme=sch, boundary=modes, **kw)) as s:
        s.upload_geometry(mask, vel)
        s.set_state(st0)
        s.set_schedule(pulses)
        mt = s.run(n)
        st = s.get_state()
    assert np.array_equal(st, ref), f"{scheme} {modes}: {np.abs(st - ref).max():.3e}"
    assert _rel(mt, ref_mt) <= 1e-12


def _kspace_case(modes, n):
    import initializator_gb300 as bt
    mask, vel, st0 = _case()
    dt = _kw()["dt"]
    # a gradient along each axis in turn, so every periodic face sees a phase
    w = bt.kspace_waveform_pgse(n + 2, dt, 0.08, 6 * dt, 14 * dt, axis=(0.6, 0.5, 0.62))
    rf = [(bt.pgse_refocus_step(dt, 14 * dt), 2, math.pi, (1.0, 0.0, 0.0))]
    kw = dict(dx=1e-6, dt=dt, d_pore=2.3e-9, t1=2.5, t2=2.0, rho1=1e-5, rho2=1e-5, p_eq=1.0, velocity=1,
              diffusion=1, gamma=bt.GAMMA_PROTON, boundary=modes)
    return mask, vel, st0, w, rf, kw


@pytest.mark.parametrize("modes", MODES)
def test_kspace_f64_boundaries_match_oracle_physics(modes, btlib, oracle_lib):
    import initializator_gb300 as bt
    import oracle
    n = 40
    mask, vel, st0, w, rf, kw = _kspace_case(modes, n)
    p = oracle.make_params(mask.shape, main_field=(0, 0, 1), vector_mult=2, **kw)
    ref, ref_mt = oracle.run(p, mask, st0, n, vel=vel, pulses=rf, grad_wave=w[:n])
    with bt.Solver(bt.make_config(mask.shape, precision=bt.BT_F64, scheme=bt.BT_SCHEME_KSPACE, **kw)) as s:
        s.upload_geometry(mask, vel)
        s.set_schedule(rf, grad_wave=w)
        s.set_state(st0)
        mt = s.run(n)
        st = s.get_state()
    assert _rel(st, ref) <= 1e-10, f"{modes}: {_rel(st, ref):.3e}"
    assert _rel(mt, ref_mt) <= 1e-10


@pytest.mark.parametrize("modes", MODES)
@pytest.mark.parametrize("scheme", ["reference", "kspace"])
def test_f32_boundaries_mt(modes, scheme, btlib):
    import initializator_gb300 as bt
    n = 40
    if scheme == "kspace":
        mask, vel, st0, w, rf, kw = _kspace_case(modes, n)
        sch, sched = bt.BT_SCHEME_KSPACE, dict(pulses=rf, grad_wave=w)
    else:
        mask, vel, st0 = _case()
        kw = dict(_kw(), boundary=modes)
        sch, sched = bt.BT_SCHEME_REFERENCE, dict(pulses=[(7, 2, 0.5 * math.pi, (1.0, 0.0, 0.0))])
    mts = {}
    for prec in (bt.BT_F64, bt.BT_F32):
        with bt.Solver(bt.make_config(mask.shape, precision=prec, scheme=sch, **kw)) as s:
            s.upload_geometry(mask, vel)
            s.set_schedule(**sched)
            s.set_state(st0)
            mts[prec] = s.run(n)
    assert _rel(mts[bt.BT_F32], mts[bt.BT_F64]) <= 1e-4
