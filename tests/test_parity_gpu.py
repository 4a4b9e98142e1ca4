"""Parity of the CUDA step (through the C ABI) with the reference and the oracle.

Tolerances (written here, checked below):
  FP64 reference scheme  vs reference / oracle: per-voxel |a-b| <= 1e-12 * max|b|
                         (bit-identical in practice: same operation order, no FMA)
  FP32 reference scheme  vs FP64 reference:     M(t) relative error <= 1e-4
  FP64 KSPACE scheme     vs oracle physics mode: <= 1e-10 (phase factors differ in rounding)
  FP32 KSPACE scheme     vs oracle physics mode: M(t) relative error <= 1e-4
"""
import math

import numpy as np
import pytest

from helpers import CASES, common, initial_state, load, pulses, rel_err, velocity

pytestmark = pytest.mark.gpu

F64_TOL = 1e-12
F32_MT_TOL = 1e-4
KS64_TOL = 1e-10


def _solver(z, precision, **over):
    import initializator_gb300 as bt
    kw = common(z)
    kw.update(over)
    s = bt.Solver(bt.make_config(z["mask"].shape, precision=precision, **kw))
    s.upload_geometry(z["mask"], velocity(z) if kw["velocity"] else None)
    return s


@pytest.mark.parametrize("case", CASES)
def test_f64_matches_reference(case, btlib):
    import initializator_gb300 as bt
    z = load(case)
    with _solver(z, bt.BT_F64) as s:
        s.set_state(initial_state(z))
        s.set_schedule(pulses(z))
        m0 = s.measure()
        mt = s.run(int(z["nsteps"]))
        st = s.get_state()
    assert rel_err(st, z["state"]) <= F64_TOL
    assert rel_err(np.vstack([m0[None], mt]), z["mt"]) <= F64_TOL
    # flags 3/4 use cos/sin of huge angles; all other cases reproduce the bits
    if case != "pulses_explicit":
        assert np.array_equal(st, z["state"])


@pytest.mark.parametrize("case", CASES)
def test_f32_mt_matches_reference(case, btlib):
    import initializator_gb300 as bt
    z = load(case)
    with _solver(z, bt.BT_F32) as s:
        s.set_state(initial_state(z))
        s.set_schedule(pulses(z))
        mt = s.run(int(z["nsteps"]))
    assert rel_err(mt, z["mt"][1:]) <= F32_MT_TOL


def _random_case(shape, seed, flow=True, prec=True):
    from initializator_gb300 import geometry
    mask = geometry.sphere_pack(shape, 3.0, 0.3, seed=seed)
    vel = geometry.curl_velocity(mask, 2.0, 1.5e-3, seed=seed + 1) if flow else None
    rng = np.random.default_rng(seed)
    st0 = rng.uniform(-1, 1, (3,) + shape) * mask
    kw = dict(dx=1e-6, dy=1.1e-6, dz=0.9e-6, dt=geometry.stable_dt(1.1e-6, 2.3e-9) * 0.8, main_field=(0.2, 0.3, 0.9),
              grad=(0.02, -0.03, 0.05), d_pore=2.3e-9, t1=0.1, t2=0.05, rho1=3e-5, rho2=5e-5, p_eq=0.5,
              vector_mult=1 if prec else 0, velocity=1 if flow else 0, diffusion=1,
              buffer=(min(1, shape[2] // 2), min(2, shape[1] // 2), 0))
    return mask, vel, st0, kw


@pytest.mark.parametrize("shape", [(1, 1, 1), (1, 5, 7), (3, 1, 40), (33, 9, 65), (40, 37, 35)])
def test_f64_matches_oracle_shapes(shape, btlib, oracle_lib):
    """Ragged tiles, single-cell axes, z-chunk edges, graph replay (70 steps)."""
    import initializator_gb300 as bt
    import oracle
    mask, vel, st0, kw = _random_case(shape, seed=sum(shape))
    mask[0, 0, 0] = 1
    n = 70
    pl = [(5, 2, 0.7, (0.0, 0.6, 0.8)), (33, 1, 2e-3, (0.2, -0.4, 0.9)), (64, 2, math.pi, (1.0, 0.0, 0.0))]
    ref, ref_mt = oracle.run(oracle.make_params(shape, **kw), mask, st0, n, vel=vel, pulses=pl)
    with bt.Solver(bt.make_config(shape, precision=bt.BT_F64, **kw)) as s:
        s.upload_geometry(mask, vel)
        s.set_state(st0)
        s.set_schedule(pl)
        mt = s.run(n)
        st = s.get_state()
    assert rel_err(st, ref) <= F64_TOL
    assert rel_err(mt, ref_mt) <= F64_TOL


def test_f32_matches_oracle_mt(btlib, oracle_lib):
    import initializator_gb300 as bt
    import oracle
    shape = (24, 40, 56)
    mask, vel, st0, kw = _random_case(shape, seed=5)
    st0 = np.abs(st0)
    n = 200
    _, ref_mt = oracle.run(oracle.make_params(shape, **kw), mask, st0, n, vel=vel)
    with bt.Solver(bt.make_config(shape, precision=bt.BT_F32, **kw)) as s:
        s.upload_geometry(mask, vel)
        s.set_state(st0)
        mt = s.run(n)
    assert rel_err(mt, ref_mt) <= F32_MT_TOL


def _kspace_case(shape, seed):
    import initializator_gb300 as bt
    from initializator_gb300 import geometry
    mask = geometry.sphere_pack(shape, 3.0, 0.35, seed=seed)
    vel = geometry.curl_velocity(mask, 2.0, 1e-3, seed=seed + 1)
    dt = geometry.stable_dt(1e-6, 2.3e-9)
    n = 120
    wave = bt.kspace_waveform_pgse(n, dt, 0.1, 10 * dt, 60 * dt, axis=(0.3, -0.2, 1.0))
    kw = dict(dx=1e-6, dt=dt, d_pore=2.3e-9, t1=2.5, t2=2.0, rho1=1e-5, rho2=1e-5, p_eq=1.0, velocity=1,
              diffusion=1, gamma=bt.GAMMA_PROTON)
    st0 = np.zeros((3,) + shape)
    st0[0] = mask
    rf = [(bt.pgse_refocus_step(dt, 60 * dt), 2, math.pi, (1.0, 0.0, 0.0)), (90, 2, 0.5 * math.pi, (0.0, 1.0, 0.0))]
    return mask, vel, st0, kw, wave, rf, n


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_kspace_matches_oracle_physics(precision, btlib, oracle_lib):
    """Exact-precession (k-space frame) kernel vs the oracle's lab-frame exact
    rotation, PGSE lobes along a tilted axis, flow, a 180 and a 90 RF pulse."""
    import initializator_gb300 as bt
    import oracle
    shape = (20, 18, 36)
    mask, vel, st0, kw, wave, rf, n = _kspace_case(shape, seed=9)
    p = oracle.make_params(shape, main_field=(0, 0, 1), vector_mult=2, **kw)
    ref, ref_mt = oracle.run(p, mask, st0, n, vel=vel, pulses=rf, grad_wave=wave)
    prec = bt.BT_F64 if precision == "f64" else bt.BT_F32
    with bt.Solver(bt.make_config(shape, precision=prec, scheme=bt.BT_SCHEME_KSPACE, **kw)) as s:
        s.upload_geometry(mask, vel)
        s.set_schedule(rf, grad_wave=wave)
        s.set_state(st0)
        mt = s.run(n)
        st = s.get_state()
    if precision == "f64":
        assert rel_err(st, ref) <= KS64_TOL
        assert rel_err(mt, ref_mt) <= KS64_TOL
    else:
        assert rel_err(mt, ref_mt) <= F32_MT_TOL


@pytest.mark.parametrize("scheme", [0, 1, 2])
def test_several_pulses_in_one_step(scheme, btlib, oracle_lib):
    """Steps holding several pulses, applied in the order given: three
    fixed-angle pulses (one about an axis that is not a unit vector), which
    FP32 fields take as one product rotation on the fast path, and a
    fixed-angle pulse beside a gradient-dependent one, which both precisions
    take in FP64 on the generic kernels (the fixed angle's cosine and sine
    formed once per CTA; KSPACE takes fixed-angle pulses only, so there the
    second one is fixed-angle too). FP64 fields and M(t) within 1e-12 of the
    oracle (KSPACE: 1e-10, its k-frame bound); FP32 fields and M(t) within
    1e-4."""
    import initializator_gb300 as bt
    import oracle
    pl = [(6, 2, 0.5 * math.pi, (1.0, 0.0, 0.0)), (6, 2, 0.3, (0.0, 0.6, 0.8)), (6, 2, math.pi, (0.2, 0.3, 0.9)),
          (19, 2, 0.7, (0.0, 1.0, 0.0)), (19, 1, 2e-3, (0.2, -0.4, 0.9)), (31, 2, math.pi, (1.0, 0.0, 0.0))]
    n = 40
    if scheme == 1:
        pl[4] = (19, 2, 1.1, (0.3, 0.0, 0.95))
        shape = (20, 18, 36)
        mask, vel, st0, kw, wave, _, _ = _kspace_case(shape, seed=4)
        st0 = np.random.default_rng(4).uniform(-1, 1, (3,) + shape) * mask
        p = oracle.make_params(shape, main_field=(0, 0, 1), vector_mult=2, **kw)
        ref, ref_mt = oracle.run(p, mask, st0, n, vel=vel, pulses=pl, grad_wave=wave)
        sched = dict(grad_wave=wave)
        tol64 = KS64_TOL
    else:
        shape = (17, 22, 30)
        mask, vel, st0, kw = _random_case(shape, seed=8)
        p = oracle.make_params(shape, **kw)
        ref, ref_mt = oracle.run(p, mask, st0, n, vel=vel, pulses=pl, maccormack=scheme == 2)
        sched = {}
        tol64 = F64_TOL
    for prec in (bt.BT_F64, bt.BT_F32):
        with bt.Solver(bt.make_config(shape, precision=prec, scheme=scheme, **kw)) as s:
            s.upload_geometry(mask, vel)
            s.set_schedule(pl, **sched)
            s.set_state(st0)
            mt = s.run(n)
            st = s.get_state()
        if prec == bt.BT_F64:
            assert rel_err(st, ref) <= tol64
            assert rel_err(mt, ref_mt) <= tol64
        else:
            assert rel_err(mt, ref_mt) <= F32_MT_TOL
            assert rel_err(st, ref) <= F32_MT_TOL


@pytest.mark.parametrize("scheme,grad", [(0, True), (1, True), (1, False)])
def test_pulse_steps_on_the_fast_path(scheme, grad, btlib, monkeypatch):
    """FP32 steps whose pulses are all fixed-angle run on the fast path (the
    step's rotation applied before its sums, the run of fast steps going on:
    with a pulse in every 32-step window, n steps take n launches and one
    closing launch) and give the generic kernel's fields and M(t) within
    1e-5: a multi-echo train (a 90 at step 0, then a 180 every 8 steps) with
    flow; KSPACE with a gradient along z and without one, REFERENCE with the
    cross product."""
    import initializator_gb300 as bt
    from initializator_gb300 import geometry
    shape = (40, 24, 48)
    mask = geometry.sphere_pack(shape, 3.0, 0.3, seed=21)
    vel = geometry.curl_velocity(mask, 2.0, 1e-3, seed=22)
    dt = geometry.stable_dt(1e-6, 2.3e-9)
    n = 64
    kw = dict(dx=1e-6, dt=dt, d_pore=2.3e-9, t1=2.5, t2=2.0, rho1=1e-5, rho2=1e-5, p_eq=1.0, velocity=1,
              diffusion=1)
    rf = [(0, 2, 0.5 * math.pi, (0.0, 1.0, 0.0))] + [(q, 2, math.pi, (1.0, 0.0, 0.0)) for q in range(4, n, 8)]
    sched = {}
    if scheme == bt.BT_SCHEME_KSPACE:
        kw.update(gamma=bt.GAMMA_PROTON)
        if grad:
            sched = dict(grad_wave=bt.kspace_waveform_pgse(n, dt, 0.1, 6 * dt, 30 * dt, axis=(0.0, 0.0, 1.0)))
    else:
        kw.update(main_field=(0.2, 0.3, 0.9), grad=(0.02, -0.03, 0.05), vector_mult=1)
    st0 = np.zeros((3,) + shape)
    st0[2] = mask
    out = []
    for no_tma in (True, False):
        if no_tma:
            monkeypatch.setenv("BT_NO_TMA", "1")
        else:
            monkeypatch.delenv("BT_NO_TMA", raising=False)
        with bt.Solver(bt.make_config(shape, precision=bt.BT_F32, scheme=scheme, **kw)) as s:
            s.upload_geometry(mask, vel)
            s.set_schedule(rf, **sched)
            s.set_state(st0)
            l0 = s.launches
            mt = s.run(n)
            n_run = s.launches - l0  # (get_state adds a frame change in KSPACE)
            out.append((s.get_state(), mt, n_run))
    (st_g, mt_g, _), (st_f, mt_f, n_f) = out
    assert n_f == n + 1, n_f
    assert rel_err(st_f, st_g) <= 1e-5
    assert rel_err(mt_f, mt_g) <= 1e-5


def test_kspace_state_roundtrip_mid_gradient(btlib):
    """set_state / get_state convert between the lab frame and the k frame."""
    import initializator_gb300 as bt
    shape = (8, 9, 10)
    mask, vel, st0, kw, wave, rf, n = _kspace_case(shape, seed=2)
    with bt.Solver(bt.make_config(shape, precision=bt.BT_F64, scheme=bt.BT_SCHEME_KSPACE, **kw)) as s:
        s.upload_geometry(mask, vel)
        s.set_schedule(rf, grad_wave=wave)
        s.set_step(7)
        x = np.random.default_rng(1).uniform(-1, 1, (3,) + shape) * mask
        s.set_state(x)
        assert rel_err(s.get_state(), x) < 1e-14
        assert rel_err(s.measure(), x.sum(axis=(1, 2, 3))) < 1e-12


def test_f32_state_transfer_pipeline(btlib):
    """FP32 host transfers convert each component on the host's cores into one
    of two pinned staging halves, alternating halves: a batch of 3 fields (9
    components, so both halves are reused) read back right after set_state is
    the FP32 rounding of the input, member by member; a second set_state at
    once (its halves wait for the first one's copies) leaves the second input;
    the field (2^21 voxels) is large enough for the conversion to use several
    threads."""
    import initializator_gb300 as bt
    shape = (32, 256, 256)
    mask = np.ones(shape, np.uint8)
    rng = np.random.default_rng(5)
    a = rng.standard_normal((3, 3) + shape)
    b = rng.standard_normal((3, 3) + shape)
    with bt.Solver(bt.make_config(shape, dx=1e-6, dt=1e-6, precision=bt.BT_F32, batch=3)) as s:
        s.upload_geometry(mask, None)
        s.set_state(a)
        got = s.get_state()
        assert np.array_equal(got, a.astype(np.float32).astype(np.float64))
        s.set_state(a)
        s.set_state(b)
        assert np.array_equal(s.get_state(), b.astype(np.float32).astype(np.float64))


def test_determinism_and_graph_equivalence(btlib):
    import initializator_gb300 as bt
    shape = (30, 41, 70)
    mask, vel, st0, kw = _random_case(shape, seed=7)
    outs = []
    for chunks in ([96], [96], [1] * 96):
        with bt.Solver(bt.make_config(shape, precision=bt.BT_F32, **kw)) as s:
            s.upload_geometry(mask, vel)
            s.set_state(st0)
            mts = [s.run(c) for c in chunks]
            outs.append((s.get_state(), np.vstack(mts)))
    for st, mt in outs[1:]:
        assert np.array_equal(st, outs[0][0]) and np.array_equal(mt, outs[0][1])


def test_solid_stays_zero_and_all_solid(btlib):
    import initializator_gb300 as bt
    shape = (6, 7, 9)
    mask = np.zeros(shape, np.uint8)
    with bt.Solver(bt.make_config(shape, dx=1e-6, dt=1e-5)) as s:
        s.upload_geometry(mask)
        s.set_state(np.ones((3,) + shape))
        mt = s.run(3)
        assert np.all(mt == 0.0) and np.all(s.get_state() == 0.0)


def test_nan_watchdog(btlib):
    import initializator_gb300 as bt
    shape = (4, 4, 4)
    with bt.Solver(bt.make_config(shape, dx=1e-6, dt=1e-5)) as s:
        s.upload_geometry(np.ones(shape, np.uint8))
        st = np.zeros((3,) + shape)
        st[0, 1, 1, 1] = np.inf
        s.set_state(st)
        with pytest.raises(bt.BtError) as e:
            s.run(2)
        assert e.value.code == -3


def test_conservation_256(btlib):
    """Size-independent property at the 256^3 workload size: with no relaxation
    and reflecting walls, diffusion conserves the total magnetization."""
    import initializator_gb300 as bt
    from initializator_gb300 import geometry
    shape = (256, 256, 256)
    mask = geometry.sphere_pack(shape, 10.0, 0.4, seed=1)
    st0 = np.zeros((3,) + shape)
    st0[0] = mask
    with bt.Solver(bt.make_config(shape, dx=1e-6, dt=geometry.stable_dt(1e-6, 2.3e-9), main_field=(1, 0, 0),
                                  t1=1e30, t2=1e30, p_eq=1.0)) as s:
        s.upload_geometry(mask)
        s.set_state(st0)
        mt = s.run(100)
    assert abs(mt[-1, 0] / mask.sum() - 1.0) < 1e-5


@pytest.mark.parametrize("shape,flow", [((33, 9, 65), True), ((8, 16, 130), True), ((5, 17, 257), True),
                                        ((70, 3, 4), True), ((12, 20, 40), False), ((9, 40, 120), False)])
@pytest.mark.parametrize("scheme", [0, 1])
def test_tma_path_matches_generic(shape, flow, scheme, btlib, monkeypatch):
    """The FP32 TMA fast path (pulse-free steps) against the generic FP32 kernel:
    same update, different FP32 operation order -> fields within 1e-5. Widths
    65 and 120 take 128-wide tiles, 4, 40, 130 and 257 64-wide ones (the width
    that pads x less); with and without flow."""
    import initializator_gb300 as bt
    mask, vel, st0, kw = _random_case(shape, seed=11 + sum(shape), flow=flow)
    if scheme == bt.BT_SCHEME_KSPACE:
        kw.update(main_field=(0, 0, 1), vector_mult=0, gamma=bt.GAMMA_PROTON)
        wave = bt.kspace_waveform_pgse(80, kw["dt"], 0.05, 8 * kw["dt"], 40 * kw["dt"], axis=(0.2, 0.5, 1.0))
    outs = []
    for no_tma in ("1", None):
        if no_tma:
            monkeypatch.setenv("BT_NO_TMA", no_tma)
        else:
            monkeypatch.delenv("BT_NO_TMA", raising=False)
        with bt.Solver(bt.make_config(shape, precision=bt.BT_F32, scheme=scheme, **kw)) as s:
            s.upload_geometry(mask, vel)
            if scheme == bt.BT_SCHEME_KSPACE:
                s.set_schedule([], grad_wave=wave)
            s.set_state(st0)
            mt = s.run(80)
            outs.append((s.get_state(), mt))
    assert rel_err(outs[1][0], outs[0][0]) <= 1e-5
    assert rel_err(outs[1][1], outs[0][1]) <= 1e-5


@pytest.mark.parametrize("axis", [(0.2, 0.5, 1.0), (0.0, 0.0, 1.0), None])
@pytest.mark.parametrize("shape", [(20, 12, 100), (18, 40, 60)])
def test_tma_phase_axes_instances(shape, axis, btlib, monkeypatch):
    """KSPACE fast path picks its instance from the schedule's wave vectors: a
    gradient with x/y components (every face phase), along z only (z phase,
    real x/y weights), none (no phase). Each against the generic FP32 kernel:
    fields and M(t) within 1e-5; with a refocusing pulse so the pulse step's
    generic launch and the fast steps around it share the field."""
    import initializator_gb300 as bt
    mask, vel, st0, kw = _random_case(shape, seed=71 + sum(shape), flow=True)
    kw.update(main_field=(0, 0, 1), vector_mult=0, gamma=bt.GAMMA_PROTON, grad=(0.0, 0.0, 0.0))
    n = 90
    wave = None if axis is None else bt.kspace_waveform_pgse(n, kw["dt"], 0.08, 8 * kw["dt"], 40 * kw["dt"],
                                                               axis=axis)
    rf = [(bt.pgse_refocus_step(kw["dt"], 40 * kw["dt"]), 2, math.pi, (1.0, 0.0, 0.0))]
    outs = []
    for no_tma in ("1", None):
        if no_tma:
            monkeypatch.setenv("BT_NO_TMA", no_tma)
        else:
            monkeypatch.delenv("BT_NO_TMA", raising=False)
        with bt.Solver(bt.make_config(shape, precision=bt.BT_F32, scheme=bt.BT_SCHEME_KSPACE, **kw)) as s:
            s.upload_geometry(mask, vel)
            s.set_schedule(rf, grad_wave=wave)
            s.set_state(st0)
            mt = s.run(n)
            outs.append((s.get_state(), mt))
    assert rel_err(outs[1][0], outs[0][0]) <= 1e-5
    assert rel_err(outs[1][1], outs[0][1]) <= 1e-5


def test_tma_zsplits_and_autotune(btlib, monkeypatch):
    """Any z-chunking of the fast path gives the same field (even chunks never
    come out empty: 38 chunks of 256 planes would leave the last one empty
    without the host's normalisation), and the autotuner restores field and
    step."""
    import initializator_gb300 as bt
    shape = (256, 8, 128)
    mask, vel, st0, kw = _random_case(shape, seed=3)
    fields = []
    for zs in ("1", "5", "38", "200"):
        monkeypatch.setenv("BT_TMA_ZSPLIT", zs)
        with bt.Solver(bt.make_config(shape, precision=bt.BT_F32, **kw)) as s:
            s.upload_geometry(mask, vel)
            s.set_state(st0)
            mt = s.run(40)
            fields.append((s.get_state(), mt))
    for st, mt in fields[1:]:
        assert np.array_equal(st, fields[0][0])
        assert rel_err(mt, fields[0][1]) <= 1e-6
    monkeypatch.delenv("BT_TMA_ZSPLIT")
    with bt.Solver(bt.make_config(shape, precision=bt.BT_F32, **kw)) as s:
        s.upload_geometry(mask, vel)
        s.set_state(st0)
        best = s.autotune(8)
        assert best >= 1 and s.step == 0
        assert rel_err(s.get_state(), st0) <= 1e-7
        s.run(40)
        assert np.array_equal(s.get_state(), fields[0][0])
    # the explicit setter, changed mid-run (0: the default for a handle alone)
    with bt.Solver(bt.make_config(shape, precision=bt.BT_F32, **kw)) as s:
        s.upload_geometry(mask, vel)
        s.set_state(st0)
        s.set_zsplit(5)
        mt_a = s.run(20)
        s.set_zsplit(0)
        mt_b = s.run(20)
        assert np.array_equal(s.get_state(), fields[0][0])
        assert rel_err(np.vstack([mt_a, mt_b]), fields[0][1]) <= 1e-6


def test_tma_uneven_chunks(btlib):
    """Chunk counts that are not a multiple of the tile columns (9 columns of
    64 x 16 here): the first columns get one chunk more, the others leave
    their last grid index empty; changed mid-run, down to 1-plane chunks in
    every column (432 = 9 x 48). Fields bit-identical to the default
    chunking, M(t) within 1e-6."""
    import initializator_gb300 as bt
    shape = (48, 40, 130)
    mask, vel, st0, kw = _random_case(shape, seed=5)
    with bt.Solver(bt.make_config(shape, precision=bt.BT_F32, **kw)) as s:
        s.upload_geometry(mask, vel)
        s.set_state(st0)
        ref = s.run(40)
        ref_st = s.get_state()
    with bt.Solver(bt.make_config(shape, precision=bt.BT_F32, **kw)) as s:
        s.upload_geometry(mask, vel)
        s.set_state(st0)
        mts = []
        for ch in (10, 20, 432, 31):
            s.set_chunks(ch)
            mts.append(s.run(10))
        assert np.array_equal(s.get_state(), ref_st)
        assert rel_err(np.vstack(mts), ref) <= 1e-6


def test_ragged_shared_chunking(btlib):
    """run_many gives handles that share the GPU longer z-chunks than each
    would take alone (here 2 instead of 8 per column for eight 256 x 128 x 64
    grids); fields stay bit-identical to each handle run alone and M(t) agrees
    to 1e-6 (only the FP32 grouping of the per-thread sums changes)."""
    import initializator_gb300 as bt
    shape = (64, 128, 256)
    cases = [_random_case(shape, seed=40 + i, prec=False) for i in range(8)]

    def make(case):
        mask, vel, st0, kw = case
        s = bt.Solver(bt.make_config(shape, precision=bt.BT_F32, **kw))
        s.upload_geometry(mask, vel)
        s.set_state(st0)
        return s

    many = [make(c) for c in cases]
    mts = bt.run_many(many, 40)
    for s, c, mt in zip(many, cases, mts):
        st = s.get_state()
        s.close()
        with make(c) as one:
            mt1 = one.run(40)
            assert np.array_equal(st, one.get_state())
        assert rel_err(mt, mt1) <= 1e-6


@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_batched_q_sweep_matches_single_fields(precision, btlib):
    """A batch of fields with different gradient strengths (one launch per
    step, shared geometry) against the same fields run one at a time: fields
    bit-identical (same per-voxel arithmetic), M(t) to 1e-12 (only the order of
    the FP64 partial sums differs)."""
    import initializator_gb300 as bt
    shape = (20, 18, 36)
    mask, vel, st0, kw, wave, rf, n = _kspace_case(shape, seed=4)
    prec = bt.BT_F64 if precision == "f64" else bt.BT_F32
    amps = [0.0, 0.7, 1.3]
    waves = np.stack([wave * a for a in amps], axis=1)  # (n, B, 3)
    with bt.Solver(bt.make_config(shape, precision=prec, scheme=bt.BT_SCHEME_KSPACE, batch=len(amps), **kw)) as s:
        s.upload_geometry(mask, vel)
        s.set_schedule(rf, grad_wave=waves)
        s.set_state(np.stack([st0] * len(amps)))
        mt = s.run(n)
        st = s.get_state()
        m_end = s.measure()
    for b, a in enumerate(amps):
        with bt.Solver(bt.make_config(shape, precision=prec, scheme=bt.BT_SCHEME_KSPACE, **kw)) as s1:
            s1.upload_geometry(mask, vel)
            s1.set_schedule(rf, grad_wave=wave * a)
            s1.set_state(st0)
            mt1 = s1.run(n)
            st1 = s1.get_state()
        assert np.array_equal(st[b], st1), b
        assert rel_err(mt[:, b], mt1) <= 1e-12, b
        assert rel_err(m_end[b], mt1[-1]) <= 1e-6, b


def test_batched_uneven_chunks(btlib):
    """A q-sweep batch on uneven chunkings (its members' CTAs side by side,
    the short columns' last grid index empty for every member): fields
    bit-identical and M(t) within 1e-6 of the default chunking (only the
    grouping of the per-thread FP32 sums changes)."""
    import initializator_gb300 as bt
    shape = (40, 40, 130)
    mask, vel, st0, kw, wave, rf, n = _kspace_case(shape, seed=14)
    amps = [0.3, 1.0, 1.7]
    waves = np.stack([wave * a for a in amps], axis=1)
    outs = []
    for chunks in (0, 13, 40):
        with bt.Solver(bt.make_config(shape, precision=bt.BT_F32, scheme=bt.BT_SCHEME_KSPACE, batch=len(amps),
                                      **kw)) as s:
            s.upload_geometry(mask, vel)
            s.set_schedule(rf, grad_wave=waves)
            s.set_state(np.stack([st0] * len(amps)))
            s.set_chunks(chunks)
            outs.append((s.run(n), s.get_state()))
    for mt, st in outs[1:]:
        assert np.array_equal(st, outs[0][1])
        assert rel_err(mt, outs[0][0]) <= 1e-6


def test_ragged_batch_matches_single_runs(btlib):
    """run_many over handles of different sizes, precisions, schemes and
    schedules (graph chunks interleaved on separate streams) against each
    handle run alone: fields and M(t) bit-identical; one member also against
    the oracle's physics mode."""
    import initializator_gb300 as bt
    import oracle
    specs = [((20, 18, 36), 5, bt.BT_F32), ((12, 10, 16), 6, bt.BT_F64), ((24, 16, 40), 7, bt.BT_F32),
             ((8, 8, 8), 8, bt.BT_F32)]
    n = 100  # three graph chunks of 32 steps plus single launches around the pulses

    def make(shape, seed, prec):
        mask, vel, st0, kw, wave, rf, nn = _kspace_case(shape, seed)
        s = bt.Solver(bt.make_config(shape, precision=prec, scheme=bt.BT_SCHEME_KSPACE, **kw))
        s.upload_geometry(mask, vel)
        s.set_schedule(rf, grad_wave=wave)
        s.set_state(st0)
        return s, (mask, vel, st0, kw, wave, rf)

    many = [make(*sp) for sp in specs]
    mts = bt.run_many([s for s, _ in many], n)
    states = [s.get_state() for s, _ in many]
    for (s, _), sp, mt, st in zip(many, specs, mts, states):
        s.close()
        one, _ = make(*sp)
        with one:
            mt1 = one.run(n)
            st1 = one.get_state()
        assert np.array_equal(st, st1), sp
        assert np.array_equal(mt, mt1), sp
    mask, vel, st0, kw, wave, rf = many[1][1]
    p = oracle.make_params(specs[1][0], main_field=(0, 0, 1), vector_mult=2, **kw)
    ref, ref_mt = oracle.run(p, mask, st0, n, vel=vel, pulses=rf, grad_wave=wave)
    assert rel_err(states[1], ref) <= KS64_TOL
    assert rel_err(mts[1], ref_mt) <= KS64_TOL


@pytest.mark.parametrize("case", ["surfrel", "two_phase"])
@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_per_voxel_fields_match_reference(case, precision, btlib):
    """SurfRel face relaxivities and two-component fluids: the reference's own
    relTime / diffusion arrays uploaded per voxel. FP64: field bit-identical,
    M(t) (one-component sums, or the six two-component sums) within 1e-12;
    FP32: M(t) within 1e-4."""
    import initializator_gb300 as bt
    from test_fluid_golden import coeffs
    z = load(case)
    two = int(z["data_n_components"]) == 2
    prec = bt.BT_F64 if precision == "f64" else bt.BT_F32
    _, (p1, p2), _ = coeffs(z)
    n = int(z["nsteps"])
    with _solver(z, prec) as s:
        s.upload_rates(z["t1f"], z["t2f"], z["diff"])
        if two:
            s.set_phase_weights(p1, p2)
        s.set_state(initial_state(z))
        s.set_schedule(pulses(z))
        mt = s.run(n)
        st = s.get_state()
        mt6 = s.read_mt_phases(n) if two else None
    tol = F64_TOL if precision == "f64" else F32_MT_TOL
    if precision == "f64":
        assert np.array_equal(st, z["state"]), f"max abs diff {np.abs(st - z['state']).max()}"
    if two:
        assert rel_err(mt6, z["mt6"][1:]) <= tol
    else:
        assert rel_err(mt, z["mt"][1:]) <= tol


def test_per_voxel_fields_reset(btlib):
    """Uploading the reference's coefficient arrays of a uniform-fluid case
    per voxel reproduces the code-table path bit for bit (FP64) and in FP32
    (there through the rate palette on the fast path: M(t) within 1e-6), and
    NULL returns to the code tables."""
    import initializator_gb300 as bt
    z = load("pfg_flow")
    for prec in (bt.BT_F64, bt.BT_F32):
        with _solver(z, prec) as s:
            s.set_state(initial_state(z))
            s.set_schedule(pulses(z))
            ref = s.run(20)
            ref_st = s.get_state()
        with _solver(z, prec) as s:
            s.upload_rates(z["t1f"], z["t2f"], z["diff"])
            s.set_state(initial_state(z))
            s.set_schedule(pulses(z))
            mt = s.run(20)
            if prec == bt.BT_F64:
                assert np.array_equal(s.get_state(), ref_st)
                assert np.array_equal(mt, ref)
            else:
                assert rel_err(mt, ref) <= 1e-6
            s.upload_rates()
            s.set_state(initial_state(z))
            s.set_step(0)
            assert np.array_equal(s.run(20), ref)


@pytest.mark.parametrize("shape", [(9, 7, 13), (16, 12, 40), (5, 33, 70)])
def test_maccormack_matches_oracle(shape, btlib, oracle_lib):
    """The reference's GPU scheme (predictor-corrector, two launches per
    step) against the oracle's restatement, with flow and the cross product:
    FP64 per voxel bit-identical without pulses; with pulses of flags 1 and 2
    (CUDA's and the C library's cos/sin may differ in the last bit) fields and
    M(t) within 1e-12; FP32 M(t) within 1e-4."""
    import initializator_gb300 as bt
    import oracle
    mask, vel, st0, kw = _random_case(shape, seed=sum(shape) + 5)
    n = 40
    p = oracle.make_params(shape, **kw)
    for pl in ([], [(5, 2, 0.7, (0.0, 0.6, 0.8)), (13, 1, 2e-3, (0.2, -0.4, 0.9)), (33, 2, math.pi, (1.0, 0.0, 0.0))]):
        ref, ref_mt = oracle.run(p, mask, st0, n, vel=vel, pulses=pl, maccormack=True)
        for prec in (bt.BT_F64, bt.BT_F32):
            with bt.Solver(bt.make_config(shape, precision=prec, scheme=bt.BT_SCHEME_MACCORMACK, **kw)) as s:
                s.upload_geometry(mask, vel)
                s.set_state(st0)
                s.set_schedule(pl)
                mt = s.run(n)
                st = s.get_state()
                assert s.launches >= 2 * n
            if prec == bt.BT_F64:
                if not pl:
                    assert np.array_equal(st, ref), f"max abs diff {np.abs(st - ref).max()}"
                assert rel_err(st, ref) <= F64_TOL
                assert rel_err(mt, ref_mt) <= F64_TOL
            else:
                assert rel_err(mt, ref_mt) <= F32_MT_TOL


@pytest.mark.parametrize("case", ["surfrel", "two_phase"])
def test_maccormack_per_voxel_fields(case, btlib, oracle_lib):
    """MacCormack with the reference's per-voxel coefficient arrays (and the
    two-component sums) against the oracle: FP64 bit-identical."""
    import initializator_gb300 as bt
    import oracle
    from test_fluid_golden import coeffs
    z = load(case)
    two = int(z["data_n_components"]) == 2
    _, (p1, p2), _ = coeffs(z)
    n = int(z["nsteps"])
    p = oracle.make_params(z["mask"].shape, **common(z))
    res = oracle.run(p, z["mask"], initial_state(z), n, vel=velocity(z), pulses=pulses(z),
                     fields=(z["t1f"], z["t2f"], z["diff"]), phases=(p1, p2) if two else None, maccormack=True)
    with _solver(z, bt.BT_F64, scheme=bt.BT_SCHEME_MACCORMACK) as s:
        s.upload_rates(z["t1f"], z["t2f"], z["diff"])
        if two:
            s.set_phase_weights(p1, p2)
        s.set_state(initial_state(z))
        s.set_schedule(pulses(z))
        mt = s.run(n)
        st = s.get_state()
        mt6 = s.read_mt_phases(n) if two else None
    assert np.array_equal(st, res[0]), f"max abs diff {np.abs(st - res[0]).max()}"
    if two:
        assert rel_err(mt6, res[2]) <= F64_TOL
    else:
        assert rel_err(mt, res[1]) <= F64_TOL


@pytest.mark.parametrize("scheme", [0, 1])
def test_state_upload_beside_running_steps(scheme, btlib):
    """bt_set_state called while queued steps still run (the upload goes
    through the inbox on the transfer stream and is moved in after them)
    gives the same M(t) and fields, bit for bit, as the serial order."""
    import initializator_gb300 as bt
    shape = (24, 30, 70)
    mask, vel, st0, kw = _random_case(shape, seed=31)
    wave = None
    if scheme == bt.BT_SCHEME_KSPACE:
        kw.update(main_field=(0, 0, 1), vector_mult=0, gamma=bt.GAMMA_PROTON)
        # a gradient, so that the second upload's frame change (at step 40)
        # is not the identity
        wave = bt.kspace_waveform_pgse(80, kw["dt"], 0.05, 8 * kw["dt"], 40 * kw["dt"], axis=(0.2, 0.5, 1.0))
    st1 = np.roll(st0, 3, axis=3) * mask
    outs = []
    for overlap in (False, True):
        with bt.Solver(bt.make_config(shape, precision=bt.BT_F32, scheme=scheme, **kw)) as s:
            s.upload_geometry(mask, vel)
            if wave is not None:
                s.set_schedule([], grad_wave=wave)
            s.set_state(st0)
            if overlap:
                s.run_async(40)
                s.set_state(st1)      # converted now, copied after the 40 steps
                mt_a = s.read_mt(40)
            else:
                mt_a = s.run(40)
                s.set_state(st1)
            mt_b = s.run(40)
            outs.append((mt_a, mt_b, s.get_state()))
    for a, b in zip(outs[0], outs[1]):
        assert np.array_equal(a, b)
