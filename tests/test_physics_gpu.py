"""Physics checks of the benched KSPACE (exact-precession) scheme on the GPU.

1. FP32 against FP64 of the same solver at the bench's 256^3 workload (sphere
   pack, curl-noise flow, PGSE with the refocusing pulse) over 1000 steps:
   max_t |M_f32(t) - M_f64(t)| / |M_f64(0)| <= 1e-4 (M = the three lab-frame
   sums). The FP32 run is the TMA fast path (generic kernel on the pulse
   step), the FP64 run the generic kernel, which is pinned to the oracle.

2. Known answer: free diffusion under PGSE (Stejskal-Tanner). An all-pore box,
   long along the gradient (z), no relaxation, no flow; the magnetisation
   starts as a slab 256 voxels away from either z wall, so over the echo time
   (diffusion length sqrt(2 D Delta) ~ 10 voxels) no spin reaches a wall and
   the box acts as free space. Rectangular lobes, narrow lobes (delta of a
   few steps) and trapezoidal lobes.

   a. Against the scheme's exact discrete answer: the echo's k = 0 mode
      followed along its k-space path kappa_n (k at the middle of each step,
      where the stencil acts, sign-flipped by the 180 pulse) decays by
      prod_n (1 - D dt lambda(kappa_n)), lambda(k) = (2 - 2 cos(k dz)) / dz^2.
      Tolerance: 1e-11 (FP64), 2e-5 (FP32) on E = S_echo / S_0.
   b. Against Stejskal-Tanner E = exp(-D b), b = gamma^2 G^2 (d^2 (Delta - d/3)
      + e^3/30 - d e^2/6) for lobes of rise time e and start-of-rise to
      start-of-fall d: |ln E - ln E_ST| is bounded by the scheme's three
      stated error terms, computed from the waveform:
        time stepping   |sum ln(1 - x_n) + sum x_n|,  x_n = D dt lambda(kappa_n)
        space (dz^2)    D dt |sum (lambda(kappa_n) - kappa_n^2)|   (~ kappa^4 dz^2 / 12)
        quadrature      D |sum kappa_n^2 dt - int k(t)^2 dt|       (midpoint k per step)
      plus the rounding allowance of (a).
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GAMMA = 2.675e8
D = 2.3e-9
DX = 1e-6


def _stable_dt():
    from initializator_gb300 import geometry
    return geometry.stable_dt(DX, D)


def test_kspace_f32_vs_f64_256(btlib):
    """The bench's 256^3 workload, 1000 steps, FP32 fast path vs FP64."""
    import torch

    import initializator_gb300 as bt
    from initializator_gb300 import geometry
    shape = (256, 256, 256)
    nsteps = 1000
    mask = geometry.sphere_pack(shape, 10.0, 0.4, seed=20261203, device="cuda")
    vel = geometry.curl_velocity(mask, 4.0, 1.0e-3, seed=20261204, device="cuda")
    dt = _stable_dt()
    wave = bt.kspace_waveform_pgse(nsteps + 8, dt, 0.1, 2e-3, 20e-3, axis=(0.0, 0.0, 1.0))
    rf = [(bt.pgse_refocus_step(dt, 20e-3), 2, math.pi, (1.0, 0.0, 0.0))]
    kw = dict(dx=DX, dt=dt, d_pore=D, t1=2.5, t2=2.0, rho1=1e-5, rho2=1e-5, p_eq=1.0, velocity=1, diffusion=1,
              gamma=bt.GAMMA_PROTON)
    mts = {}
    for prec in (bt.BT_F32, bt.BT_F64):
        with bt.Solver(bt.make_config(shape, precision=prec, scheme=bt.BT_SCHEME_KSPACE, **kw)) as s:
            s.upload_geometry(mask, vel)
            s.set_schedule(rf, grad_wave=wave)
            tdt = torch.float64 if prec == bt.BT_F64 else torch.float32
            m = torch.as_tensor(mask, device="cuda").to(tdt)
            z = torch.zeros_like(m)
            s.set_state_device([m, z, z.clone()])
            mts[prec] = (s.measure(), s.run(nsteps))
    m0 = mts[bt.BT_F64][0]
    err = np.linalg.norm(mts[bt.BT_F32][1] - mts[bt.BT_F64][1], axis=1).max() / np.linalg.norm(m0)
    assert err <= 1e-4, f"FP32 vs FP64 M(t) error {err:.3e}"
    # the refocusing pulse took effect: the echo recovers most of the signal
    assert abs(mts[bt.BT_F64][1][-1][0]) > 0.1 * abs(m0[0])


def _lam(k, dz):
    return (2.0 - 2.0 * np.cos(k * dz)) / (dz * dz)


def _pgse_case(kind, dt):
    """(g, delta, Delta, ramp) of each waveform."""
    if kind == "rect":
        return 0.1, 2e-3, 20e-3, 0.0
    if kind == "narrow":
        # three steps long, ten times the amplitude (about the same q)
        return 0.1 * (2e-3 / (3 * dt)), 3 * dt, 20e-3, 0.0
    return 0.1, 2e-3, 20e-3, 0.5e-3


@pytest.mark.parametrize("kind", ["rect", "narrow", "trapezoid"])
@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_pgse_free_diffusion_stejskal_tanner(kind, precision, btlib):
    import initializator_gb300 as bt
    dt = _stable_dt()
    g, delta, Delta, ramp = _pgse_case(kind, dt)
    shape = (1024, 8, 64)  # (nz, ny, nx): long along the gradient
    nz = shape[0]
    t_echo = Delta + delta
    nsteps = int(math.ceil(t_echo / dt)) + 4
    wave = bt.kspace_waveform_pgse(nsteps + 1, dt, g, delta, Delta, axis=(0.0, 0.0, 1.0), ramp=ramp)
    s_pi = bt.pgse_refocus_step(dt, Delta)
    rf = [(s_pi, 2, math.pi, (1.0, 0.0, 0.0))]
    mask = np.ones(shape, dtype=np.uint8)
    st0 = np.zeros((3,) + shape)
    st0[0, nz // 4: 3 * nz // 4] = 1.0          # the slab, 256 voxels from each wall
    prec = bt.BT_F64 if precision == "f64" else bt.BT_F32
    kw = dict(dx=DX, dt=dt, d_pore=D, t1=1e30, t2=1e30, rho1=0.0, rho2=0.0, p_eq=0.0, velocity=0, diffusion=1,
              gamma=GAMMA)
    with bt.Solver(bt.make_config(shape, precision=prec, scheme=bt.BT_SCHEME_KSPACE, **kw)) as s:
        s.upload_geometry(mask)
        s.set_schedule(rf, grad_wave=wave)
        s.set_state(st0)
        s0 = s.measure()
        mt = s.run(nsteps)
    S0 = s0[0] + 1j * s0[1]
    S = mt[-1, 0] + 1j * mt[-1, 1]
    E_sim = S / S0

    # (a) the discrete answer along the echo mode's k-space path
    gz = wave[:nsteps, 2]
    k = np.concatenate([[0.0], np.cumsum(GAMMA * gz * dt)])     # k at the start of each step
    kap = k[:nsteps] + 0.5 * GAMMA * gz * dt                      # at the middle of each step
    kap[s_pi + 1:] = kap[s_pi + 1:] - 2.0 * k[s_pi + 1]            # the pulse after step s_pi flips the mode
    assert abs(k[nsteps] - 2.0 * k[s_pi + 1]) < 1e-6 * abs(k[s_pi + 1]), "the echo is not refocused at the end"
    x = D * dt * _lam(kap, DX)
    E_disc = float(np.prod(1.0 - x))
    tol_a = 1e-11 if precision == "f64" else 2e-5
    assert abs(E_sim - E_disc) <= tol_a, f"E_sim {E_sim} vs discrete {E_disc}"

    # (b) Stejskal-Tanner with the stated error terms of the scheme
    d, e = delta - ramp, ramp
    b_st = GAMMA ** 2 * g ** 2 * (d * d * (Delta - d / 3) + e ** 3 / 30 - d * e * e / 6)
    E_st = math.exp(-D * b_st)
    # int k(t)^2 dt of the true waveform, finely sampled (the pulse flips k)
    fine = 400
    tf = (np.arange(nsteps * fine) + 0.5) * (dt / fine)
    w_true = bt.kspace_waveform_pgse(nsteps * fine, dt / fine, g, delta, Delta, axis=(0.0, 0.0, 1.0), ramp=ramp)[:, 2]
    kt = np.cumsum(GAMMA * w_true * (dt / fine)) - 0.5 * GAMMA * w_true * (dt / fine)
    t_pi = (s_pi + 1) * dt
    kt = np.where(tf > t_pi, kt - 2.0 * np.interp(t_pi, tf, kt), kt)
    b_true = float(np.sum(kt * kt) * (dt / fine))
    assert math.isclose(b_true, b_st, rel_tol=2e-4), f"waveform b {b_true} vs Stejskal-Tanner {b_st}"
    t_time = abs(np.sum(np.log1p(-x)) + np.sum(x))
    t_space = D * dt * abs(np.sum(_lam(kap, DX) - kap * kap))
    t_quad = D * abs(np.sum(kap * kap) * dt - b_true) + D * abs(b_true - b_st)
    bound = t_time + t_space + t_quad + 2.0 * tol_a / E_disc
    dev = abs(math.log(abs(E_sim)) - math.log(E_st))
    assert dev <= bound, (f"|ln E - ln E_ST| = {dev:.3e} > {bound:.3e} (time {t_time:.1e}, space {t_space:.1e}, "
                          f"quadrature {t_quad:.1e})")
    # the echo is attenuated as Stejskal-Tanner says, to the per-mille
    assert abs(abs(E_sim) - E_st) <= 1e-3 * E_st + bound
