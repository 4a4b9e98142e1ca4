"""Shared test helpers: turn a golden fixture (reference run) into the
oracle's parameters, the solver's config, its initial field and its pulses."""
from __future__ import annotations

import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ["fid", "pfg_flow", "pulses_explicit", "cpmg_oil"]


def load(case):
    return dict(np.load(os.path.join(GOLDEN, case + ".npz")))


def main_field(z):
    ndf = int(z["data_n_direction_field"])
    bx, by, bz = float(z["data_bx0"]), float(z["data_by0"]), float(z["data_bz0"])
    return [(bx, by, bz), (bx, 0.0, 0.0), (0.0, by, 0.0), (0.0, 0.0, bz)][ndf]


def fluid(z):
    pre = "water" if int(z["data_n_fluid"]) == 1 else "oil"
    return dict(d_pore=float(z["data_d_" + pre]), t1=float(z["data_t1_" + pre]), t2=float(z["data_t2_" + pre]),
                rho1=float(z["data_r1_" + pre]), rho2=float(z["data_r2_" + pre]))


def common(z):
    return dict(dx=float(z["data_dx"]), dy=float(z["data_dy"]), dz=float(z["data_dz"]), dt=float(z["dt"]),
                main_field=main_field(z),
                grad=(float(z["data_grad_x"]), float(z["data_grad_y"]), float(z["data_grad_z"])),
                p_eq=float(z["p_eq"]), vector_mult=int(z["data_n_vector_mult"]),
                velocity=int(z["data_n_velocity"]), diffusion=int(z["data_n_diffusion"]),
                buffer=(int(z["data_buffer_x"]), int(z["data_buffer_y"]), int(z["data_buffer_z"])), **fluid(z))


def velocity(z):
    m = float(z["data_vel_mult"])
    return (z["vx"] * m, z["vy"] * m, z["vz"] * m)


def initial_state(z):
    """The field the reference started from: the injected one, or FillInMagnetization
    (cpp:2472-2517): p_eq on the field axis (unit vector for NDIRECT_FIELD 0) in pores."""
    if bool(z["state0_given"]):
        return z["state0"].copy()
    mf = np.array(main_field(z))
    ndf = int(z["data_n_direction_field"])
    st = np.zeros((3,) + z["mask"].shape)
    peq = float(z["p_eq"])
    for c in range(3):
        if ndf == 0:
            v = peq * (mf[c] / np.sqrt(mf[0] * mf[0] + mf[1] * mf[1] + mf[2] * mf[2]))
        else:
            v = peq if ndf == c + 1 else 0.0
        st[c] = np.where(z["mask"] == 1, v, 0.0)
    return st


def pulses(z):
    """Explicit pulse list of the case, or the reference CPU Sequence() schedule
    replayed by the library's host schedule builder."""
    if len(z["pulses"]):
        return [(int(r[0]), int(r[1]), float(r[2]), tuple(float(a) for a in r[3:])) for r in z["pulses"]]
    from initializator_gb300 import sequence_schedule
    d = z["direction"]
    return sequence_schedule(int(z["data_n_sequence"]), int(z["nsteps"]), dt=float(z["dt"]),
                             time1=float(z["data_time1"]), time2=float(z["data_time2"]),
                             direction=tuple(float(v) for v in d), gradient_pulse=float(z["grads"][0]),
                             gpu_variant=False)


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))
