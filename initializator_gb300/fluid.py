"""Per-voxel fluid coefficients for the inputs the uniform-fluid path cannot
express: face surface relaxivities from SurfRel*.dat files and the
two-component (NCOMP 2) water/oil model.

Each function restates one step of the reference's set-up
(src/NmrRelaxationSolve.cpp) in FP64, in the reference's operation order, so
that the arrays are bit-identical to what the reference leaves in its fields:

* ``concentrations``   — FillInConcentration (cpp:935-1008)
* ``phase_fractions``  — the z1/z2 interpolation (cpp:1780-1786, 3311-3316)
* ``surface_relaxivities`` — ReadSurfRel (cpp:1012-1435)
* ``coefficients``     — FillInDiffusinAndTime (cpp:1756-1841)

The results feed ``Solver.upload_rates`` (T1, T2, D) and
``Solver.set_phase_weights`` (c1, c2).
"""
from __future__ import annotations

import math

import numpy as np

SMALL = 1.0e-50
BIG = 1.0e50


def concentrations(data, shape, n1=None):
    """(concentration[0], concentration[1]) per voxel. One component: the
    fluid selected by NFLUID is 1 everywhere. Two components: n1_init.dat
    (read as float by the reference) and 1 - n1."""
    if data.n_components == 2:
        if n1 is None:
            raise ValueError("NCOMP 2 needs n1_init.dat")
        c0 = np.asarray(n1, dtype=np.float32).astype(np.float64).reshape(shape)
        return c0, 1.0 - c0
    c0 = np.zeros(shape)
    c1 = np.zeros(shape)
    if data.n_fluid == 1:
        c0[:] = 1.0
    elif data.n_fluid == 2:
        c1[:] = 1.0
    return c0, c1


def phase_fractions(data, conc0, conc1):
    """(c1, c2): for two components the distances of (conc0, conc1) to the
    phase points (AN(1), AN(2)) and (BN(1), BN(2)) give c1 = z2 / (z1 + z2),
    c2 = z1 / (z1 + z2); for one component the concentrations themselves."""
    if data.n_components != 2:
        return conc0, conc1
    z1 = np.sqrt((conc0 - data.an1) * (conc0 - data.an1) + (conc1 - data.an2) * (conc1 - data.an2))
    z2 = np.sqrt((conc0 - data.bn1) * (conc0 - data.bn1) + (conc1 - data.bn2) * (conc1 - data.bn2))
    return z2 / (z1 + z2), z1 / (z1 + z2)


def surface_relaxivities(data, shape, files=None):
    """Face relaxivities {"1Water", "2Water", "1Oil", "2Oil"} -> (fx, fy, fz)
    with fx[k, j, i] for i in [0, nx] (face i is the low face of cell i), as
    the velocity faces. From ``files`` (the SurfRel*.dat arrays, e.g. from
    datfiles.read_surfrel) when nSurfRelWater / nSurfRelOil is 1, otherwise the
    constants R1/R2 of the fluid on every face."""
    nz, ny, nx = shape
    out = {}
    for fluid, flag, r1, r2 in (("Water", data.n_surf_rel_water, data.r1_water, data.r2_water),
                                ("Oil", data.n_surf_rel_oil, data.r1_oil, data.r2_oil)):
        for n, r in (("1", r1), ("2", r2)):
            key = n + fluid
            if flag == 1:
                if files is None or key not in files:
                    raise ValueError(f"SurfRel{key}X/Y/Z.dat needed")
                out[key] = tuple(np.asarray(a, dtype=np.float64) for a in files[key])
            else:
                out[key] = (np.full((nz, ny, nx + 1), r), np.full((nz, ny + 1, nx), r), np.full((nz + 1, ny, nx), r))
    return out


def coefficients(data, mask, c1, c2, surf):
    """(T1, T2, D) per voxel as FillInDiffusinAndTime forms them (solid: D =
    1e-50, T = 1e50). Per pore voxel: D = (c1 Dw + c2 Do) (1 - 2 c1 c2 /
    (c1^2 + c2^2))^10 (1e-50 without diffusion); 1/T = c1/Tw + c2/To, then for
    each solid face neighbour in the order -x, +x, -y, +y, -z, +z
    (c1 r_water + c2 r_oil) / d with that face's relaxivities."""
    mask = np.asarray(mask).astype(bool)
    nz, ny, nx = mask.shape
    cd = c1 * data.d_water + c2 * data.d_oil
    with np.errstate(divide="ignore", invalid="ignore"):
        base = 1.0 - 2.0 * c1 * c2 / (c1 * c1 + c2 * c2)
    # the C library's pow, as the reference calls it (numpy's own power can
    # differ in the last bit); a base of exactly 1 (one pure phase) gives 1
    pw = np.ones_like(base)
    mixed = base != 1.0
    pw[mixed] = [math.pow(b, 10.0) for b in base[mixed]]
    D = cd * pw
    if data.n_diffusion == 0:
        D = np.full(mask.shape, SMALL)
    with np.errstate(divide="ignore"):
        ct1 = c1 / data.t1_water + c2 / data.t1_oil
        ct2 = c1 / data.t2_water + c2 / data.t2_oil
    # solid neighbours inside the domain (the ghost layer copies the edge voxel)
    pad = np.pad(mask, 1, mode="edge")
    solid = [~pad[1:-1, 1:-1, :-2], ~pad[1:-1, 1:-1, 2:], ~pad[1:-1, :-2, 1:-1], ~pad[1:-1, 2:, 1:-1],
             ~pad[:-2, 1:-1, 1:-1], ~pad[2:, 1:-1, 1:-1]]
    w1, w2, o1, o2 = surf["1Water"], surf["2Water"], surf["1Oil"], surf["2Oil"]
    face = [
        (lambda a: a[:, :, :-1], 0, data.dx), (lambda a: a[:, :, 1:], 0, data.dx),
        (lambda a: a[:, :-1, :], 1, data.dy), (lambda a: a[:, 1:, :], 1, data.dy),
        (lambda a: a[:-1, :, :], 2, data.dz), (lambda a: a[1:, :, :], 2, data.dz),
    ]
    for f, (sel, ax, d) in enumerate(face):
        t1 = ct1 + (c1 * sel(w1[ax]) + c2 * sel(o1[ax])) / d
        t2 = ct2 + (c1 * sel(w2[ax]) + c2 * sel(o2[ax])) / d
        ct1 = np.where(solid[f], t1, ct1)
        ct2 = np.where(solid[f], t2, ct2)
    with np.errstate(divide="ignore"):
        T1 = 1.0 / ct1
        T2 = 1.0 / ct2
    T1 = np.where(mask, T1, BIG)
    T2 = np.where(mask, T2, BIG)
    D = np.where(mask, D, SMALL)
    return T1, T2, D
