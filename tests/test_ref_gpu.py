"""Parity with the reference's own GPU path: its CUDA kernels (the MacCormack
predictor/corrector and the BC_* ghost-layer kernels of
src/NmrRelaxationSolveKernels.cu, compiled unmodified into a cubin) driven by
oracle/ref_gpu.cpp as solve_gpu drives them.

Bars (written here, checked below):
  library MacCormack FP64 and the oracle's restatement vs the reference's
      kernels built without multiply-add contraction: fields bit-identical,
      M(t) <= 1e-12 relative (the sums are added in another order);
  vs the kernels as the reference's own build makes them (nvcc's default
      -fmad=true): fields and M(t) <= 1e-12 relative;
  ghost layers (nBoundary 1 copy, 3 periodic, 2 zero on x, and pairs the
      reference leaves alone): the oracle's boundary modes bit-identical to
      the reference's BC kernels.

Races of the reference: with flow, NMR_predictor_upgrade writes a pore
voxel's value into each solid -x/-y/-z neighbour before differencing against
it, and NMR_corrector_upgrade does the same into the predictor's +x/+y/+z
solid neighbours (cu:765-782, 931-948). A solid voxel with two or more pore
writers gets whichever write lands last, so the reference's own result there
depends on scheduling. Cases with flow are chosen race-free (no solid, or
solid slabs normal to z: one writer per solid voxel); on a porous case with
flow the comparison leaves out every voxel within 2 steps' reach of a
contested solid voxel and checks the rest bit for bit.

Skipped where the reference's kernels were not compiled (oracle.build_ref with
BT_REFERENCE_DIR, in the container that holds the reference sources; the
cubins travel with the repository to the GPU).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MT_TOL = 1e-12


def _need(fmad=False):
    import oracle
    if oracle.ref_gpu_cubin(fmad) is None:
        pytest.skip("the reference's GPU kernels were not compiled here (BT_REFERENCE_DIR)")


def modes_from_nb(nb):
    """Ghost-layer kind per axis the reference's GPU path ends up with for
    nBoundary1..6 (cu:1321-1396): copy when both faces of the pair are 1,
    periodic when both are 3, zero otherwise (BC_Advanced on x for a 2; other
    pairs are left untouched, and their never-written ghosts hold zero)."""
    pairs = [(nb[0], nb[2]), (nb[1], nb[3]), (nb[4], nb[5])]
    return tuple(0 if p == (1, 1) else 1 if p == (3, 3) else 2 for p in pairs)


def _case(kind, shape=(16, 20, 24), seed=5, radius=3.0, solid=0.3):
    from initializator_gb300 import geometry
    nz, ny, nx = shape
    if kind == "porous":
        mask = geometry.sphere_pack(shape, radius, solid, seed=seed)
    elif kind == "open":
        mask = np.ones(shape, dtype=np.uint8)
    elif kind == "slabs":
        mask = np.ones(shape, dtype=np.uint8)
        mask[nz // 3] = 0
        mask[2 * nz // 3] = 0
    else:
        raise ValueError(kind)
    vel = geometry.curl_velocity(mask, 2.0, 1e-3, seed=seed + 1)
    return mask, vel


def _params(shape, flow, **over):
    import oracle
    from initializator_gb300 import geometry
    kw = dict(dx=1e-6, dt=geometry.stable_dt(1e-6, 2.3e-9), main_field=(0.0, 0.3, 1.0), grad=(0.0, 0.02, 0.05),
              d_pore=2.3e-9, t1=0.5, t2=0.2, rho1=1e-5, rho2=2e-5, p_eq=1.0, vector_mult=1,
              velocity=1 if flow else 0, diffusion=1)
    kw.update(over)
    return kw, oracle.make_params(shape, **kw)


def _start(mask):
    st = np.zeros((3,) + mask.shape)
    st[0] = mask
    st[2] = 0.25 * mask
    return st


def _library(kw, mask, vel, st0, n, boundary=None):
    import initializator_gb300 as bt
    cfg = bt.make_config(mask.shape, precision=bt.BT_F64, scheme=bt.BT_SCHEME_MACCORMACK, **kw)
    if boundary is not None:
        cfg.boundary[:] = list(boundary)
    with bt.Solver(cfg) as s:
        s.upload_geometry(mask, vel if kw["velocity"] else None)
        s.set_state(st0)
        mt = s.run(n)
        return s.get_state(), mt


def _reference(p, mask, vel, st0, n, nb=(1,) * 6, fmad=False):
    import oracle
    with oracle.RefGpu(p, mask, st0, vel=vel if p.velocity else None, nb=nb, fmad=fmad) as r:
        mt, _ = r.run(n, 1)
        return r.state(), mt


def _rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("kind,flow", [("porous", False), ("open", True), ("slabs", True)])
def test_maccormack_bit_identical_to_reference_kernels(kind, flow, btlib, oracle_lib):
    import oracle
    _need()
    mask, vel = _case(kind)
    kw, p = _params(mask.shape, flow)
    st0 = _start(mask)
    n = 30
    ref, ref_mt = _reference(p, mask, vel, st0, n)
    lib, lib_mt = _library(kw, mask, vel, st0, n)
    orc, orc_mt = oracle.run(p, mask, st0, n, vel=vel if flow else None, maccormack=True)
    assert np.array_equal(orc, ref), f"oracle vs reference kernels: {np.abs(orc - ref).max():.3e}"
    assert np.array_equal(lib, ref), f"library vs reference kernels: {np.abs(lib - ref).max():.3e}"
    assert _rel(lib_mt, ref_mt) <= MT_TOL and _rel(orc_mt, ref_mt) <= MT_TOL


@pytest.mark.parametrize("kind,flow", [("porous", False), ("open", True)])
def test_maccormack_close_to_reference_fma_build(kind, flow, btlib):
    """The kernels as the reference builds them contract multiply-adds; the
    fields then differ in the last bits only."""
    _need(fmad=True)
    mask, vel = _case(kind, seed=9)
    kw, p = _params(mask.shape, flow)
    st0 = _start(mask)
    n = 30
    ref, ref_mt = _reference(p, mask, vel, st0, n, fmad=True)
    lib, lib_mt = _library(kw, mask, vel, st0, n)
    assert _rel(lib, ref) <= MT_TOL
    assert _rel(lib_mt, ref_mt) <= MT_TOL


def _contested(mask, reach):
    """Voxels within `reach` (cube) of a solid voxel that two or more pore
    neighbours write into (the predictor's writers sit at +x/+y/+z of it, the
    corrector's at -x/-y/-z)."""
    nz, ny, nx = mask.shape
    pore = np.pad(mask.astype(bool), 1, constant_values=False)
    solid = ~pore[1:-1, 1:-1, 1:-1]
    up = sum(pore[1 + dz:nz + 1 + dz, 1 + dy:ny + 1 + dy, 1 + dx:nx + 1 + dx].astype(int)
             for dz, dy, dx in ((0, 0, 1), (0, 1, 0), (1, 0, 0)))
    dn = sum(pore[1 - dz:nz + 1 - dz, 1 - dy:ny + 1 - dy, 1 - dx:nx + 1 - dx].astype(int)
             for dz, dy, dx in ((0, 0, 1), (0, 1, 0), (1, 0, 0)))
    bad = solid & ((up >= 2) | (dn >= 2))
    out = bad.copy()
    for _ in range(reach):
        grown = out.copy()
        for ax in range(3):
            grown |= np.roll(out, 1, ax) | np.roll(out, -1, ax)
        out = grown
    return out


def test_maccormack_porous_flow_away_from_races(btlib):
    _need()
    # large spheres, so that race-free voxels remain after two steps' reach
    mask, vel = _case("porous", shape=(24, 32, 40), seed=13, radius=6.0, solid=0.15)
    kw, p = _params(mask.shape, True)
    st0 = _start(mask)
    n = 2
    ref, _ = _reference(p, mask, vel, st0, n)
    lib, _ = _library(kw, mask, vel, st0, n)
    skip = _contested(mask, 2 * n + 1)
    keep = ~skip
    assert keep.sum() > 0.2 * keep.size, "the case leaves too few voxels to compare"
    for c in range(3):
        assert np.array_equal(lib[c][keep], ref[c][keep]), f"component {c} differs away from the races"
    # where the reference's writes race its result is one of the writers' picks:
    # the field stays close, well within the size of one upwind term
    assert _rel(lib, ref) <= 1e-2


NB_CASES = [
    (3, 3, 3, 3, 3, 3),   # periodic on every axis (BC_Inf_X/Y/Z)
    (2, 3, 1, 3, 1, 1),   # x: nBoundary1 = 2 -> BC_Advanced_XM/XP with 0; y periodic; z copy
    (1, 1, 3, 2, 3, 3),   # x left alone (1, 3), y left alone (1, 2), z periodic
    (1, 2, 2, 2, 1, 3),   # x zero (nBoundary3 = 2), y left alone (2, 2), z left alone (1, 3)
]


@pytest.mark.parametrize("nb", NB_CASES)
@pytest.mark.parametrize("kind,flow", [("porous", False), ("open", True)])
def test_boundaries_match_reference_bc_kernels(nb, kind, flow, btlib, oracle_lib):
    """The oracle's ghost-layer kinds restate BC_Inf_*, BC_Advanced_* and the
    pairs the reference leaves alone, bit for bit through MacCormack; so do
    the library's (bt_config.boundary)."""
    import oracle
    _need()
    mask, vel = _case(kind, seed=21)
    modes = modes_from_nb(nb)
    kw, p = _params(mask.shape, flow, boundary=modes)
    st0 = _start(mask)
    n = 25
    ref, ref_mt = _reference(p, mask, vel, st0, n, nb=nb)
    orc, orc_mt = oracle.run(p, mask, st0, n, vel=vel if flow else None, maccormack=True)
    assert np.array_equal(orc, ref), f"nb {nb}: {np.abs(orc - ref).max():.3e}"
    assert _rel(orc_mt, ref_mt) <= MT_TOL
    # the library's boundary kinds, through its MacCormack kernels
    import initializator_gb300 as bt
    assert bt.boundary_from_nb(nb) == modes
    lkw = {k: v for k, v in kw.items() if k != "boundary"}
    lib, lib_mt = _library(lkw, mask, vel, st0, n, boundary=modes)
    assert np.array_equal(lib, ref), f"library, nb {nb}: {np.abs(lib - ref).max():.3e}"
    assert _rel(lib_mt, ref_mt) <= MT_TOL
