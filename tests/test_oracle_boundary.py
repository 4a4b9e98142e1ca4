"""The oracle's ghost-layer kinds on the CPU (no GPU): properties that hold
for any correct periodic / zero layer, checked on the oracle's restatement of
BC_Inf_* and BC_Advanced_* (the GPU tests pin it bit for bit to the
reference's own BC kernels). Every run's first step reads copy ghosts (the
reference's initial layer); the cases are built so that this is visible or
harmless, as each test says."""
import numpy as np

import oracle


def _p(shape, boundary, **over):
    kw = dict(dx=1e-6, dt=0.9e-12 / (6 * 2.3e-9), d_pore=2.3e-9, t1=1e30, t2=1e30, rho1=0.0, rho2=0.0, p_eq=0.0,
              main_field=(0.0, 0.0, 1.0), vector_mult=0, velocity=0, diffusion=1, boundary=boundary)
    kw.update(over)
    return oracle.make_params(shape, **kw)


def _blob(shape, seed=3):
    rng = np.random.default_rng(seed)
    st = np.zeros((3,) + shape)
    st[0] = rng.random(shape)
    st[1] = rng.random(shape) - 0.5
    return st


def test_periodic_diffusion_conserves():
    """All-pore box, diffusion only, periodic on every axis: the total stays."""
    shape = (6, 7, 8)
    mask = np.ones(shape, dtype=np.uint8)
    st0 = _blob(shape)
    _, mt = oracle.run(_p(shape, (1, 1, 1)), mask, st0, 12)
    assert np.allclose(mt[:, 0], st0[0].sum(), rtol=1e-13, atol=0)
    assert np.allclose(mt[:, 1], st0[1].sum(), rtol=0, atol=1e-12)


def test_zero_faces_drain_and_copy_faces_keep():
    """Diffusion only: a zero layer makes the faces a sink (from the second
    step on: the first reads the initial copies), a copy layer conserves."""
    shape = (8, 8, 8)
    mask = np.ones(shape, dtype=np.uint8)
    st0 = np.zeros((3,) + shape)
    st0[0] = 1.0
    n = 10
    _, mt_copy = oracle.run(_p(shape, (0, 0, 0)), mask, st0, n)
    _, mt_zero = oracle.run(_p(shape, (2, 0, 0)), mask, st0, n)
    assert np.allclose(mt_copy[:, 0], st0[0].sum(), rtol=1e-13)
    assert abs(mt_zero[0, 0] - st0[0].sum()) <= 1e-12 * st0[0].sum()
    assert np.all(np.diff(mt_zero[:, 0]) < 0)


def test_periodic_equals_the_middle_of_a_tiled_box():
    """Periodic layers on x act as the middle period of a box three periods
    long with copy layers, bit for bit, until the outer copy walls' influence
    (one cell per step) reaches the middle period. The start has equal x-edge
    planes, so the first step's copy ghosts equal the periodic ones."""
    shape = (5, 6, 9)
    nx = shape[2]
    mask = np.ones(shape, dtype=np.uint8)
    st0 = _blob(shape, seed=7)
    st0[..., -1] = st0[..., 0]
    n = nx - 1
    per, _ = oracle.run(_p(shape, (1, 0, 0)), mask, st0, n)
    tshape = (5, 6, 3 * nx)
    tiled = np.concatenate([st0, st0, st0], axis=3)
    big, _ = oracle.run(_p(tshape, (0, 0, 0)), np.ones(tshape, np.uint8), tiled, n)
    assert np.array_equal(per, big[..., nx:2 * nx])
    # and the same box with a copy layer differs: the wrap is visible
    cpy, _ = oracle.run(_p(shape, (0, 0, 0)), mask, st0, n)
    assert not np.array_equal(per, cpy)


def test_zero_equals_a_box_with_a_pinned_zero_layer():
    """A zero layer on z acts as a copy-layer box one cell taller on each
    side whose outer planes are held at zero (diffusion only, no gradient):
    compare step by step, re-zeroing the outer planes of the bigger box after
    each step. The start's z-edge planes are zero, so the first step's copy
    ghosts are zero too."""
    shape = (6, 5, 7)
    mask = np.ones(shape, dtype=np.uint8)
    st = _blob(shape, seed=11)
    st[:, 0] = 0.0
    st[:, -1] = 0.0
    n = 5
    zer, _ = oracle.run(_p(shape, (0, 0, 2)), mask, st, n)
    bshape = (shape[0] + 2, shape[1], shape[2])
    big = np.zeros((3,) + bshape)
    big[:, 1:-1] = st
    for _ in range(n):
        big, _ = oracle.run(_p(bshape, (0, 0, 0)), np.ones(bshape, np.uint8), big, 1)
        big[:, 0] = 0.0
        big[:, -1] = 0.0
    assert np.array_equal(zer, big[:, 1:-1])
