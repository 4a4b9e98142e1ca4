"""bt_step_noalloc, the entry point for callers that may not allocate device
memory (stream-capture regions, hosts whose framework has reserved the
device's memory, plugin hosts that forbid allocations).

It is checked through the C ABI against the handle-based entry point
(bt_create / bt_run) on the same inputs, for two calls in a row, the second
fed with the first one's output. Its scratch is a fixed array inside the
library, so nothing here allocates on the library's side: the caller (this
test, with torch tensors) owns every buffer.

Tolerances as in test_parity_gpu: FP64 per voxel and M(t) <= 1e-12 relative
(the same kernel runs, so the bits match); FP32 <= 1e-5 (the handle-based
FP32 path runs the TMA fast kernel for pulse-free steps, a different FP32
operation order).
"""
import ctypes

import numpy as np
import pytest

from helpers import rel_err

pytestmark = pytest.mark.gpu


def _case():
    from initializator_gb300 import geometry
    shape = (40, 37, 35)
    mask = geometry.sphere_pack(shape, 3.0, 0.3, seed=21)
    vel = geometry.curl_velocity(mask, 2.0, 1.5e-3, seed=22)
    st0 = np.random.default_rng(23).uniform(-1, 1, (3,) + shape) * mask
    kw = dict(dx=1e-6, dy=1.1e-6, dz=0.9e-6, dt=0.8 * geometry.stable_dt(1.1e-6, 2.3e-9), main_field=(0.2, 0.3, 0.9),
              grad=(0.02, -0.03, 0.05), d_pore=2.3e-9, t1=0.1, t2=0.05, rho1=3e-5, rho2=5e-5, p_eq=0.5,
              vector_mult=1, velocity=1, diffusion=1, buffer=(1, 2, 1))
    return shape, mask, vel, st0, kw


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_noalloc_matches_handle_api_two_calls(precision, btlib):
    import torch

    import initializator_gb300 as bt
    shape, mask, vel, st0, kw = _case()
    prec = bt.BT_F64 if precision == "f64" else bt.BT_F32
    tol = 1e-12 if precision == "f64" else 1e-5
    cfg = bt.make_config(shape, precision=prec, **kw)
    # the existing entry point: two single steps
    with bt.Solver(cfg) as s:
        s.upload_geometry(mask, vel)
        s.set_state(st0)
        ref = []
        for _ in range(2):
            mt = s.run(1)
            ref.append((s.get_state(), mt[0]))
    # the allocation-free entry point on caller-owned device buffers
    dt = torch.float64 if precision == "f64" else torch.float32
    dev = torch.device("cuda", 0)
    mask_d = torch.from_numpy(mask).to(dev)
    vel_d = [torch.from_numpy(v).to(dev, dt).contiguous() for v in vel]
    cur = [torch.from_numpy(st0[c]).to(dev, dt).contiguous() for c in range(3)]
    stream = torch.cuda.current_stream(dev)
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    for call in range(2):
        out = [torch.empty_like(cur[c]) for c in range(3)]
        sums = torch.full((3,), float("nan"), dtype=torch.float64, device=dev)
        rc = btlib.bt_step_noalloc(ctypes.byref(cfg), p(mask_d), p(vel_d[0]), p(vel_d[1]), p(vel_d[2]),
                                   p(cur[0]), p(cur[1]), p(cur[2]), p(out[0]), p(out[1]), p(out[2]), p(sums),
                                   ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0
        torch.cuda.synchronize()
        field = np.stack([o.double().cpu().numpy() for o in out])
        ref_field, ref_mt = ref[call]
        assert rel_err(field, ref_field) <= tol, call
        assert rel_err(sums.cpu().numpy(), ref_mt) <= tol, call
        if precision == "f64":
            assert np.array_equal(field, ref_field)
        cur = out


def test_noalloc_rejects_grids_above_its_limit(btlib):
    import initializator_gb300 as bt
    cfg = bt.make_config((256, 256, 256), dx=1e-6, dt=1e-5)
    dummy = ctypes.c_void_p(256)  # never dereferenced: the size check comes first
    rc = btlib.bt_step_noalloc(ctypes.byref(cfg), dummy, None, None, None, dummy, dummy, dummy, dummy, dummy,
                               dummy, dummy, None)
    assert rc == -7  # BT_E_SIZE
