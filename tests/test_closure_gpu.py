"""The learned closure's kernels against the FP64 numpy oracle of the net.

Tolerances: the tensor-core MMA self-test is exact up to FP32 summation
(1e-6); convolutions take BF16 operands, so outputs are compared with the
oracle evaluated on the same BF16-rounded inputs — FP32 outputs to 1e-5,
BF16-stored outputs to 1e-2 relative (BF16 has an 8-bit mantissa)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bf16(a):
    import torch
    return torch.as_tensor(a, dtype=torch.float32).to(torch.bfloat16).float().numpy().astype(np.float64)


def test_umma_selftest(btlib):
    import ctypes

    import torch
    rng = np.random.default_rng(0)
    a = torch.tensor(rng.standard_normal((128, 16)), dtype=torch.bfloat16, device="cuda")
    b = torch.tensor(rng.standard_normal((16, 16)), dtype=torch.bfloat16, device="cuda")
    d = torch.zeros((128, 16), dtype=torch.float32, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    assert btlib.bt_umma_selftest(ctypes.c_void_p(a.data_ptr()), ctypes.c_void_p(b.data_ptr()),
                                  ctypes.c_void_p(d.data_ptr()), ctypes.c_void_p(st.data_ptr()), None) == 0
    torch.cuda.synchronize()
    ref = a.double().cpu().numpy() @ b.double().cpu().numpy().T
    assert int(st.item()) == 0
    assert np.abs(d.cpu().numpy() - ref).max() <= 1e-6 * np.abs(ref).max()


@pytest.mark.parametrize("shape", [(2, 6, 7, 9), (1, 12, 10, 33)])
def test_conv3d_forward_modes(shape, btlib):
    import torch

    import oracle.closure_oracle as co
    from initializator_gb300 import closure
    nb, nz, ny, nx = shape
    rng = np.random.default_rng(1)
    x = _bf16(rng.standard_normal((nb, nz, ny, nx, 16)))
    w = rng.standard_normal((27, 16, 16)) * 0.1
    b = rng.standard_normal(16) * 0.1
    lay = closure.PaddedRows(nb, nz, ny, nx)
    xr = lay.pack(x, "cuda")
    wt = torch.tensor(w, dtype=torch.float32, device="cuda")
    wf, wd = closure.pack_weights(wt)
    bt_ = torch.tensor(b, dtype=torch.float32, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    wq = _bf16(w)
    ref = co.conv3d(x, wq, b)
    # mode 1: FP32 rows
    outf = torch.zeros((lay.rows, 16), dtype=torch.float32, device="cuda")
    closure.conv3d(lay, xr, wf, 1, bias=bt_, outf=outf, status=st)
    # mode 0: GELU to BF16 padded rows + FP32 pre-activation
    out = lay.empty("cuda")
    pre = torch.zeros((lay.rows, 16), dtype=torch.float32, device="cuda")
    closure.conv3d(lay, xr, wf, 0, bias=bt_, out=out, pre=pre, status=st)
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    got1 = lay.unpack(outf, fp32_rows=True).cpu().numpy()
    assert np.abs(got1 - ref).max() <= 1e-5 * np.abs(ref).max()
    gotp = lay.unpack(pre, fp32_rows=True).cpu().numpy()
    assert np.abs(gotp - ref).max() <= 1e-5 * np.abs(ref).max()
    got0 = lay.unpack(out).cpu().numpy()
    g = co.gelu(ref)
    assert np.abs(got0 - g).max() <= 1e-2 * np.abs(g).max()
    # the halo rows of the BF16 output are zero (a valid input for the next layer)
    full = out[lay.margin:lay.margin + lay.rows].float().reshape(nb, nz + 2, ny + 2, nx + 2, 16)
    assert float(full[:, 0].abs().max()) == 0.0 and float(full[:, :, :, -1].abs().max()) == 0.0
