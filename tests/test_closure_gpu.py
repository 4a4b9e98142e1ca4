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


def test_net_gradients_match_oracle(btlib):
    """Forward and backward of the 4-layer net (tcgen05 convolutions, weight
    gradients, GELU') against the FP64 oracle, same parameters and inputs:
    relative max-norm error of output and of every gradient <= 3e-2 (BF16
    activations and gradients between layers)."""
    import torch

    import oracle.closure_oracle as co
    from initializator_gb300 import closure
    nb, nz, ny, nx = 2, 8, 9, 11
    rng = np.random.default_rng(3)
    lay = closure.PaddedRows(nb, nz, ny, nx)
    net = closure.Net(seed=5, scale=1.5, zero_last=False)
    x = _bf16(rng.standard_normal((nb, nz, ny, nx, 16)))
    t = rng.standard_normal((nb, nz, ny, nx, 16)) * 0.1
    y = net.forward(lay, lay.pack(x, "cuda"))
    yg = lay.unpack(y, fp32_rows=True).cpu().numpy()
    ws = [net.w(i).double().cpu().numpy() for i in range(4)]
    bs = [net.b(i).double().cpu().numpy() for i in range(4)]
    ws_q = [_bf16(w) for w in ws]
    yo, pres, acts = co.net_forward(x, ws_q, bs)
    assert np.abs(yg - yo).max() <= 3e-2 * np.abs(yo).max()
    # loss 0.5 * sum (y - t)^2 -> dy = y - t (interior rows; the halo stays zero)
    dy = torch.zeros((lay.rows, 16), dtype=torch.float32, device="cuda")
    full = dy.view(nb, nz + 2, ny + 2, nx + 2, 16)
    full[:, 1:-1, 1:-1, 1:-1] = torch.as_tensor(yo - t, dtype=torch.float32, device="cuda")
    net.backward(lay, dy)
    torch.cuda.synchronize()
    net.check_status()
    gws, gbs = co.net_backward(yo - t, ws_q, pres, acts)
    gw = net.grad[:net.NW].view(4, 27, 16, 16).double().cpu().numpy()
    gb = net.grad[net.NW:].view(4, 16).double().cpu().numpy()
    for i in range(4):
        assert np.abs(gw[i] - gws[i]).max() <= 3e-2 * np.abs(gws[i]).max(), i
        assert np.abs(gb[i] - gbs[i]).max() <= 3e-2 * np.abs(gbs[i]).max(), i


def test_adamw_decreases_loss(btlib):
    """A few AdamW steps on a fixed batch lower the loss (the net can fit)."""
    import torch

    from initializator_gb300 import closure
    nb, nz, ny, nx = 2, 8, 8, 8
    rng = np.random.default_rng(4)
    lay = closure.PaddedRows(nb, nz, ny, nx)
    net = closure.Net(seed=1, scale=1.0, zero_last=True)
    x = lay.pack(rng.standard_normal((nb, nz, ny, nx, 7)), "cuda")
    tgt = torch.zeros((lay.rows, 16), device="cuda")
    tv = tgt.view(nb, nz + 2, ny + 2, nx + 2, 16)
    tv[:, 1:-1, 1:-1, 1:-1, :3] = torch.as_tensor(rng.standard_normal((nb, nz, ny, nx, 3)) * 0.1, device="cuda",
                                                  dtype=torch.float32)
    losses = []
    for _ in range(30):
        y = net.forward(lay, x)
        diff = y - tgt
        diff[:, 3:] = 0.0
        losses.append(float((diff ** 2).sum()))
        net.backward(lay, 2.0 * diff)
        net.adamw(lr=3e-3)
    assert losses[-1] < 0.7 * losses[0]
