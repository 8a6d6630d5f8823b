"""Emulator kernels: the tcgen05 BF16 implicit-GEMM 3x3 convolution against
an FP64 numpy convolution of the same BF16-rounded operands (FP32
accumulation: relative tolerance 1e-4 of the output scale)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bf16_round(a):
    import torch
    return torch.tensor(a, dtype=torch.float32).to(torch.bfloat16).to(torch.float32).numpy()


def conv_ref(x, w, b, relu):
    """x [B,H,W,Cin], w [9,Cout,Cin], b [Cout] -> [B,H,W,Cout], FP64."""
    B, H, W, C = x.shape
    xp = np.zeros((B, H + 2, W + 2, C))
    xp[:, 1:-1, 1:-1] = x
    out = np.zeros((B, H, W, w.shape[1]))
    for tap in range(9):
        dy, dx = divmod(tap, 3)
        out += np.einsum("bhwc,oc->bhwo", xp[:, dy:dy + H, dx:dx + W], w[tap].astype(np.float64))
    out += b
    return np.maximum(out, 0) if relu else out


@pytest.mark.parametrize("cin,cout,relu", [(16, 48, 1), (48, 48, 1), (48, 16, 0), (16, 16, 0)])
def test_conv3x3_tcgen05_matches_fp64(gpulib, cin, cout, relu):
    import torch
    rng = np.random.default_rng(cin * 100 + cout)
    B, H, W = 2, 5, 256
    x = bf16_round(rng.normal(size=(B, H, W, cin)).astype(np.float32))
    w = bf16_round((rng.normal(size=(9, cout, cin)) / np.sqrt(9 * cin)).astype(np.float32))
    b = rng.normal(size=cout).astype(np.float32)
    dx = torch.tensor(x).to(torch.bfloat16).cuda()
    dw = torch.tensor(w).to(torch.bfloat16).cuda()
    db = torch.tensor(b).cuda()
    y32 = torch.zeros((B, H, W, cout), dtype=torch.float32, device="cuda")
    y16 = torch.zeros((B, H, W, cout), dtype=torch.bfloat16, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    rc = gpulib.nl2d_emu_conv3x3(dx.data_ptr(), dw.data_ptr(), db.data_ptr(), y16.data_ptr(),
                                 y32.data_ptr(), B, H, W, cin, cout, relu, err.data_ptr(), None)
    assert rc == 0
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    want = conv_ref(x, w, b, relu)
    got = y32.cpu().numpy()
    scale = np.abs(want).max()
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-4 * scale)
    np.testing.assert_allclose(y16.float().cpu().numpy(), want, rtol=1e-2, atol=1e-2 * scale)
