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


def test_conv_backward_matches_fp64(gpulib):
    """Input gradient (tcgen05 conv with flipped, transposed weights) and
    weight / bias gradients (FP32 reduction) of L = sum(y * G) against the
    FP64 numpy gradients."""
    import torch
    rng = np.random.default_rng(5)
    B, H, W, cin, cout = 2, 4, 128, 48, 16
    x = bf16_round(rng.normal(size=(B, H, W, cin)).astype(np.float32))
    w = bf16_round((rng.normal(size=(9, cout, cin)) / 20).astype(np.float32))
    G = bf16_round(rng.normal(size=(B, H, W, cout)).astype(np.float32))
    # FP64 reference gradients of L = sum(conv(x, w) * G)
    xp = np.zeros((B, H + 2, W + 2, cin))
    xp[:, 1:-1, 1:-1] = x
    dw_ref = np.zeros((9, cout, cin))
    dx_ref = np.zeros((B, H + 2, W + 2, cin))
    for tap in range(9):
        dy_, dx_ = divmod(tap, 3)
        dw_ref[tap] = np.einsum("bhwo,bhwc->oc", G, xp[:, dy_:dy_ + H, dx_:dx_ + W])
        dx_ref[:, dy_:dy_ + H, dx_:dx_ + W] += np.einsum("bhwo,oc->bhwc", G, w[tap])
    dx_ref = dx_ref[:, 1:-1, 1:-1]
    db_ref = G.sum(axis=(0, 1, 2))
    dxd = torch.tensor(x).to(torch.bfloat16).cuda()
    dwd = torch.tensor(w).to(torch.bfloat16).cuda()
    dG = torch.tensor(G).to(torch.bfloat16).cuda()
    wt = torch.zeros(9, cin, cout, dtype=torch.bfloat16, device="cuda")
    assert gpulib.nl2d_emu_flip_transpose(dwd.data_ptr(), wt.data_ptr(), cout, cin, None) == 0
    gx = torch.zeros(B, H, W, cin, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    assert gpulib.nl2d_emu_conv3x3(dG.data_ptr(), wt.data_ptr(), None, None, gx.data_ptr(), B, H,
                                   W, cout, cin, 0, err.data_ptr(), None) == 0
    gw = torch.zeros(9, cout, cin, device="cuda")
    gb = torch.zeros(cout, device="cuda")
    assert gpulib.nl2d_emu_conv_wgrad(dxd.data_ptr(), dG.data_ptr(), gw.data_ptr(),
                                      gb.data_ptr(), B, H, W, cin, cout, None) == 0
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    for got, want in ((gx, dx_ref), (gw, dw_ref), (gb, db_ref)):
        g = got.cpu().numpy()
        np.testing.assert_allclose(g, want, rtol=0, atol=1e-4 * np.abs(want).max())


def test_training_fits_a_known_convolution(gpulib):
    """A few hundred Adam steps of the 6-layer network on a target made by a
    fixed linear 3x3 map of the inputs reduce the loss by 10x."""
    import torch
    from psyclonebench_gb300.emulator import CPAD_IN, ConvNet
    torch.manual_seed(0)
    B, H, W = 2, 16, 128
    net = ConvNet(B, H, W, seed=1, lib=gpulib)
    P = B * H * W
    x = torch.zeros(P, CPAD_IN, dtype=torch.bfloat16, device="cuda")
    x[:, :5] = torch.randn(P, 5, device="cuda").to(torch.bfloat16)
    xi = x.float().reshape(B, H, W, CPAD_IN)[..., :5]
    t = torch.zeros(B, H, W, 3, device="cuda")
    t[..., 0] = 0.5 * xi[..., 0] - 0.3 * xi[..., 3]
    t[..., 1] = 0.2 * torch.roll(xi[..., 1], 1, dims=2)
    t[..., 2] = 0.4 * xi[..., 4] + 0.1 * xi[..., 2]
    t = t.reshape(P, 3).contiguous()
    first = net.train_step(x, t, lr=3e-3)
    for _ in range(300):
        last = net.train_step(x, t, lr=3e-3)
    assert last < 0.1 * first, (first, last)
