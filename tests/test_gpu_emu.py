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


@pytest.mark.parametrize("cin,cout,relu,B,H", [
    (16, 48, 1, 2, 5), (48, 48, 1, 2, 5), (48, 16, 0, 2, 5), (16, 16, 0, 2, 5),
    # several strips per image, a partial last strip, more units than CTAs;
    # 64 channels take one CTA per SM
    (48, 48, 1, 3, 19), (64, 64, 1, 2, 17), (32, 16, 0, 100, 9)])
def test_conv3x3_tcgen05_matches_fp64(gpulib, cin, cout, relu, B, H):
    """The pipelined tcgen05 convolution (strips of rows, ring of staged
    input rows, two TMEM accumulators) against an FP64 convolution."""
    import torch
    rng = np.random.default_rng(cin * 100 + cout + H)
    W = 256
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


@pytest.mark.parametrize("B,H,W,cin,cout", [(2, 4, 128, 48, 16), (2, 3, 256, 16, 48),
                                             (1, 5, 128, 48, 48),
                                             # several strips per image; more strips
                                             # than CTAs, so TMEM accumulates across them
                                             (3, 19, 256, 48, 48), (60, 17, 128, 16, 48)])
def test_conv_backward_matches_fp64(gpulib, B, H, W, cin, cout):
    """Input gradient (tcgen05 conv with flipped, transposed weights) and
    weight gradient (pipelined tcgen05 GEMM over pixels, FP32 in tensor
    memory) and bias gradient
    of L = sum(y * G) against the FP64 numpy gradients, for the layer shapes
    of the network (16 -> 48, 48 -> 48, 48 -> 16)."""
    import torch
    rng = np.random.default_rng(5)
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
                                      gb.data_ptr(), B, H, W, cin, cout, err.data_ptr(),
                                      None) == 0
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    for got, want in ((gx, dx_ref), (gw, dw_ref), (gb, db_ref)):
        g = got.cpu().numpy()
        np.testing.assert_allclose(g, want, rtol=0, atol=1e-4 * np.abs(want).max())
    # the partial sums are added in a fixed order: the same call gives the
    # same bits again
    gw2, gb2 = torch.zeros_like(gw), torch.zeros_like(gb)
    assert gpulib.nl2d_emu_conv_wgrad(dxd.data_ptr(), dG.data_ptr(), gw2.data_ptr(),
                                      gb2.data_ptr(), B, H, W, cin, cout, err.data_ptr(),
                                      None) == 0
    torch.cuda.synchronize()
    assert torch.equal(gw, gw2) and torch.equal(gb, gb2)


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


def test_training_is_reproducible(gpulib):
    """Two networks from the same seed, trained on the same batches, end
    with the same weights bit for bit: no reduction of the training step
    depends on the order in which blocks finish."""
    import torch
    from psyclonebench_gb300.emulator import CPAD_IN, ConvNet
    B, H, W = 2, 16, 128
    P = B * H * W
    g = torch.Generator(device="cuda").manual_seed(3)
    x = torch.zeros(P, CPAD_IN, dtype=torch.bfloat16, device="cuda")
    x[:, :5] = torch.randn(P, 5, device="cuda", generator=g).to(torch.bfloat16)
    t = torch.randn(P, 3, device="cuda", generator=g)
    weights = []
    for _ in range(2):
        net = ConvNet(B, H, W, seed=1, lib=gpulib)
        for _ in range(40):
            net.train_step(x, t, lr=3e-3)
        torch.cuda.synchronize()
        weights.append([w.clone() for w in net.w32])
    assert all(torch.equal(a, b) for a, b in zip(*weights))


@pytest.fixture(scope="module")
def small_dataset(gpulib):
    """Solver trajectories of 8 domains of 128 x 128 cells, 21 snapshots
    (200 FP64 solver steps) each."""
    from psyclonebench_gb300.emulator import Dataset
    return Dataset(count=8, nsnap=21, seed=3, n=128, lib=gpulib)


def _derived(eta, u, v, d):
    """East / north ssh differences and depth-weighted flux divergence of
    one image, zero across the image edge."""
    gx = np.zeros_like(eta)
    gx[:, :-1] = eta[:, 1:] - eta[:, :-1]
    gy = np.zeros_like(eta)
    gy[:-1] = eta[1:] - eta[:-1]
    de = d.copy()
    de[:, :-1] = 0.5 * (d[:, :-1] + d[:, 1:])
    dn = d.copy()
    dn[:-1] = 0.5 * (d[:-1] + d[1:])
    fe, fn = de * u, dn * v
    div = fe + fn
    div[:, 1:] -= fe[:, :-1]
    div[1:] -= fn[:-1]
    return gx, gy, div


@pytest.mark.parametrize("noise_frac", [0.0, 0.5])
def test_assemble_channels_match_numpy(gpulib, small_dataset, noise_frac):
    """Every input channel and the target of one assembled pair against the
    same quantities formed in numpy.  With noise, the perturbed state is
    recovered from the target (next snapshot minus increment); the noise
    has the requested standard deviation and every channel is consistent
    with the same perturbed state."""
    import torch
    from psyclonebench_gb300.emulator import CPAD_IN, STATE_SCALE
    ds = small_dataset
    n = ds.n
    dom, snap = 5, 7
    x = torch.zeros(n * n, CPAD_IN, dtype=torch.bfloat16, device="cuda")
    tg = torch.zeros(n * n, 3, device="cuda")
    ds.batch([(dom, snap)], x, tg, noise_frac=noise_frac, seed=1234)
    torch.cuda.synchronize()
    s0 = ds.snaps[dom * ds.nsnap + snap].cpu().numpy().reshape(n, n, 3).astype(np.float64)
    s1 = ds.snaps[dom * ds.nsnap + snap + 1].cpu().numpy().reshape(n, n, 3).astype(np.float64)
    st = ds.statics[dom].cpu().numpy().reshape(n, n, 4).astype(np.float64)
    # the solver holds velocities on wall faces at zero
    assert st[..., 2].any() and st[..., 3].any()
    assert not s0[..., 1][st[..., 2] > 0].any() and not s0[..., 2][st[..., 3] > 0].any()
    inc_scale = np.array(ds.inc_scale)
    tgt = tg.cpu().numpy().reshape(n, n, 3).astype(np.float64)
    if noise_frac:
        state = s1 - tgt * inc_scale
        noise = state - s0
        for ch in range(3):
            sd = noise[..., ch].std()
            assert abs(sd / (noise_frac * inc_scale[ch]) - 1.0) < 0.05
            assert abs(noise[..., ch].mean()) < 0.05 * sd
    else:
        state = s0
        np.testing.assert_allclose(tgt, (s1 - s0) / inc_scale, rtol=1e-4,
                                   atol=1e-4 * np.abs((s1 - s0) / inc_scale).max())
    eta, u, v, d = state[..., 0], state[..., 1], state[..., 2], st[..., 0]
    gx, gy, div = _derived(eta, u, v, d)
    want = [(eta - ds.forcing(dom, snap)) / STATE_SCALE[0], u / STATE_SCALE[1], v / STATE_SCALE[2], d,
            ds.forcing(dom, snap) * st[..., 1] / STATE_SCALE[0],
            gx / ds.diff_scale[0], gy / ds.diff_scale[1], div / ds.diff_scale[2],
            st[..., 1], (eta - ds.forcing(dom, snap)) * st[..., 1] / STATE_SCALE[0],
            st[..., 2], st[..., 3]]
    got = x.float().cpu().numpy().reshape(n, n, CPAD_IN)
    for c, w in enumerate(want):
        np.testing.assert_allclose(got[..., c], w, rtol=2 ** -7, atol=2e-3 * np.abs(w).max(),
                                   err_msg="channel %d" % c)
    # low BF16 parts: high + low carries the state channels to ~2^-16
    for c in range(3):
        full = got[..., c].astype(np.float64) + got[..., 12 + c]
        np.testing.assert_allclose(full, want[c], rtol=2 ** -14, atol=1e-6 * np.abs(want[c]).max(),
                                   err_msg="channel %d high + low" % c)
    assert not got[..., 15:].any()


def test_emulator_beats_persistence_on_held_out_domains(gpulib, small_dataset):
    """Trained on 6 domains' solver trajectories, the network's 10-step ssh
    error on the 2 held-out domains is well below that of persistence (the
    state left unchanged, the method without the network)."""
    from psyclonebench_gb300.emulator import ConvNet, evaluate, train
    ds = small_dataset
    net = ConvNet(4, ds.n, ds.n, seed=2, lib=gpulib)
    hist = train(ds, net, iters=400, lr=2e-3, holdout=2)
    assert hist[-1] < 0.5 * hist[0]
    err_net, err_pers = evaluate(ds, net, [6, 7], list(range(2, ds.nsnap - 1, 3)))
    assert err_net < 0.5 * err_pers, (err_net, err_pers)


def test_hybrid_rollout_judges_and_falls_back(gpulib, small_dataset):
    """A roll-out with the FP64 solver re-running each window as judge (every
    domain judged every window here).  With an unreachable threshold the
    first window fails for both domains: they take the solver's window-end
    state and the solver advances them through the second window, so the
    result equals the pure-solver truth up to the FP32 hand-off of the state
    between windows.  With a loose threshold the emulator keeps every
    window and the judge still reports each window's error."""
    from psyclonebench_gb300.emulator import ConvNet, rollout
    ds = small_dataset
    net = ConvNet(4, ds.n, ds.n, seed=2, lib=gpulib)
    strict = rollout(ds, net, [6, 7], start_snap=2, emu_steps=6, judge_every=3, threshold=0.0,
                     judge_share=1.0)
    assert strict["judged"] == 2 and strict["judge_failed"] == 2
    assert strict["solver_windows"] == 2
    assert strict["final_ssh_rms_error_m"] < 1e-6
    loose = rollout(ds, net, [6, 7], start_snap=2, emu_steps=6, judge_every=3, threshold=1e9,
                    judge_share=1.0)
    assert loose["judged"] == 4 and loose["judge_failed"] == 0 and loose["solver_windows"] == 0
    assert len(loose["judge_errors_m"]) == 4
    assert all(e > 0 for e in loose["judge_errors_m"])
    # every domain judged in the last window continues from the solver's state
    assert loose["final_ssh_rms_error_m"] < 1e-6
    # a share of one half judges each domain every other window
    half = rollout(ds, net, [6, 7], start_snap=2, emu_steps=6, judge_every=3, threshold=1e9,
                   judge_share=0.5)
    assert half["judged"] == 2


def test_advance_applies_the_solver_boundary_conditions(gpulib, small_dataset):
    """state + increment x scale everywhere, except: zero velocity on wall
    faces and the tide at the target time on cells next to the open side."""
    import torch
    from psyclonebench_gb300.emulator import CPAD_OUT
    ds = small_dataset
    n = ds.n
    doms, tsnaps = [1, 4], [3, 9]
    torch.manual_seed(0)
    state = torch.randn(2, n * n, 3, device="cuda")
    out = torch.randn(2 * n * n, CPAD_OUT, device="cuda")
    want = state.cpu().numpy().astype(np.float64) + \
        out.cpu().numpy()[:, :3].reshape(2, n * n, 3) * np.array(ds.inc_scale)
    ds.advance(state, out, doms, tsnaps)
    torch.cuda.synchronize()
    got = state.cpu().numpy()
    for q, (d, t) in enumerate(zip(doms, tsnaps)):
        st = ds.statics[d].cpu().numpy()
        w = want[q].copy()
        w[st[:, 1] > 0, 0] = ds.forcing(d, t)
        w[st[:, 2] > 0, 1] = 0.0
        w[st[:, 3] > 0, 2] = 0.0
        assert (st[:, 1] > 0).any()
        np.testing.assert_allclose(got[q], w, rtol=1e-6, atol=1e-6)


def test_bounded_wait_runs_out_and_reports(gpulib):
    """The tcgen05 kernels' mbarrier waits are bounded: a wait on a barrier
    that nothing arrives on gives up after its limit (here 2^22 clocks, about
    2 ms), sets the error flag the host reads and returns; the context stays
    usable, so a convolution afterwards still matches its FP64 reference."""
    import ctypes
    st = ctypes.c_int(-1)
    assert gpulib.nl2d_selftest_wait(1 << 22, ctypes.byref(st)) == 0
    assert st.value == 1
    test_conv3x3_tcgen05_matches_fp64(gpulib, 16, 16, 0, 2, 5)
