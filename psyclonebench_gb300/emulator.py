"""Learned emulator of the NEMOLite2D solver (no counterpart in the
reference): a residual CNN that advances (ssh, u, v) by k = 10 solver steps,
trained only on trajectories the solver itself generates, with the FP64
solver as judge and fallback during roll-outs.

Network: six 3x3 convolutions, 48 channels, ReLU between them, inputs
(ssh, u, v, depth, tidal forcing) in BF16, FP32 accumulation; the output is
the increment of the state, scaled.  Every FLOP of the forward pass, the
backward pass and inference runs in this library's kernels: the tcgen05
implicit-GEMM convolution (forward, and the input gradient with flipped,
transposed weights), the FP32 weight-gradient reduction, the loss and Adam
kernels.  torch only provides device buffers.

Pixels are the interior T cells of a domain; pixel (i, j) carries sshn_t,
and un / vn of the east / north faces of that cell.  The forcing channel is
the tide's bc_ssh value at the target time on wet cells next to the open
side, zero elsewhere; depth is ht / 500 m.
"""
import ctypes
import math
import time

import numpy as np

from . import NL2D_OK, Nl2dError, load_library
from .ensemble import Ensemble, build_domain
from .workloads import ensemble_domains

CPAD_IN = 16   # 5 input channels padded for the MMA K granularity
CPAD_OUT = 16  # 3 output channels padded (N multiple of 16)
WIDTH = 48
LAYERS = [(CPAD_IN, WIDTH, 1)] + [(WIDTH, WIDTH, 1)] * 4 + [(WIDTH, CPAD_OUT, 0)]
K_STEPS = 10
STATE_SCALE = (0.5, 1.0, 1.0)  # m, m/s, m/s


def _torch():
    import torch
    return torch


def _ck(rc, what):
    if rc != NL2D_OK:
        raise Nl2dError("%s failed (%d)" % (what, rc))


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def tide_value(amp, period_h, istep, rdt):
    """bc_ssh_code's value (boundary_conditions_kern.c:183-192) with this
    domain's amplitude and period."""
    omega_tide = 2.0 * 3.14159 / (period_h * 3600.0)
    return amp * math.sin(omega_tide * (istep * rdt))


class ConvNet:
    """Parameters and buffers of the 6-layer network for a fixed batch."""

    def __init__(self, batch, H, W, seed=0, lib=None):
        torch = _torch()
        self.lib = lib or load_library()
        self.batch, self.H, self.W = batch, H, W
        g = torch.Generator().manual_seed(seed)
        self.w32, self.w16, self.b, self.dw, self.db = [], [], [], [], []
        self.mw, self.vw, self.mb, self.vb, self.wt = [], [], [], [], []
        for cin, cout, _ in LAYERS:
            fan_in = 9 * (5 if cin == CPAD_IN else cin)
            w = torch.randn(9, cout, cin, generator=g) * math.sqrt(2.0 / fan_in)
            if cin == CPAD_IN:
                w[:, :, 5:] = 0.0
            if cout == CPAD_OUT:
                w *= 0.1  # start near the identity step (zero increment)
            w = w.cuda()
            self.w32.append(w)
            self.w16.append(w.to(torch.bfloat16))
            self.b.append(torch.zeros(cout, device="cuda"))
            self.dw.append(torch.zeros_like(w))
            self.db.append(torch.zeros(cout, device="cuda"))
            self.mw.append(torch.zeros_like(w))
            self.vw.append(torch.zeros_like(w))
            self.mb.append(torch.zeros(cout, device="cuda"))
            self.vb.append(torch.zeros(cout, device="cuda"))
            self.wt.append(torch.zeros(9, cin, cout, dtype=torch.bfloat16, device="cuda"))
        P = batch * H * W
        self.acts = [torch.zeros(P, c, dtype=torch.bfloat16, device="cuda") for _, c, _ in LAYERS]
        self.out32 = torch.zeros(P, CPAD_OUT, device="cuda")
        self.gbuf = [torch.zeros(P, c, dtype=torch.bfloat16, device="cuda") for c, _, _ in LAYERS]
        self.g32 = torch.zeros(P, WIDTH, device="cuda")
        self.gout = torch.zeros(P, CPAD_OUT, dtype=torch.bfloat16, device="cuda")
        self.err = torch.zeros(1, dtype=torch.int32, device="cuda")
        self.loss = torch.zeros(1, device="cuda")
        self.step = 0

    def _conv(self, x, w, b, y, y32, batch, cin, cout, relu):
        _ck(self.lib.nl2d_emu_conv3x3(_p(x), _p(w), _p(b) if b is not None else None,
                                      _p(y) if y is not None else None,
                                      _p(y32) if y32 is not None else None, batch, self.H,
                                      self.W, cin, cout, relu, _p(self.err), None),
            "nl2d_emu_conv3x3")

    def forward(self, x, batch=None):
        """x: BF16 [batch*H*W, CPAD_IN] -> FP32 increments out32[:, :3]."""
        batch = batch or self.batch
        inp = x
        for li, (cin, cout, relu) in enumerate(LAYERS):
            last = li == len(LAYERS) - 1
            self._conv(inp, self.w16[li], self.b[li], None if last else self.acts[li],
                       self.out32 if last else None, batch, cin, cout, relu)
            inp = self.acts[li]
        return self.out32

    def train_step(self, x, target, lr=1e-3):
        """One Adam step on the batch (x BF16, target FP32 [P, 3]); returns
        the loss of the batch before the step."""
        torch = _torch()
        P = self.batch * self.H * self.W
        self.forward(x)
        self.loss.zero_()
        _ck(self.lib.nl2d_emu_mse(_p(self.out32), _p(target), _p(self.gout), _p(self.loss),
                                  P, 3, CPAD_OUT, None), "nl2d_emu_mse")
        for t in self.dw + self.db:
            t.zero_()
        g = self.gout  # gradient of the loss w.r.t. layer li's pre-activation
        for li in range(len(LAYERS) - 1, -1, -1):
            cin, cout, _ = LAYERS[li]
            xin = x if li == 0 else self.acts[li - 1]
            _ck(self.lib.nl2d_emu_conv_wgrad(_p(xin), _p(g), _p(self.dw[li]), _p(self.db[li]),
                                             self.batch, self.H, self.W, cin, cout, None),
                "nl2d_emu_conv_wgrad")
            if li == 0:
                break
            _ck(self.lib.nl2d_emu_flip_transpose(_p(self.w16[li]), _p(self.wt[li]), cout, cin,
                                                 None), "nl2d_emu_flip_transpose")
            g32 = self.g32[:, :cin] if cin < WIDTH else self.g32
            g32 = g32.contiguous() if cin < WIDTH else g32
            self._conv(g, self.wt[li], None, None, g32, self.batch, cout, cin, 0)
            gprev = self.gbuf[li]
            _ck(self.lib.nl2d_emu_relu_bwd(_p(g32), _p(self.acts[li - 1]), _p(gprev),
                                           P * cin, None), "nl2d_emu_relu_bwd")
            g = gprev
        self.step += 1
        for li in range(len(LAYERS)):
            _ck(self.lib.nl2d_emu_adam(_p(self.w32[li]), _p(self.mw[li]), _p(self.vw[li]),
                                       _p(self.dw[li]), _p(self.w16[li]), self.w32[li].numel(),
                                       lr, 0.9, 0.999, 1e-8, self.step, None), "adam w")
            _ck(self.lib.nl2d_emu_adam(_p(self.b[li]), _p(self.mb[li]), _p(self.vb[li]),
                                       _p(self.db[li]), None, self.b[li].numel(), lr, 0.9,
                                       0.999, 1e-8, self.step, None), "adam b")
        torch.cuda.synchronize()
        if int(self.err.item()) != 0:
            raise Nl2dError("tensor-core convolution timed out waiting for its MMAs")
        return float(self.loss.item())


def emulator_domain_specs(count, seed, n=256):
    """Config-3-style domains of a fixed n x n interior."""
    specs = ensemble_domains(count, seed)
    for s in specs:
        s["nx"] = s["ny"] = n
    return specs


class Dataset:
    """Solver trajectories of `count` seeded domains on the GPU:
    snaps [count * nsnap][n][n][3] FP32 (every K_STEPS steps), statics
    [count][n][n][2]."""

    def __init__(self, count=200, nsnap=101, seed=11, n=256, rdt=5.0, lib=None):
        torch = _torch()
        self.lib = lib or load_library()
        self.n, self.nsnap, self.rdt = n, nsnap, rdt
        self.specs = emulator_domain_specs(count, seed, n)
        doms = [build_domain(s) for s in self.specs]
        self.doms = doms
        ens = Ensemble(doms, rdt=rdt, lib=self.lib)
        HW = n * n
        self.snaps = torch.zeros(count, nsnap, HW, 3, device="cuda")
        buf = torch.zeros(count, HW, 3, device="cuda")
        t0 = time.perf_counter()
        ens.run(1, 0)  # builds the schedule
        solver_ms = 0.0
        for s in range(nsnap):
            if s > 0:
                ms, _ = ens.run(1 + (s - 1) * K_STEPS, K_STEPS)
                solver_ms += ms
            _ck(self.lib.nl2d_ens_export_interior(ctypes.c_void_p(buf.data_ptr())), "export")
            self.snaps[:, s] = buf
        self.gen_seconds = time.perf_counter() - t0
        self.solver_ms_per_step = solver_ms / max(1, (nsnap - 1) * K_STEPS)
        ens.close()
        self.snaps = self.snaps.reshape(count * nsnap, HW, 3)
        st = np.zeros((count, HW, 2), np.float32)
        for k, d in enumerate(doms):
            w, h, xs, xe, ys, ye = d["dims"]
            st[k, :, 0] = (d["ht"][ys:ye + 1, xs:xe + 1] / 500.0).reshape(-1)
            m = d["tmask"]
            inner = m[ys:ye + 1, xs:xe + 1] > 0
            nb = ((m[ys - 1:ye, xs:xe + 1] < 0) | (m[ys + 1:ye + 2, xs:xe + 1] < 0) |
                  (m[ys:ye + 1, xs - 1:xe] < 0) | (m[ys:ye + 1, xs + 1:xe + 2] < 0))
            st[k, :, 1] = (inner & nb).reshape(-1).astype(np.float32)
        self.statics = torch.tensor(st, device="cuda")
        # increment scales from the data (RMS of each channel's k-step change),
        # accumulated domain by domain
        acc = torch.zeros(3, dtype=torch.float64, device="cuda")
        view = self.snaps.reshape(count, nsnap, HW, 3)
        for k in range(count):
            inc = view[k, 1:] - view[k, :-1]
            acc += inc.double().pow(2).sum(dim=(0, 1))
        rms = (acc / (count * (nsnap - 1) * HW)).sqrt().cpu().numpy()
        self.inc_scale = tuple(float(max(v, 1e-12)) for v in rms)

    def forcing(self, dom, snap):
        """Tide at the target time of pair (dom, snap)."""
        s = self.specs[dom]
        return tide_value(s["tide_amp"], s["tide_period_h"], (snap + 1) * K_STEPS, self.rdt)

    def batch(self, pairs, x, target):
        """Fills x (BF16) and target (FP32, or None) for (dom, snap) pairs."""
        torch = _torch()
        src = torch.tensor([d * self.nsnap + s for d, s in pairs], dtype=torch.int32,
                           device="cuda")
        dom = torch.tensor([d for d, _ in pairs], dtype=torch.int32, device="cuda")
        forcing = torch.tensor([self.forcing(d, s) for d, s in pairs], dtype=torch.float32,
                               device="cuda")
        scale6 = (ctypes.c_float * 6)(*(STATE_SCALE + self.inc_scale))
        _ck(self.lib.nl2d_emu_assemble(_p(self.snaps), _p(self.statics), _p(src), _p(dom),
                                       _p(forcing), scale6, _p(x),
                                       _p(target) if target is not None else None,
                                       self.n * self.n, CPAD_IN, len(pairs), None),
            "nl2d_emu_assemble")


def train(ds, net, iters=2000, lr=1e-3, seed=0, holdout=20):
    """Trains on pairs of the first count - holdout domains; returns the loss
    history."""
    torch = _torch()
    rng = np.random.default_rng(seed)
    ntrain = len(ds.specs) - holdout
    P = net.batch * ds.n * ds.n
    x = torch.zeros(P, CPAD_IN, dtype=torch.bfloat16, device="cuda")
    tgt = torch.zeros(P, 3, device="cuda")
    hist = []
    for it in range(iters):
        pairs = [(int(rng.integers(0, ntrain)), int(rng.integers(0, ds.nsnap - 1)))
                 for _ in range(net.batch)]
        ds.batch(pairs, x, tgt)
        hist.append(net.train_step(x, tgt, lr=lr * (0.1 if it > 0.8 * iters else 1.0)))
    return hist


def evaluate(ds, net, domains, snaps):
    """ssh RMS error (m) of one emulator step on held-out pairs, for the
    network and for persistence (no change)."""
    torch = _torch()
    P = net.batch * ds.n * ds.n
    x = torch.zeros(P, CPAD_IN, dtype=torch.bfloat16, device="cuda")
    tgt = torch.zeros(P, 3, device="cuda")
    pairs = [(d, s) for d in domains for s in snaps]
    se_net = se_pers = 0.0
    count = 0
    for k in range(0, len(pairs), net.batch):
        chunk = pairs[k:k + net.batch]
        ds.batch(chunk, x, tgt)
        out = net.forward(x, batch=len(chunk))
        torch.cuda.synchronize()
        n = len(chunk) * ds.n * ds.n
        d_net = (out[:n, 0] - tgt[:n, 0]) * ds.inc_scale[0]
        d_pers = tgt[:n, 0] * ds.inc_scale[0]
        se_net += float(d_net.pow(2).sum())
        se_pers += float(d_pers.pow(2).sum())
        count += d_net.numel()
    return math.sqrt(se_net / count), math.sqrt(se_pers / count)


def rollout(ds, net, domains, start_snap, emu_steps=500, judge_every=50, threshold=1e-3):
    """Hybrid roll-out of `domains` (indices into ds) from snapshot
    start_snap: the emulator advances K_STEPS solver steps per step; every
    judge_every emulator steps the FP64 solver advances the same state by
    K_STEPS steps and the ssh RMS difference of the two is the judge's error;
    above `threshold` (m) the next window runs on the solver instead.  A
    pure-solver run from the same start gives the truth.  Returns a report."""
    torch = _torch()
    lib = ds.lib
    nd, n = len(domains), ds.n
    HW = n * n
    assert nd <= net.batch
    sol = Ensemble([ds.doms[d] for d in domains], rdt=ds.rdt, lib=lib)
    sol.run(1, 0)
    state = torch.stack([ds.snaps[d * ds.nsnap + start_snap] for d in domains]).contiguous()
    start = state.clone()
    x = torch.zeros(net.batch * HW, CPAD_IN, dtype=torch.bfloat16, device="cuda")
    inc_scale = (ctypes.c_float * 3)(*ds.inc_scale)
    scale6 = (ctypes.c_float * 6)(*(STATE_SCALE + ds.inc_scale))
    src = torch.arange(nd, dtype=torch.int32, device="cuda")
    domt = torch.tensor(list(domains), dtype=torch.int32, device="cuda")
    buf = torch.zeros(nd, HW, 3, device="cuda")
    report = {"windows_emulator": 0, "windows_solver": 0, "judge_errors_m": []}
    step0 = start_snap * K_STEPS
    emu_ms = sol_ms = 0.0

    def emu_step(st, istep):
        forcing = torch.tensor([tide_value(ds.specs[d]["tide_amp"], ds.specs[d]["tide_period_h"],
                                           istep + K_STEPS, ds.rdt) for d in domains],
                               dtype=torch.float32, device="cuda")
        _ck(lib.nl2d_emu_assemble(_p(st), _p(ds.statics), _p(src), _p(domt), _p(forcing),
                                  scale6, _p(x), None, HW, CPAD_IN, nd, None), "assemble")
        out = net.forward(x, batch=nd)
        _ck(lib.nl2d_emu_advance(_p(st), _p(out), inc_scale, nd * HW, CPAD_OUT, None),
            "advance")

    def solve(st, istep, nsteps):
        _ck(lib.nl2d_ens_import_interior(_p(st)), "import")
        ms, _ = sol.run(istep + 1, nsteps)
        _ck(lib.nl2d_ens_export_interior(_p(buf)), "export")
        return buf.clone(), ms

    istep = step0
    k = 0
    while k < emu_steps:
        # judge: one emulator step against K_STEPS solver steps from this state
        pred = state.clone()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        emu_step(pred, istep)
        torch.cuda.synchronize()
        emu_ms += (time.perf_counter() - t0) * 1e3
        ref, ms = solve(state, istep, K_STEPS)
        sol_ms += ms
        err = float((pred[:, :, 0] - ref[:, :, 0]).pow(2).mean().sqrt())
        report["judge_errors_m"].append(err)
        window = min(judge_every, emu_steps - k)
        if err > threshold:
            state, ms = solve(state, istep, window * K_STEPS)
            sol_ms += ms
            report["windows_solver"] += 1
        else:
            state = pred
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for q in range(1, window):
                emu_step(state, istep + q * K_STEPS)
            torch.cuda.synchronize()
            emu_ms += (time.perf_counter() - t0) * 1e3
            report["windows_emulator"] += 1
        istep += window * K_STEPS
        k += window
    truth, truth_ms = solve(start, step0, emu_steps * K_STEPS)
    sol.close()
    d = (state[:, :, 0] - truth[:, :, 0])
    report.update({
        "emu_steps": emu_steps, "solver_steps_equivalent": emu_steps * K_STEPS,
        "final_ssh_rms_error_m": float(d.pow(2).mean().sqrt()),
        "final_ssh_rms_m": float(truth[:, :, 0].pow(2).mean().sqrt()),
        "hybrid_ms": emu_ms + sol_ms, "emulator_ms": emu_ms, "judge_and_fallback_ms": sol_ms,
        "solver_only_ms": truth_ms,
    })
    return report
