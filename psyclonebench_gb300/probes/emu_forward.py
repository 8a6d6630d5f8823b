"""Runs the emulator network on synthetic inputs for profiling:
`python -m psyclonebench_gb300.probes.emu_forward [--batch B] [--reps R] [--train T]`.

B images of 256 x 256 pixels (at B = 24 every 48-channel activation, 151 MB,
is larger than L2), R forward passes, then T training steps (forward, loss,
input- and weight-gradient convolutions, Adam).  Prints the CUDA-event time
of each phase."""
import argparse
import sys

import torch

from .. import load_library
from .. import emulator as E


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--batch", type=int, default=24)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--train", type=int, default=1)
    a = ap.parse_args()
    lib = load_library()
    net = E.ConvNet(a.batch, 256, 256, seed=0, lib=lib)
    P = a.batch * 256 * 256
    g = torch.Generator(device="cuda").manual_seed(0)
    x = torch.randn(P, E.CPAD_IN, device="cuda", generator=g).to(torch.bfloat16)
    target = torch.randn(P, 3, device="cuda", generator=g)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(a.reps):
        net.forward(x)
    e1.record()
    torch.cuda.synchronize()
    print("forward: %.3f ms per pass (%d images of 256^2)" % (
        e0.elapsed_time(e1) / max(1, a.reps), a.batch))
    if a.train:
        e0.record()
        for _ in range(a.train):
            net.train_step(x, target)
        e1.record()
        torch.cuda.synchronize()
        print("train step: %.3f ms" % (e0.elapsed_time(e1) / a.train))
    if int(net.err.item()) != 0:
        print("a tensor-core wait ran out", file=sys.stderr)
        sys.exit(1)


if __name__ == "__main__":
    main()
