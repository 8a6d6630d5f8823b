"""Runs the tracer-advection iteration on the GPU for profiling:
`python -m psyclonebench_gb300.probes.tra_adv [--size N] [--levels K] [--iters T]`.

The benchmark's own initial values (tra_adv.F90:63-98) on an N x N x K
domain, T iterations through tra_adv_compute, then the device time of T
more iterations (tra_adv_run) and the checksum."""
import argparse
import ctypes
import sys

from .. import load_library
from ..workloads import tra_adv_fields


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--size", type=int, default=512)
    ap.add_argument("--levels", type=int, default=75)
    ap.add_argument("--iters", type=int, default=3)
    a = ap.parse_args()
    lib = load_library()
    f = tra_adv_fields(a.size, a.size, a.levels)
    D = ctypes.POINTER(ctypes.c_double)
    args = [f[n].ctypes.data_as(D) for n in ("ztfreez", "pun", "pvn", "pwn", "umask", "vmask",
                                             "tmask", "rnfmsk", "rnfmsk_z", "upsmsk",
                                             "mydomain", "tsn")]
    for _ in range(a.iters):
        lib.tra_adv_compute(*args, a.size, a.size, a.levels)
    ms = ctypes.c_double(0.0)
    rc = lib.tra_adv_run(a.iters, ctypes.byref(ms))
    s = ctypes.c_double(0.0)
    rc = rc or lib.tra_adv_checksum(ctypes.byref(s))
    buf = ctypes.create_string_buffer(256)
    if rc or lib.tra_adv_last_error(buf, 256):
        print("tracer advection failed: %s" % buf.value.decode(), file=sys.stderr)
        sys.exit(1)
    print("%d x %d x %d: %.3f ms per iteration, checksum %.16e" % (
        a.size, a.size, a.levels, ms.value / max(1, a.iters), s.value))
    lib.tra_adv_finalize()


if __name__ == "__main__":
    main()
