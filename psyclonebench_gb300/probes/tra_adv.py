"""Runs the tracer-advection iteration on the GPU for profiling:
`python -m psyclonebench_gb300.probes.tra_adv [--size N] [--levels K] [--iters T]`.

The benchmark's own initial values (tra_adv.F90:63-98) on an N x N x K
domain, T iterations through tra_adv_compute, then the device time of T
more iterations (tra_adv_run) and the checksum."""
import argparse
import ctypes
import sys

import numpy as np

from .. import load_library


def benchmark_fields(jpi, jpj, jpk):
    k, j, i = np.meshgrid(np.arange(1, jpk + 1), np.arange(1, jpj + 1), np.arange(1, jpi + 1),
                          indexing="ij")
    v3 = (k * j * i).astype(np.float64) / float(jpi * jpj * jpk)
    j2, i2 = np.meshgrid(np.arange(1, jpj + 1), np.arange(1, jpi + 1), indexing="ij")
    v2 = (j2 * i2).astype(np.float64) / float(jpi * jpj)
    f = {n: v3.copy() for n in ("mydomain", "tsn", "pun", "pvn", "pwn", "umask", "vmask",
                                "tmask")}
    f.update({n: v2.copy() for n in ("ztfreez", "rnfmsk", "upsmsk")})
    f["rnfmsk_z"] = np.array([float(kk // jpk) for kk in range(1, jpk + 1)])
    return f


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--size", type=int, default=512)
    ap.add_argument("--levels", type=int, default=75)
    ap.add_argument("--iters", type=int, default=3)
    a = ap.parse_args()
    lib = load_library()
    f = benchmark_fields(a.size, a.size, a.levels)
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
