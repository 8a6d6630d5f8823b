"""Generates the golden fixtures in this directory from the reference's own
serial PSy layer (psykal_cpp/time_step.cpp + kernels/c_family/*.c), compiled
unchanged by `make -C oracle ref` into oracle/_ref/libnl2d_ref_serial.so.

Run here, where the reference checkout exists:
    make -C oracle ref && python tests/golden/make_golden.py

Each case starts from the reference's initial state (model_init +
initialisation, restated in tests/nl2d_testlib.py) or from a seeded
bathymetry, runs the reference step, and stores the final 13 fields (small
grids) or the per-100-step checksums (the 128x128 parity configuration).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
import nl2d_testlib as T  # noqa: E402

# (name, jpiglo, jpjglo, jphgr_msh, nsteps, width pad, bathymetry seed or None)
FIELD_CASES = [
    ("small_s_open", 24, 18, 1, 120, 0, None),
    ("small_e_open", 19, 21, 2, 90, 3, None),
    ("small_se_open", 20, 20, 3, 150, 0, None),
    ("small_bathy", 23, 17, 1, 80, 5, 7),
]


def bathymetry(m, seed):
    """Smooth seeded depth (50-500 m) at T, U and V points."""
    rng = np.random.default_rng(seed)
    H, W = m.height, m.width
    jj, ii = np.mgrid[0:H, 0:W].astype(np.float64)
    k = rng.integers(1, 4, size=(4, 2))
    a = rng.uniform(20.0, 80.0, size=4)
    ph = rng.uniform(0.0, 2 * np.pi, size=4)

    def depth(x, y):
        h = 200.0 + sum(a[q] * np.cos(2 * np.pi * (k[q, 0] * x / W + k[q, 1] * y / H) + ph[q])
                        for q in range(4))
        return np.clip(h, 50.0, 500.0)

    m.f["ht"][:] = depth(ii, jj)
    m.f["hu"][:] = depth(ii + 0.5, jj)
    m.f["hv"][:] = depth(ii, jj + 0.5)


def main():
    ref = T.load_ref("serial")
    if ref is None:
        sys.exit("oracle/_ref/libnl2d_ref_serial.so is missing: run `make -C oracle ref`")
    for name, nx, ny, jphgr, nsteps, pad, seed in FIELD_CASES:
        m = T.make_model(nx, ny, jphgr, width=nx + 1 + pad)
        if seed is not None:
            bathymetry(m, seed)
        init = {k: v.copy() for k, v in m.f.items()}
        T.run(ref.c_invoke_time_step, m, nsteps)
        np.savez_compressed(
            os.path.join(HERE, name + ".npz"),
            meta=np.array([nx, ny, jphgr, nsteps, m.width, m.height], np.int64),
            **{"init_" + k: v for k, v in init.items() if k in ("ht", "hu", "hv")},
            **{"final_" + k: m.f[k] for k in T.FIELDS})
        print(name, "ok")
    # The 128x128 parity configuration: checksums every 100 steps.
    m = T.make_model(130, 130, 1)
    sums = []
    T.run(ref.c_invoke_time_step, m, 2000, every=100, checksums=sums)
    arr = np.array([[s[k] for k in ("sshn_t", "un", "vn", "ua", "va")] for s in sums])
    np.savetxt(os.path.join(HERE, "cfg0_checksums.txt"), arr, fmt="%.17e",
               header="130x130 namelist (128x128 interior), jphgr_msh=1, rdt=20, "
                      "cbfr=1.5e-4, visc=0.1, dep=100; columns: sshn_t un vn ua va "
                      "checksums after steps 100, 200, ..., 2000 (reference serial build)")
    print("cfg0 ok")


if __name__ == "__main__":
    main()
