"""Synthetic NEMOLite2D inputs beyond the reference's constant-depth
namelist configuration (the reference publishes no dataset).

* ``fourier_depth``: seeded smooth bathymetry, the sum of 16 Fourier modes
  about a mean depth, clipped to [50, 500] m and then to at least 20 m,
  evaluated at T, U (x + dx/2) and V (y + dy/2) points so that every form
  sees identical inputs.
* ``ensemble_domains``: seeded descriptions of many independent domains
  (sizes log-uniform per axis, bathymetry seed, tidal amplitude and period,
  which side is open).
"""
import math

import numpy as np

# Physics of the ensemble and emulator domains (configurations 3 and 4),
# which state bathymetry, tides and open sides but not viscosity or
# friction.  These take the reference namelist reader's own defaults,
# visc = 100 m^2/s and cbfr = 1e-3 (common/gocean2d_io_mod.f90:57-68); the
# parity namelist's 0.1 and 1.5e-4 (original/namelist.128) describe a
# flat-bottomed basin with a 0.2 m tide.  With those weak values, tides of
# up to 0.5 m over 50-500 m Fourier bathymetry drive the open-boundary
# faces of the scheme's explicit step into growth: about half of the seeded
# domains overflow within 5000 steps at rdt = 5 s (a quarter at rdt = 1 s,
# so not a time-step limit), where with the defaults 1 of 64 does.
ENSEMBLE_RDT = 5.0     # s; 500 m of water carries gravity waves at 70 m/s
ENSEMBLE_CBFR = 1.0e-3
ENSEMBLE_VISC = 100.0


def fourier_depth(width, height, seed, mean=275.0, nmodes=16, dx=1000.0, dy=1000.0):
    """(ht, hu, hv) as [height][width] FP64 arrays."""
    rng = np.random.default_rng(seed)
    lx, ly = width * dx, height * dy
    m = rng.integers(-6, 7, size=nmodes)
    n = rng.integers(-6, 7, size=nmodes)
    zero = (m == 0) & (n == 0)
    m[zero] = 1
    a = rng.uniform(10.0, 35.0, size=nmodes)
    ph = rng.uniform(0.0, 2.0 * math.pi, size=nmodes)
    x_t = np.arange(width, dtype=np.float64) * dx
    y_t = np.arange(height, dtype=np.float64) * dy

    def depth(x, y):
        # cos(A + B) = cos A cos B - sin A sin B with A along x, B along y:
        # each mode is two outer products of 1-D vectors.
        h = np.full((y.size, x.size), mean)
        for k in range(nmodes):
            A = 2.0 * math.pi * m[k] * x / lx + ph[k]
            B = 2.0 * math.pi * n[k] * y / ly
            h += a[k] * (np.outer(np.cos(B), np.cos(A)) - np.outer(np.sin(B), np.sin(A)))
        return np.maximum(np.clip(h, 50.0, 500.0), 20.0)

    return depth(x_t, y_t), depth(x_t + 0.5 * dx, y_t), depth(x_t, y_t + 0.5 * dy)


def ensemble_domains(count, seed, lo=64, hi=1024):
    """List of dicts: nx, ny (interior cells), depth_seed, tide_amp (m),
    tide_period_h, open_side in {"S", "N", "E", "W"}."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        nx = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
        ny = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
        out.append({
            "nx": nx, "ny": ny,
            "depth_seed": int(rng.integers(0, 2 ** 31 - 1)),
            "tide_amp": float(rng.uniform(0.05, 0.5)),
            "tide_period_h": float(rng.uniform(10.0, 14.0)),
            "open_side": "SNEW"[int(rng.integers(0, 4))],
        })
    return out


def tra_adv_fields(jpi, jpj, jpk):
    """The tracer-advection benchmark's initial values
    (tracer_advection/original/tra_adv.F90:63-98), Fortran layout
    a(ji, jj, jk) -> a[jk, jj, ji]: the 3-d fields k j i / (jpi jpj jpk),
    the 2-d ones j i / (jpi jpj), rnfmsk_z(jk) = jk / jpk in integer
    division."""
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
