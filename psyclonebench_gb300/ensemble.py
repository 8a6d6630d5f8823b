"""Host side of the ensemble form: many independent NEMOLite2D domains
(uneven sizes, bathymetries, tides, open sides) advanced together by one
persistent kernel launch per step (libnl2d_gpu's nl2d_ens_* entry points).

Each domain is laid out like the reference's single domain: interior
nx x ny T cells inside a one-cell boundary ring, fields one larger than the
mask for the NE stagger, rows padded to 8 doubles.  The T-mask generalises
setup_tpoints_mask (common/model_mod.f90:94-249), which opens the south
and/or east side, to an open side S, N, E or W, keeping its assignment order
(west, north, east, south).
"""
import ctypes

import numpy as np

from . import NL2D_OK, Nl2dError, load_library
from .workloads import ENSEMBLE_CBFR, ENSEMBLE_RDT, ENSEMBLE_VISC, fourier_depth

PI = 3.1415926535897932
G = 9.80665
OMEGA = 7.292116e-05
D2R = PI / 180.0

_DP = ctypes.POINTER(ctypes.c_double)
_IP = ctypes.POINTER(ctypes.c_int)


def _dp(a):
    return a.ctypes.data_as(_DP)


def _ip(a):
    return a.ctypes.data_as(_IP)


def domain_layout(nx, ny):
    """(width, height, xs, xe, ys, ye) for an nx x ny interior."""
    jpi, jpj = nx + 2, ny + 2
    width = ((jpi + 1 + 7) // 8) * 8
    return width, jpj + 1, 1, jpi - 2, 1, jpj - 2


def open_side_mask(side, width, height, xs, xe, ys, ye):
    m = np.zeros((height, width), np.int32)
    m[ys:ye + 1, xs:xe + 1] = 1
    m[:, :xs] = -1 if side == "W" else 0
    m[ye + 1:, :] = -1 if side == "N" else 0
    m[:, xe + 1:] = -1 if side == "E" else 0
    m[:ys, :] = -1 if side == "S" else 0
    return m


def build_domain(spec):
    """Arrays of one domain from an ensemble_domains() spec."""
    width, height, xs, xe, ys, ye = domain_layout(spec["nx"], spec["ny"])
    ht, hu, hv = fourier_depth(width, height, spec["depth_seed"])
    return {"dims": (width, height, xs, xe, ys, ye),
            "tmask": open_side_mask(spec["open_side"], width, height, xs, xe, ys, ye),
            "ht": ht, "hu": hu, "hv": hv,
            "tide": (spec["tide_amp"], spec["tide_period_h"])}


def shard_domains(specs, world):
    """Partition domain indices over `world` ranks, balanced by interior
    cells (largest first to the least-loaded rank).  Each domain lands on
    exactly one rank; no data moves between ranks during a run."""
    order = sorted(range(len(specs)), key=lambda k: -specs[k]["nx"] * specs[k]["ny"])
    load = [0] * world
    parts = [[] for _ in range(world)]
    for k in order:
        r = min(range(world), key=lambda q: load[q])
        parts[r].append(k)
        load[r] += specs[k]["nx"] * specs[k]["ny"]
    return [sorted(p) for p in parts]


def gather_results(local, timeout_s=30.0):
    """Merges every rank's {domain index: result} over the default process
    group (host side; the domains never exchange data during a run).  A
    monitored barrier runs first: a rank that died or never reaches the
    gather makes rank 0 fail within `timeout_s` with Nl2dError naming the
    ranks that did not report, instead of waiting forever.  Needs the gloo
    backend (the barrier's failure report is gloo's)."""
    import datetime

    import torch.distributed as dist
    try:
        dist.monitored_barrier(timeout=datetime.timedelta(seconds=timeout_s),
                               wait_all_ranks=True)
    except RuntimeError as e:
        raise Nl2dError("ensemble ranks did not report: %s" % str(e).splitlines()[0]) from e
    gathered = [None] * dist.get_world_size()
    dist.all_gather_object(gathered, local)
    merged = {}
    for g in gathered:
        merged.update(g)
    return merged


class Ensemble:
    """A set of domains resident on the GPU.  `domains` are build_domain()
    dicts; all share rdt, cbfr and visc (by default the ensemble
    configuration's, workloads.ENSEMBLE_*), and dx, dy and latitude unless a
    domain carries its own as "geo": (dx, dy, gphi)."""

    def __init__(self, domains, rdt=ENSEMBLE_RDT, cbfr=ENSEMBLE_CBFR, visc=ENSEMBLE_VISC,
                 dx=1000.0, dy=1000.0, gphi=50.0, lib=None):
        self.lib = lib or load_library()
        self.domains = domains
        n = len(domains)
        dims = np.array([d["dims"] for d in domains], np.int32).reshape(-1)
        geo = np.array([d.get("geo", (dx, dy, gphi)) for d in domains], np.float64).reshape(-1)
        tide = np.array([d["tide"] for d in domains], np.float64).reshape(-1)
        phys = np.array([rdt, cbfr, visc, OMEGA, D2R, G], np.float64)
        self._check(self.lib.nl2d_ens_create(n, _ip(dims), _dp(geo), _dp(tide), _dp(phys)),
                    "nl2d_ens_create")
        for k, d in enumerate(domains):
            self._check(self.lib.nl2d_ens_set_domain(
                k, _ip(np.ascontiguousarray(d["tmask"])), _dp(np.ascontiguousarray(d["ht"])),
                _dp(np.ascontiguousarray(d["hu"])), _dp(np.ascontiguousarray(d["hv"]))),
                "nl2d_ens_set_domain(%d)" % k)

    @staticmethod
    def _check(rc, what):
        if rc != NL2D_OK:
            raise Nl2dError("%s failed (%d)" % (what, rc))

    def uses_march(self):
        """Whether the mixed-precision form has been built (it runs the
        column march, with per-domain constants where the domains' grids
        differ)."""
        return bool(self.lib.nl2d_ens_uses_march())

    def schedule(self, ctas_per_sm=2, policy=0, boundary_weight=4.0, tile=(32, 16),
                 march_rows=32):
        """Schedule and tile knobs (nl2d_ens_schedule, nl2d_ens_tile): CTAs
        per SM, tile assignment policy, boundary-edge cost weight, the FP64
        tile shape and the mixed form's march strip height."""
        self._check(self.lib.nl2d_ens_schedule(ctas_per_sm, policy, boundary_weight),
                    "nl2d_ens_schedule")
        self._check(self.lib.nl2d_ens_tile(int(tile[0]), int(tile[1]), march_rows),
                    "nl2d_ens_tile")

    def run(self, istep0, nsteps, checksum_every=0):
        """Returns (device ms, checksums [samples, domains, 3])."""
        nsums = nsteps // checksum_every if checksum_every else 0
        out = np.zeros(max(1, nsums * len(self.domains) * 3), np.float64)
        ms = ctypes.c_double(0.0)
        self._check(self.lib.nl2d_ens_run(istep0, nsteps, checksum_every, _dp(out),
                                          ctypes.byref(ms)), "nl2d_ens_run")
        return ms.value, out[:nsums * len(self.domains) * 3].reshape(nsums, len(self.domains), 3)

    def set_precision(self, precision):
        """0: FP64 (bit-identical to the reference); 1: mixed; 2:
        FP64-equivalent (double-float interior, exact FP64 elsewhere).
        Restarts every domain from rest."""
        self._check(self.lib.nl2d_ens_set_precision(precision), "nl2d_ens_set_precision")

    def reset(self):
        self._check(self.lib.nl2d_ens_reset(), "nl2d_ens_reset")

    def read(self, k):
        w, h = self.domains[k]["dims"][:2]
        sn, un, vn = (np.zeros((h, w)) for _ in range(3))
        self._check(self.lib.nl2d_ens_read(k, _dp(sn), _dp(un), _dp(vn)), "nl2d_ens_read")
        return sn, un, vn

    def info(self):
        cells, ntiles, nctas = ctypes.c_longlong(0), ctypes.c_int(0), ctypes.c_int(0)
        self.lib.nl2d_ens_info(ctypes.byref(cells), ctypes.byref(ntiles), ctypes.byref(nctas))
        return cells.value, ntiles.value, nctas.value

    def close(self):
        self.lib.nl2d_ens_destroy()
