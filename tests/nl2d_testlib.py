"""Shared helpers for the NEMOLite2D tests: loading the CPU oracle (and, when
it was built here, the reference's own compiled PSy layer), building
dl_esm_inf-style models as numpy arrays, and stepping them.

The oracle is only ever what the tests compare with; the GPU library is the
thing under test.
"""
import os
import sys

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

from oracle import cpu as _O  # noqa: E402
from oracle.cpu import (REF_ARGTYPES, STEP_ARGTYPES, build_oracle,  # noqa: E402,F401
                        load_oracle, load_ref)
from psyclonebench_gb300.model import (D2R, FIELDS, G, GRID, OMEGA, PI,  # noqa: E402,F401
                                       Model, dptr, iptr)

STATE = ("sshn_t", "un", "vn", "ua", "va", "ssha_t", "sshn_u", "sshn_v")


def make_model(jpiglo=130, jpjglo=130, jphgr_msh=1, dx=1000.0, dy=1000.0,
               dep_const=100.0, width=None, height=None, oracle=None):
    """The reference's start state through the oracle's set-up
    (model_mod.f90:26-69, initialisation_mod.f90:7-63)."""
    return _O.setup_model(Model(jpiglo, jpjglo, width, height), jphgr_msh, dx, dy,
                          dep_const, lib=oracle)


def run(step_fn, m, nsteps, nit000=1, every=0, checksums=None):
    """Advance `m` in place by nsteps calls of step_fn (a ctypes function with
    the 7-int argument list, or the reference's 6-int one)."""
    nargs = len(step_fn.argtypes)
    for k in range(nsteps):
        istep = nit000 + k
        args = m.step_args(istep)
        if nargs == len(REF_ARGTYPES):
            del args[31]  # the reference's serial signature has no height
        step_fn(*args)
        if every and (k + 1) % every == 0 and checksums is not None:
            checksums.append(model_checksums(m))
    return m


def regions(m):
    """Checksum regions (0-based inclusive x0, x1, y0, y1) per field kind:
    the loop ranges the PSy layer updates (time_step.cpp:53-77)."""
    return Model.regions(m)


def model_checksums(m, oracle=None):
    lib = oracle or load_oracle()
    r = regions(m)
    out = {}
    for name, kind in (("sshn_t", "t"), ("un", "u"), ("vn", "v"),
                       ("ua", "u"), ("va", "v")):
        x0, x1, y0, y1 = r[kind]
        out[name] = lib.oracle_field_checksum(dptr(m.f[name]), m.width, x0,
                                              x1, y0, y1)
    return out


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.sqrt(np.sum(b * b))
    num = np.sqrt(np.sum((a - b) ** 2))
    return num / den if den > 0 else num


# ---- GPU side (the product, through its C-ABI) ----------------------------

def gpu_lib():
    import psyclonebench_gb300 as P
    return P.load_library()


def gpu_check(lib, what):
    import psyclonebench_gb300 as P
    P.check(None, what)


def gpu_read_all(lib, m):
    """Pulls all 13 fields back into m's host arrays (c_read_from_device)."""
    from psyclonebench_gb300.model import read_fields
    return read_fields(lib, m)


def gpu_run_calls(lib, m, nsteps, nit000=1, mode=0):
    """nsteps calls of c_invoke_time_step (the reference-facing path), then a
    read-back of every field.  Returns the list of paths the steps took."""
    lib.nl2d_set_mode(mode)
    paths = []
    for k in range(nsteps):
        lib.c_invoke_time_step(*m.step_args(nit000 + k))
        paths.append(lib.nl2d_last_path())
    gpu_check(lib, "c_invoke_time_step")
    gpu_read_all(lib, m)
    lib.nl2d_set_mode(0)
    return paths


def gpu_register(lib, m):
    from psyclonebench_gb300.model import register
    register(lib, m)


def gpu_run_graph(lib, m, nsteps, nit000=1, every=0):
    """Registers m and advances it with nl2d_run_steps (graph path)."""
    gpu_register(lib, m)
    nsums = nsteps // every if every else 0
    out = np.zeros(max(3 * nsums, 3), np.float64)
    import psyclonebench_gb300 as P
    P.check(lib.nl2d_run_steps(nit000, nsteps, every, dptr(out)), "nl2d_run_steps")
    gpu_read_all(lib, m)
    return out[:3 * nsums].reshape(-1, 3)


def ensemble_oracle_run(dom, nsteps, rdt=None, oracle=None, every=0, cbfr=None, visc=None):
    """Runs one ensemble domain (a build_domain() dict, at rest) through the
    oracle with its tide; returns (model, checksums list)."""
    lib = oracle or load_oracle()
    fn = lib.oracle_invoke_time_step_tide
    m = Model.from_extents(*dom["dims"]).uniform_metrics()
    m.grid["tmask"][:] = np.ascontiguousarray(dom["tmask"], np.int32)
    m.f["ht"][:], m.f["hu"][:], m.f["hv"][:] = dom["ht"], dom["hu"], dom["hv"]
    from psyclonebench_gb300 import workloads as W
    m.rdt = W.ENSEMBLE_RDT if rdt is None else rdt
    m.cbfr = W.ENSEMBLE_CBFR if cbfr is None else cbfr
    m.visc = W.ENSEMBLE_VISC if visc is None else visc
    amp, per = dom["tide"]
    sums = []
    for k in range(nsteps):
        fn(*(m.step_args(1 + k) + [amp, per]))
        if every and (k + 1) % every == 0:
            sums.append(model_checksums(m, lib))
    return m, sums


def pin_model(lib, m, page=4096):
    """Moves every array of m into page-aligned buffers of its own and pins
    them (nl2d_host_register); returns what unpin_model releases."""
    import psyclonebench_gb300 as P
    held = []
    for d in (m.f, m.grid):
        for k, a in list(d.items()):
            nb = -(-a.nbytes // page) * page
            raw = np.empty(nb + page, np.uint8)
            off = (-raw.ctypes.data) % page
            b = raw[off:off + a.nbytes].view(a.dtype).reshape(a.shape)
            b[...] = a
            d[k] = b
            P.check(lib.nl2d_host_register(b.ctypes.data, b.nbytes), "host register")
            held.append(b)
    return held


def unpin_model(lib, held):
    for b in held:
        lib.nl2d_host_unregister(b.ctypes.data)
