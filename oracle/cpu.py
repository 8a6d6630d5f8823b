"""Python loaders of the CPU oracle — TEST INFRASTRUCTURE ONLY.

Only the tests, ``__graft_entry__.smoke()`` and bench.py's CPU legs (the
``cpu_baseline`` and the ``--impl reference`` arm) import this module, and
only as what the tests compare with or as the timed CPU baseline.  The GPU product never
imports, links or calls anything under ``oracle/``.

It loads:
  * ``_build/libnl2d_oracle.so``: this repo's C restatements of the
    NEMOLite2D step (serial, the OpenMP worksharing of time_step_omp.cpp,
    the partial fusion of time_step_ompopt.cpp, a tide-parametrised step) and
    of the tracer-advection iteration, plus the driver pieces (namelist,
    T-mask, checksum);
  * ``_ref/libnl2d_ref_{serial,omp,ompopt}.so``: the reference's own PSy
    layers compiled unchanged from its sources, where the reference checkout
    was present when the oracle was built (never on a machine without it).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libnl2d_oracle.so")
REF_DIR = os.path.join(HERE, "_ref")

_DP = ctypes.POINTER(ctypes.c_double)
_IP = ctypes.POINTER(ctypes.c_int)
STEP_ARGTYPES = ([_DP] * 13 + [_IP] + [_DP] * 11 + [ctypes.c_int] * 7 +
                 [ctypes.c_double] * 6)
# the reference's serial signature has no `height` (psykal_cpp/time_step.cpp:10-51)
REF_ARGTYPES = ([_DP] * 13 + [_IP] + [_DP] * 11 + [ctypes.c_int] * 6 +
                [ctypes.c_double] * 6)

_oracle = None


def build_oracle():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def load_oracle():
    """The restatement library (built on first use)."""
    global _oracle
    if _oracle is not None:
        return _oracle
    if not os.path.exists(ORACLE_SO):
        build_oracle()
    lib = ctypes.CDLL(ORACLE_SO)
    for name in ("oracle_invoke_time_step", "oracle_invoke_time_step_omp",
                 "oracle_invoke_time_step_ompopt"):
        fn = getattr(lib, name)
        fn.argtypes = STEP_ARGTYPES
        fn.restype = None
    lib.oracle_invoke_time_step_tide.argtypes = STEP_ARGTYPES + [ctypes.c_double] * 2
    lib.oracle_invoke_time_step_tide.restype = None
    lib.oracle_field_checksum.argtypes = [_DP] + [ctypes.c_int] * 5
    lib.oracle_field_checksum.restype = ctypes.c_double
    lib.oracle_setup_tmask.argtypes = [ctypes.c_int] * 7 + [_IP]
    lib.oracle_setup_tmask.restype = ctypes.c_int
    lib.oracle_read_namelist.argtypes = [ctypes.c_char_p, _IP, _DP]
    lib.oracle_read_namelist.restype = ctypes.c_int
    for name in ("tra_oracle_step", "tra_oracle_step_omp"):
        fn = getattr(lib, name)
        fn.argtypes = [ctypes.c_int] * 3 + [_DP] * 17
        fn.restype = None
    lib.tra_oracle_init.argtypes = [ctypes.c_int] * 3 + [_DP] * 12
    lib.tra_oracle_init.restype = None
    lib.tra_oracle_checksum.argtypes = [ctypes.c_int] * 3 + [_DP]
    lib.tra_oracle_checksum.restype = ctypes.c_double
    _oracle = lib
    return lib


def load_ref(kind="serial"):
    """The reference's own c_invoke_time_step compiled from its sources
    (kind: serial, omp or ompopt), or None where it was not built."""
    path = os.path.join(REF_DIR, "libnl2d_ref_%s.so" % kind)
    if not os.path.exists(path):
        return None
    lib = ctypes.CDLL(path, mode=ctypes.RTLD_LOCAL)
    lib.c_invoke_time_step.argtypes = REF_ARGTYPES
    lib.c_invoke_time_step.restype = None
    return lib


def setup_model(m, jphgr_msh=1, dx=1000.0, dy=1000.0, dep_const=100.0, lib=None):
    """Fills a model (psyclonebench_gb300.model.Model or any object with the
    same arrays and extents) with the reference's start state through the
    oracle's restatement: setup_tpoints_mask (common/model_mod.f90:94-249),
    the uniform metrics of original/nemolite2d.f90:218-290 and the rest
    state of initialisation_mod.f90:7-63."""
    lib = lib or load_oracle()
    rc = lib.oracle_setup_tmask(jphgr_msh, m.width, m.height, m.xs, m.xe, m.ys, m.ye,
                                m.grid["tmask"].ctypes.data_as(_IP))
    assert rc == 0
    g = m.grid
    for k in ("dx_u", "dx_v", "dx_t"):
        g[k][:] = dx
    for k in ("dy_u", "dy_v", "dy_t"):
        g[k][:] = dy
    for k in ("area_t", "area_u", "area_v"):
        g[k][:] = dx * dy
    g["gphiu"][:] = 50.0
    g["gphiv"][:] = 50.0
    for k in ("ht", "hu", "hv"):
        m.f[k][:] = dep_const
    return m


def cpu_step_fns():
    """The CPU forms of the step that a baseline may time, fastest first
    unknown: [(callable, kind, description)] with the reference's own OpenMP
    PSy layers where oracle/_ref holds them, else the oracle's ports of the
    same two layers."""
    out = []
    for kind, src in (("omp", "time_step_omp.cpp"), ("ompopt", "time_step_ompopt.cpp")):
        ref = load_ref(kind)
        if ref is not None:
            out.append((ref.c_invoke_time_step, "reference",
                        "psykal_cpp/%s (-O3 -fopenmp)" % src))
    if out:
        return out
    o = load_oracle()
    return [(o.oracle_invoke_time_step_omp, "port", "oracle OpenMP port of time_step_omp.cpp"),
            (o.oracle_invoke_time_step_ompopt, "port",
             "oracle OpenMP port of time_step_ompopt.cpp (partially fused)")]


def call_step(fn, args):
    """Calls a step function with a 7-int argument list, dropping `height`
    for the reference's 6-int serial signature."""
    if len(fn.argtypes) == len(REF_ARGTYPES):
        args = list(args)
        del args[31]
    fn(*args)


# ---- tracer advection ------------------------------------------------------

TRA_WORK = ("zwx", "zwy", "zslpx", "zslpy", "zind")


def tra_zero_work(shape):
    return {n: np.zeros(shape) for n in TRA_WORK}


def tra_oracle_run(lib, f, w, niter, omp=False):
    """Advances f (mydomain in place) and the work arrays w by niter oracle
    iterations of tra_adv.F90's loop body."""
    K, J, I = f["mydomain"].shape
    fn = lib.tra_oracle_step_omp if omp else lib.tra_oracle_step
    p = [f[n].ctypes.data_as(_DP) for n in ("mydomain", "tsn", "pun", "pvn", "pwn", "umask",
                                             "vmask", "tmask", "ztfreez", "rnfmsk", "upsmsk",
                                             "rnfmsk_z")]
    p += [w[n].ctypes.data_as(_DP) for n in TRA_WORK]
    for _ in range(niter):
        fn(I, J, K, *p)
