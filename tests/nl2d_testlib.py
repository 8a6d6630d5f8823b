"""Shared helpers for the NEMOLite2D tests: loading the CPU oracle (and, when
it was built here, the reference's own compiled PSy layer), building
dl_esm_inf-style models as numpy arrays, and stepping them.

The oracle is only ever the checker here; the GPU library is the thing under
test.
"""
import ctypes
import os
import subprocess

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(REPO, "oracle")
ORACLE_SO = os.path.join(ORACLE_DIR, "_build", "libnl2d_oracle.so")
REF_DIR = os.path.join(ORACLE_DIR, "_ref")

# physical_params_mod.f90:9-15 of the reference
PI = 3.1415926535897932
G = 9.80665
OMEGA = 7.292116e-05
D2R = PI / 180.0

FIELDS = ("ssha_t", "sshn_t", "sshn_u", "sshn_v", "hu", "hv", "un", "vn",
          "ua", "ht", "ssha_u", "va", "ssha_v")
GRID = ("tmask", "area_t", "area_u", "area_v", "dx_u", "dx_v", "dx_t",
        "dy_u", "dy_v", "dy_t", "gphiu", "gphiv")
STATE = ("sshn_t", "un", "vn", "ua", "va", "ssha_t", "sshn_u", "sshn_v")

_DP = ctypes.POINTER(ctypes.c_double)
_IP = ctypes.POINTER(ctypes.c_int)
STEP_ARGTYPES = ([_DP] * 13 + [_IP] + [_DP] * 11 + [ctypes.c_int] * 7 +
                 [ctypes.c_double] * 6)
REF_ARGTYPES = ([_DP] * 13 + [_IP] + [_DP] * 11 + [ctypes.c_int] * 6 +
                [ctypes.c_double] * 6)


def build_oracle():
    subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True)


def load_oracle():
    if not os.path.exists(ORACLE_SO):
        build_oracle()
    lib = ctypes.CDLL(ORACLE_SO)
    for name in ("oracle_invoke_time_step", "oracle_invoke_time_step_omp"):
        fn = getattr(lib, name)
        fn.argtypes = STEP_ARGTYPES
        fn.restype = None
    lib.oracle_field_checksum.argtypes = [_DP] + [ctypes.c_int] * 5
    lib.oracle_field_checksum.restype = ctypes.c_double
    lib.oracle_setup_tmask.argtypes = [ctypes.c_int] * 7 + [_IP]
    lib.oracle_setup_tmask.restype = ctypes.c_int
    lib.oracle_read_namelist.argtypes = [ctypes.c_char_p, _IP, _DP]
    lib.oracle_read_namelist.restype = ctypes.c_int
    return lib


def load_ref(kind="serial"):
    """The reference's own c_invoke_time_step compiled from its sources
    (oracle/Makefile `ref`), or None where it was not built."""
    path = os.path.join(REF_DIR, "libnl2d_ref_%s.so" % kind)
    if not os.path.exists(path):
        return None
    lib = ctypes.CDLL(path, mode=ctypes.RTLD_LOCAL)
    lib.c_invoke_time_step.argtypes = REF_ARGTYPES
    lib.c_invoke_time_step.restype = None
    return lib


def dptr(a):
    return a.ctypes.data_as(_DP)


def iptr(a):
    return a.ctypes.data_as(_IP)


class Model:
    """A dl_esm_inf-style single-rank model: row-major [height][width] FP64
    fields, an int32 T-mask, metric arrays and the 0-based internal bounds."""

    def __init__(self, jpiglo, jpjglo, width=None, height=None):
        self.jpiglo, self.jpjglo = jpiglo, jpjglo
        # Internal T cells are 1..jpiglo-2 (0-based): the outermost ring of
        # the jpiglo x jpjglo mask is boundary (model_mod.f90:144-239).
        self.xs, self.xe = 1, jpiglo - 2
        self.ys, self.ye = 1, jpjglo - 2
        # Fields are one larger than the mask in each direction for the NE
        # stagger, optionally padded.
        self.width = width if width is not None else jpiglo + 1
        self.height = height if height is not None else jpjglo + 1
        assert self.width >= jpiglo and self.height >= jpjglo
        shp = (self.height, self.width)
        self.f = {k: np.zeros(shp, np.float64) for k in FIELDS}
        self.grid = {k: np.zeros(shp, np.float64) for k in GRID if k != "tmask"}
        self.grid["tmask"] = np.zeros(shp, np.int32)
        self.rdt, self.cbfr, self.visc = 20.0, 1.5e-4, 0.1

    def copy(self):
        m = Model.__new__(Model)
        m.__dict__.update(self.__dict__)
        m.f = {k: v.copy() for k, v in self.f.items()}
        m.grid = {k: v.copy() for k, v in self.grid.items()}
        return m

    def step_args(self, istep):
        f, g = self.f, self.grid
        # time_step_mod.f90:65-79: dy_v and dy_t slots receive dx_v and dx_t.
        return ([dptr(f[k]) for k in FIELDS] + [iptr(g["tmask"])] +
                [dptr(g[k]) for k in ("area_t", "area_u", "area_v", "dx_u",
                                       "dx_v", "dx_t", "dy_u")] +
                [dptr(g["dx_v"]), dptr(g["dx_t"])] +
                [dptr(g["gphiu"]), dptr(g["gphiv"])] +
                [istep, self.xs, self.xe, self.ys, self.ye, self.width,
                 self.height, self.rdt, self.cbfr, self.visc, OMEGA, D2R, G])


def make_model(jpiglo=130, jpjglo=130, jphgr_msh=1, dx=1000.0, dy=1000.0,
               dep_const=100.0, width=None, height=None, oracle=None):
    """The reference's start state: model_init + initialisation
    (model_mod.f90:26-69, initialisation_mod.f90:7-63)."""
    m = Model(jpiglo, jpjglo, width, height)
    lib = oracle or load_oracle()
    rc = lib.oracle_setup_tmask(jphgr_msh, m.width, m.height, m.xs, m.xe,
                                m.ys, m.ye, iptr(m.grid["tmask"]))
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
    return {
        "t": (m.xs, m.xe, m.ys, m.ye),
        "u": (m.xs, m.xe - 1, m.ys, m.ye),
        "v": (m.xs, m.xe, m.ys, m.ye - 1),
    }


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
    for k in FIELDS:
        a = m.f[k]
        lib.c_read_from_device(a.ctypes.data, a.ctypes.data, 1, 1, m.width, m.height, True)
    gpu_check(lib, "c_read_from_device")
    return m


def gpu_run_calls(lib, m, nsteps, nit000=1, mode=0):
    """nsteps calls of c_invoke_time_step (the reference-facing path), then a
    read-back of every field.  Returns the list of paths the steps took."""
    import ctypes as C
    lib.nl2d_set_mode(mode)
    paths = []
    for k in range(nsteps):
        lib.c_invoke_time_step(*m.step_args(nit000 + k))
        paths.append(lib.nl2d_last_path())
    gpu_check(lib, "c_invoke_time_step")
    gpu_read_all(lib, m)
    lib.nl2d_set_mode(0)
    del C
    return paths


def gpu_register(lib, m):
    args = m.step_args(0)
    del args[25]  # nl2d_register takes no istep
    import psyclonebench_gb300 as P
    P.check(lib.nl2d_register(*args), "nl2d_register")


def gpu_run_graph(lib, m, nsteps, nit000=1, every=0):
    """Registers m and advances it with nl2d_run_steps (graph path)."""
    gpu_register(lib, m)
    nsums = nsteps // every if every else 0
    out = np.zeros(max(3 * nsums, 3), np.float64)
    import psyclonebench_gb300 as P
    P.check(lib.nl2d_run_steps(nit000, nsteps, every, dptr(out)), "nl2d_run_steps")
    gpu_read_all(lib, m)
    return out[:3 * nsums].reshape(-1, 3)


def ensemble_oracle_run(dom, nsteps, rdt=5.0, oracle=None, every=0):
    """Runs one ensemble domain (a build_domain() dict, at rest) through the
    oracle with its tide; returns (model, checksums list)."""
    import ctypes as C
    lib = oracle or load_oracle()
    fn = lib.oracle_invoke_time_step_tide
    fn.argtypes = STEP_ARGTYPES + [C.c_double, C.c_double]
    fn.restype = None
    w, h, xs, xe, ys, ye = dom["dims"]
    m = Model.__new__(Model)
    m.jpiglo, m.jpjglo = xe + 2, ye + 2
    m.xs, m.xe, m.ys, m.ye, m.width, m.height = xs, xe, ys, ye, w, h
    shp = (h, w)
    m.f = {k: np.zeros(shp, np.float64) for k in FIELDS}
    m.grid = {k: np.zeros(shp, np.float64) for k in GRID if k != "tmask"}
    m.grid["tmask"] = np.ascontiguousarray(dom["tmask"], np.int32).copy()
    for k in ("dx_u", "dx_v", "dx_t", "dy_u", "dy_v", "dy_t"):
        m.grid[k][:] = 1000.0
    for k in ("area_t", "area_u", "area_v"):
        m.grid[k][:] = 1.0e6
    m.grid["gphiu"][:] = 50.0
    m.grid["gphiv"][:] = 50.0
    m.f["ht"][:], m.f["hu"][:], m.f["hv"][:] = dom["ht"], dom["hu"], dom["hv"]
    m.rdt, m.cbfr, m.visc = rdt, 1.5e-4, 0.1
    amp, per = dom["tide"]
    sums = []
    for k in range(nsteps):
        fn(*(m.step_args(1 + k) + [amp, per]))
        if every and (k + 1) % every == 0:
            sums.append(model_checksums(m, lib))
    return m, sums
