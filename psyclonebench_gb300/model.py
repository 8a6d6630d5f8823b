"""Host-side model of one NEMOLite2D domain as the reference's driver holds
it: dl_esm_inf-style r2d fields and grid arrays (row-major [height][width]
FP64, the T-mask int32), the 0-based internal bounds, and the argument list
of ``c_invoke_time_step`` built from them.

This is what a caller of the library owns; the library itself only ever sees
the arrays' addresses through its C-ABI.  The set-up here is the library's
own (``nl2d_setup_model``: setup_tpoints_mask, grid metrics and the initial
state of common/model_mod.f90:26-249, initialisation_mod.f90:7-63).
"""
import ctypes

import numpy as np

from . import check, load_library

# physical_params_mod.f90:9-15 of the reference
PI = 3.1415926535897932
G = 9.80665
OMEGA = 7.292116e-05
D2R = PI / 180.0

# c_invoke_time_step's array arguments, in order (psykal_cpp/time_step.cpp:10-37)
FIELDS = ("ssha_t", "sshn_t", "sshn_u", "sshn_v", "hu", "hv", "un", "vn",
          "ua", "ht", "ssha_u", "va", "ssha_v")
GRID = ("tmask", "area_t", "area_u", "area_v", "dx_u", "dx_v", "dx_t",
        "dy_u", "dy_v", "dy_t", "gphiu", "gphiv")

_DP = ctypes.POINTER(ctypes.c_double)
_IP = ctypes.POINTER(ctypes.c_int)


def dptr(a):
    return a.ctypes.data_as(_DP)


def iptr(a):
    return a.ctypes.data_as(_IP)


class Model:
    """A single-rank model: 13 fields, 12 grid arrays, internal T cells
    [xs, xe] x [ys, ye] (0-based; the outermost ring of the jpiglo x jpjglo
    mask is boundary, model_mod.f90:144-239), physics scalars."""

    def __init__(self, jpiglo, jpjglo, width=None, height=None):
        self.jpiglo, self.jpjglo = jpiglo, jpjglo
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

    @classmethod
    def from_extents(cls, width, height, xs, xe, ys, ye):
        """An empty model with explicit array and internal extents."""
        m = cls.__new__(cls)
        m.jpiglo, m.jpjglo = xe + 2, ye + 2
        m.xs, m.xe, m.ys, m.ye, m.width, m.height = xs, xe, ys, ye, width, height
        shp = (height, width)
        m.f = {k: np.zeros(shp, np.float64) for k in FIELDS}
        m.grid = {k: np.zeros(shp, np.float64) for k in GRID if k != "tmask"}
        m.grid["tmask"] = np.zeros(shp, np.int32)
        m.rdt, m.cbfr, m.visc = 20.0, 1.5e-4, 0.1
        return m

    def copy(self):
        m = Model.__new__(Model)
        m.__dict__.update(self.__dict__)
        m.f = {k: v.copy() for k, v in self.f.items()}
        m.grid = {k: v.copy() for k, v in self.grid.items()}
        return m

    def uniform_metrics(self, dx=1000.0, dy=1000.0, lat=50.0):
        """dx / dy / area and latitude as the reference's set-up writes them
        for a uniform grid (original/nemolite2d.f90:218-290)."""
        g = self.grid
        for k in ("dx_u", "dx_v", "dx_t"):
            g[k][:] = dx
        for k in ("dy_u", "dy_v", "dy_t"):
            g[k][:] = dy
        for k in ("area_t", "area_u", "area_v"):
            g[k][:] = dx * dy
        g["gphiu"][:] = lat
        g["gphiv"][:] = lat
        return self

    def step_args(self, istep):
        """c_invoke_time_step's arguments (the 7-int form, with height)."""
        f, g = self.f, self.grid
        # time_step_mod.f90:65-79: dy_v and dy_t slots receive dx_v and dx_t.
        return ([dptr(f[k]) for k in FIELDS] + [iptr(g["tmask"])] +
                [dptr(g[k]) for k in ("area_t", "area_u", "area_v", "dx_u",
                                       "dx_v", "dx_t", "dy_u")] +
                [dptr(g["dx_v"]), dptr(g["dx_t"])] +
                [dptr(g["gphiu"]), dptr(g["gphiv"])] +
                [istep, self.xs, self.xe, self.ys, self.ye, self.width,
                 self.height, self.rdt, self.cbfr, self.visc, OMEGA, D2R, G])

    def regions(self):
        """Checksum regions (0-based inclusive x0, x1, y0, y1) per field
        kind: the loop ranges the PSy layer updates (time_step.cpp:53-77)."""
        return {
            "t": (self.xs, self.xe, self.ys, self.ye),
            "u": (self.xs, self.xe - 1, self.ys, self.ye),
            "v": (self.xs, self.xe, self.ys, self.ye - 1),
        }


def setup_model(m, jphgr_msh=1, dx=1000.0, dy=1000.0, dep_const=100.0, lib=None):
    """Fills m with the reference's start state through the library's own
    set-up (nl2d_setup_model)."""
    lib = lib or load_library()
    fp = (_DP * 13)(*[dptr(m.f[k]) for k in FIELDS])
    gp = (_DP * 11)(*[dptr(m.grid[k]) for k in GRID[1:]])
    check(lib.nl2d_setup_model(jphgr_msh, m.jpiglo, m.jpjglo, dx, dy, dep_const, m.width,
                               m.height, fp, iptr(m.grid["tmask"]), gp, None, None),
          "nl2d_setup_model")
    return m


def reference_problem(n, written=False, lib=None):
    """The reference's initial state for an n x n interior (namelist jpiglo
    = jpjglo = n + 2, jphgr_msh = 1, dx = dy = 1000 m, depth 100 m), rows
    padded to a multiple of 8 doubles.

    written: every array written once more, as the reference's driver writes
    them during set-up (the grid and field constructors); numpy's zero-filled
    arrays are otherwise untouched pages, which the first host-to-device copy
    would have to fault in."""
    jp = n + 2
    width = ((jp + 1 + 7) // 8) * 8
    m = setup_model(Model(jp, jp, width=width), lib=lib)
    if written:
        for a in list(m.f.values()) + list(m.grid.values()):
            a[...] = a.copy()
    return m


def register(lib, m):
    """Uploads m's 25 arrays and makes them the resident problem
    (nl2d_register: c_invoke_time_step's argument list without istep)."""
    args = m.step_args(0)
    del args[25]
    check(lib.nl2d_register(*args), "nl2d_register")


def read_fields(lib, m, names=FIELDS):
    """Copies the device state of the named fields into m's host arrays
    (c_read_from_device, as dl_esm_inf's get_data() would)."""
    for k in names:
        a = m.f[k]
        lib.c_read_from_device(a.ctypes.data, a.ctypes.data, 1, 1, m.width, m.height, True)
    check(None, "c_read_from_device")
    return m
