"""Host side of the reference executable (no GPU): the &namctl reader, the
single-rank set-up, and the go2d / tmask writers in the Fortran edit
descriptors the reference uses (common/gocean2d_io_mod.f90,
common/model_mod.f90)."""
import ctypes
import math
import os

import numpy as np
import pytest

from nl2d_testlib import FIELDS, GRID, dptr, iptr, make_model

NAMELISTS = {
    "config0": """&namctl
 jpiglo = 130, jpjglo = 130, jphgr_msh = 1,
 dx = 1000.0, dy = 1000.0, dep_const = 100.0,
 nit000 = 1, nitend = 2000, irecord = 2500,
 rdt = 20.0, cbfr = 0.00015, visc = 0.1
/
""",
    "fortran_literals": """! leading comment
&NAMCTL JPIGLO=66 JPJGLO=50   ! trailing comment
  jphgr_msh=3,dx=5.0D2,dy=2.5d+2 dep_const=1.e2
  nitend = 7, rdt = .5D1 /
""",
    "defaults": "&namctl /\n",
    "other_group_first": "&other a = 1 /\n&namctl visc = 7.25 , irecord = 3 /\n",
}


def _lib():
    import psyclonebench_gb300 as P
    return P.load_library()


def _read(lib, path):
    iv = (ctypes.c_int * 6)()
    dv = (ctypes.c_double * 6)()
    rc = lib.nl2d_read_namelist(str(path).encode(), iv, dv)
    return rc, list(iv), list(dv)


@pytest.mark.parametrize("name", sorted(NAMELISTS))
def test_namelist_reader(tmp_path, name, oracle):
    lib = _lib()
    p = tmp_path / "namelist"
    p.write_text(NAMELISTS[name])
    rc, iv, dv = _read(lib, p)
    assert rc == 0
    expect = {
        "config0": ([130, 130, 1, 1, 2000, 2500], [1000.0, 1000.0, 100.0, 20.0, 0.00015, 0.1]),
        "fortran_literals": ([66, 50, 3, 1, 7, 1], [500.0, 250.0, 100.0, 5.0, 0.001, 100.0]),
        # gocean2d_io_mod.f90:57-68
        "defaults": ([50, 100, 1, 1, 1000, 1], [1000.0, 1000.0, 100.0, 10.0, 0.001, 100.0]),
    }.get(name)
    if expect:
        assert iv == expect[0] and dv == expect[1]
    if name != "other_group_first":
        # the oracle's reader agrees on well-formed groups
        oi = (ctypes.c_int * 6)()
        od = (ctypes.c_double * 6)()
        assert oracle.oracle_read_namelist(str(p).encode(), oi, od) == 0
        assert list(oi) == iv and list(od) == dv
    else:
        assert dv[5] == 7.25 and iv[5] == 3


@pytest.mark.parametrize("text,code", [
    ("&namctl jpiglo = 10, bogus = 3 /\n", 8),
    ("&namctl jpiglo = ten /\n", 8),
    ("&namctl jpiglo = 10\n", 8),          # never closed
    ("jpiglo = 10 /\n", 8),                # no group
    ("&namctl dx 1000 /\n", 8),
])
def test_namelist_errors(tmp_path, text, code):
    import psyclonebench_gb300 as P
    lib = _lib()
    p = tmp_path / "namelist"
    p.write_text(text)
    assert _read(lib, p)[0] == code == P.NL2D_ERR_PARSE
    assert _read(lib, tmp_path / "missing")[0] == P.NL2D_ERR_IO


def _setup(lib, jphgr, jpiglo, jpjglo, dx=1000.0, dy=1000.0, dep=100.0):
    w, h = jpiglo + 1, jpjglo + 1
    f = {k: np.full((h, w), np.nan) for k in FIELDS}
    g = {k: np.full((h, w), np.nan) for k in GRID if k != "tmask"}
    tm = np.full((h, w), 99, np.int32)
    xt, yt = np.zeros((h, w)), np.zeros((h, w))
    DPP = ctypes.POINTER(ctypes.c_double)
    fp = (DPP * 13)(*[dptr(f[k]) for k in FIELDS])
    order = ("area_t", "area_u", "area_v", "dx_u", "dx_v", "dx_t", "dy_u", "dy_v", "dy_t",
             "gphiu", "gphiv")
    gp = (DPP * 11)(*[dptr(g[k]) for k in order])
    rc = lib.nl2d_setup_model(jphgr, jpiglo, jpjglo, dx, dy, dep, w, h, fp, iptr(tm), gp,
                              dptr(xt), dptr(yt))
    return rc, f, g, tm, xt, yt


@pytest.mark.parametrize("jphgr", [1, 2, 3])
def test_setup_matches_the_reference_start_state(jphgr, oracle):
    """T mask, metrics, depths and rest state of nl2d_setup_model against
    the oracle-built model (setup_tpoints_mask + initialisation)."""
    lib = _lib()
    rc, f, g, tm, xt, yt = _setup(lib, jphgr, 34, 27, dx=900.0, dy=1100.0, dep=75.0)
    assert rc == 0
    m = make_model(34, 27, jphgr, dx=900.0, dy=1100.0, dep_const=75.0, oracle=oracle)
    np.testing.assert_array_equal(tm, m.grid["tmask"])
    for k in FIELDS:
        np.testing.assert_array_equal(f[k], m.f[k], err_msg=k)
    for k in g:
        np.testing.assert_array_equal(g[k], m.grid[k], err_msg=k)
    # T-point coordinates: dx / 2 on the first internal column, + dx onward
    assert xt[5, 1] == 450.0 and xt[5, 2] == 1350.0 and yt[1, 7] == 550.0
    assert yt[3, 0] == 550.0 + 2 * 1100.0


def test_setup_from_file_keeps_the_callers_mask(tmp_path):
    """jphgr_msh = 0 (a STOP in the reference) sets up everything but the
    mask, which comes from a grid file; a raw dump_tmask reads back."""
    import psyclonebench_gb300 as P
    lib = _lib()
    rc, f, g, tm, xt, yt = _setup(lib, 3, 20, 14)
    assert rc == 0
    tm[5:8, 6:9] = 0  # an island
    d = str(tmp_path).encode()
    assert lib.nl2d_dump_tmask(d, 0, 1, 21, 20, 14, iptr(tm), 1, 18, 1, 12, dptr(xt),
                               dptr(yt)) == 0
    back = np.full_like(tm, 42)
    assert lib.nl2d_read_grid_file(str(tmp_path / "tmask_00000.dat").encode(), 20, 14, 21, 1,
                                   back.ctypes.data) == 0
    np.testing.assert_array_equal(back[:14, :20], tm[:14, :20])
    assert (back[:, 20] == 42).all() and (back[14] == 42).all()  # outside the mask: untouched
    rc2, f2, g2, tm2, _, _ = _setup(lib, 0, 20, 14)
    assert rc2 == 0 and (tm2 == 99).all()  # the caller's mask is kept as it is
    np.testing.assert_array_equal(f2["ht"], f["ht"])
    assert _setup(lib, 4, 34, 27)[0] == P.NL2D_ERR_ARGS


@pytest.mark.parametrize("text", [
    "1 1 0\n2 1 0\n1 2 0\n",                 # a point missing
    "1 1 0\n2 1 0\n1 2 0\n1 2 1\n",         # a point twice
    "1 1 0\n2 1 0\n1 2 0\n3 2 1\n",         # out of range
    "1 1 0\n2 1 0\n1 2 0\n2 2 x\n",         # not a number
])
def test_grid_file_errors(tmp_path, text):
    import psyclonebench_gb300 as P
    lib = _lib()
    p = tmp_path / "g.dat"
    p.write_text(text)
    out = np.zeros((2, 2), np.int32)
    assert lib.nl2d_read_grid_file(str(p).encode(), 2, 2, 2, 1, out.ctypes.data) == \
        P.NL2D_ERR_PARSE
    assert lib.nl2d_read_grid_file(str(tmp_path / "none").encode(), 2, 2, 2, 1,
                                   out.ctypes.data) == P.NL2D_ERR_IO


def test_grid_file_depths_and_face_depths(tmp_path):
    lib = _lib()
    rng = np.random.default_rng(1)
    ht = rng.uniform(50, 150, size=(3, 4))
    lines = ["%d %d %.17g" % (i + 1, j + 1, ht[j, i]) for j in range(3) for i in range(4)]
    rng.shuffle(lines)
    (tmp_path / "d.dat").write_text("\n".join(lines) + "\n")
    out = np.zeros((3, 5))
    assert lib.nl2d_read_grid_file(str(tmp_path / "d.dat").encode(), 4, 3, 5, 0,
                                   out.ctypes.data) == 0
    np.testing.assert_array_equal(out[:, :4], ht)
    hu, hv = np.zeros_like(out), np.zeros_like(out)
    assert lib.nl2d_face_depths(5, 3, dptr(out), dptr(hu), dptr(hv)) == 0
    np.testing.assert_array_equal(hu[:, :4], 0.5 * (out[:, :4] + out[:, 1:]))
    np.testing.assert_array_equal(hu[:, 4], out[:, 4])
    np.testing.assert_array_equal(hv[:2], 0.5 * (out[:2] + out[1:]))
    np.testing.assert_array_equal(hv[2], out[2])


def _fmt(lib, v, w=16, d=7):
    buf = ctypes.create_string_buffer(64)
    assert lib.nl2d_format_e(v, w, d, buf, 64) == 0
    return buf.value.decode()


@pytest.mark.parametrize("v,w,d,want", [
    (1000.0, 16, 7, "   0.1000000E+04"),
    (-1.5, 16, 7, "  -0.1500000E+01"),
    (0.0, 16, 7, "   0.0000000E+00"),
    (9.999999999, 16, 7, "   0.1000000E+02"),
    (0.000123456789, 16, 7, "   0.1234568E-03"),
    (1e-300, 16, 7, "   0.1000000-299"),
    (-1.23456789e100, 16, 7, "  -0.1234568+101"),
    (1234.5678, 16, 8, "  0.12345678E+04"),
    (float("nan"), 16, 7, "             NaN"),
    (float("-inf"), 16, 7, "       -Infinity"),
    (1.0, 8, 7, "********"),
])
def test_fortran_e_layout(v, w, d, want):
    assert _fmt(_lib(), v, w, d) == want


def _py_e(v, d=7):
    """E16.d restated in Python: correctly rounded d significant digits."""
    if v == 0.0:
        return "   0.%sE+00" % ("0" * d)
    mant, exp = ("%.*e" % (d - 1, abs(v))).split("e")
    e = int(exp) + 1
    es = "E%+03d" % e if abs(e) <= 99 else "%+04d" % e
    s = ("-" if v < 0 else "") + "0." + mant.replace(".", "") + es
    return s.rjust(16)


def test_fortran_e_random_values():
    lib = _lib()
    rng = np.random.default_rng(0)
    vals = np.concatenate([rng.normal(size=300) * 10.0 ** rng.integers(-30, 30, size=300),
                           rng.normal(size=50) * 1e-3])
    for v in vals:
        assert _fmt(lib, float(v)) == _py_e(float(v)), v


def test_model_write_and_dump_tmask(tmp_path, oracle):
    lib = _lib()
    rc, f, g, tm, xt, yt = _setup(lib, 1, 12, 9)
    assert rc == 0
    rng = np.random.default_rng(3)
    for k in ("sshn_t", "un", "vn"):
        f[k][:] = rng.normal(size=f[k].shape) * 0.1
    w = 13
    xs, xe, ys, ye = 1, 10, 1, 7
    d = str(tmp_path).encode()
    assert lib.nl2d_model_write(d, 120, 3, w, xs, xe, ys, ye, dptr(xt), dptr(yt),
                                dptr(f["ht"]), dptr(f["sshn_t"]), dptr(f["un"]),
                                dptr(f["vn"])) == 0
    text = (tmp_path / "go2d_00120_00003.dat").read_text()
    lines = text.split("\n")
    assert lines[-1] == ""
    body = lines[:-1]
    assert len(body) == (ye - ys + 1) * (xe - xs + 2)
    k = 0
    for j in range(ys, ye + 1):
        for i in range(xs, xe + 1):
            ln = body[k]
            k += 1
            assert len(ln) == 96
            want = [xt[j, i], yt[j, i], f["ht"][j, i], f["sshn_t"][j, i],
                    0.5 * (f["un"][j, i - 1] + f["un"][j, i]),
                    0.5 * (f["vn"][j - 1, i] + f["vn"][j, i])]
            assert ln == "".join(_py_e(v) for v in want)
        assert body[k] == ""
        k += 1
    assert lib.nl2d_dump_tmask(d, 0, 1, w, 12, 9, iptr(tm), xs, xe, ys, ye, dptr(xt),
                               dptr(yt)) == 0
    raw = (tmp_path / "tmask_00000.dat").read_text().split("\n")
    assert raw[0] == "   1    1   -1" and raw[12] == "" and raw[13] == "   1    2    0"
    assert raw[14] == "   2    2    1"
    assert lib.nl2d_dump_tmask(d, 7, 0, w, 12, 9, iptr(tm), xs, xe, ys, ye, dptr(xt),
                               dptr(yt)) == 0
    cooked = (tmp_path / "tmask_00007.dat").read_text().split("\n")
    assert cooked[0] == _py_e(500.0) + _py_e(500.0) + "   1"
    assert lib.nl2d_model_write(os.path.join(str(tmp_path), "no", "dir").encode(), 1, 0, w,
                                xs, xe, ys, ye, dptr(xt), dptr(yt), dptr(f["ht"]),
                                dptr(f["sshn_t"]), dptr(f["un"]), dptr(f["vn"])) == 7
