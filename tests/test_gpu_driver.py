"""The nemolite2d_gb300 executable (the reference executable's driver
around this library's time step) against the oracle: its tmask and go2d
output files are byte-identical to the files written from the oracle's
fields, and its printed ua / va checksums are the oracle's."""
import os
import subprocess

import numpy as np
import pytest

import nl2d_testlib as T

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXE = os.path.join(REPO, "psyclonebench_gb300", "_lib", "nemolite2d_gb300")


def _fmt(lib, v, d):
    import ctypes
    buf = ctypes.create_string_buffer(64)
    assert lib.nl2d_format_e(v, 16, d, buf, 64) == 0
    return buf.value.decode()


@pytest.mark.parametrize("jphgr,jpiglo,jpjglo,nitend,irecord", [
    (1, 66, 50, 60, 30),     # the reference configuration's open south side
    (3, 41, 37, 45, 15),     # open south and east sides (Flather on both)
])
def test_driver_outputs_match_the_oracle(gpulib, oracle, tmp_path, jphgr, jpiglo, jpjglo,
                                         nitend, irecord):
    assert os.path.exists(EXE), "build the library first (__graft_entry__.build())"
    run_dir = tmp_path / "gpu"
    run_dir.mkdir()
    (run_dir / "namelist").write_text(
        "&namctl\n jpiglo = %d, jpjglo = %d, jphgr_msh = %d,\n"
        " dx = 1000.0, dy = 1000.0, dep_const = 100.0,\n"
        " nit000 = 1, nitend = %d, irecord = %d,\n"
        " rdt = 20.0d0, cbfr = 1.5d-4, visc = 0.1\n/\n" % (jpiglo, jpjglo, jphgr, nitend,
                                                           irecord))
    r = subprocess.run([EXE], cwd=run_dir, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Simulation finished!!" in r.stdout

    # the same run on the oracle, written with the library's writers
    exp_dir = tmp_path / "oracle"
    exp_dir.mkdir()
    m = T.make_model(jpiglo, jpjglo, jphgr, oracle=oracle)
    xt = np.zeros((m.height, m.width))
    yt = np.zeros((m.height, m.width))
    xt[:] = (np.arange(m.width) - m.xs) * 1000.0 + 500.0
    yt[:] = ((np.arange(m.height) - m.ys) * 1000.0 + 500.0)[:, None]
    d = str(exp_dir).encode()
    assert gpulib.nl2d_dump_tmask(d, 0, 1, m.width, jpiglo, jpjglo, T.iptr(m.grid["tmask"]),
                                  m.xs, m.xe, m.ys, m.ye, T.dptr(xt), T.dptr(yt)) == 0

    def write(istp):
        assert gpulib.nl2d_model_write(d, istp, 0, m.width, m.xs, m.xe, m.ys, m.ye,
                                       T.dptr(xt), T.dptr(yt), T.dptr(m.f["ht"]),
                                       T.dptr(m.f["sshn_t"]), T.dptr(m.f["un"]),
                                       T.dptr(m.f["vn"])) == 0

    write(0)
    for istp in range(1, nitend + 1):
        T.run(oracle.oracle_invoke_time_step, m, 1, nit000=istp)
        if istp % irecord == 0:
            write(istp)
    names = sorted(os.listdir(exp_dir))
    assert names == sorted(n for n in os.listdir(run_dir) if n != "namelist")
    assert len(names) == 2 + nitend // irecord
    for n in names:
        assert (run_dir / n).read_bytes() == (exp_dir / n).read_bytes(), n
    sums = T.model_checksums(m, oracle)
    assert "ua checksum = %s" % _fmt(gpulib, sums["ua"], 8) in r.stdout
    assert "va checksum = %s" % _fmt(gpulib, sums["va"], 8) in r.stdout


def test_driver_reports_namelist_errors(tmp_path):
    (tmp_path / "namelist").write_text("&namctl jpiglo = 34, colour = 3 /\n")
    r = subprocess.run([EXE], cwd=tmp_path, capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "err found in reading namelist file" in r.stderr
    (tmp_path / "namelist").write_text("&namctl jphgr_msh = 0 /\n")
    r = subprocess.run([EXE], cwd=tmp_path, capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "tmask_in.dat: file not found" in r.stderr


def test_driver_reads_a_coastline_grid(gpulib, oracle, tmp_path):
    """jphgr_msh = 0: a T mask with an island, a peninsula and a ragged
    north coast (open south side) from tmask_in.dat and variable depths
    from depth_in.dat.  The executable's output files equal the oracle's
    run on the same grid, byte for byte."""
    jpiglo, jpjglo, nitend, irecord = 48, 40, 40, 20
    m = T.make_model(jpiglo, jpjglo, 1, oracle=oracle)
    tm = m.grid["tmask"]
    tm[15:20, 20:26] = 0          # island
    tm[30, 1:11] = 0              # peninsula from the west coast
    for i in range(1, jpiglo - 1):  # ragged north coast
        tm[jpjglo - 2 - (i % 3 == 0), i] = 0 if i % 3 == 0 else tm[jpjglo - 2, i]
    rng = np.random.default_rng(4)
    ht = 100.0 + 40.0 * np.sin(np.arange(jpiglo) / 5.0)[None, :] * \
        np.cos(np.arange(jpjglo) / 7.0)[:, None] + rng.uniform(0, 5, size=(jpjglo, jpiglo))
    run_dir = tmp_path / "gpu"
    run_dir.mkdir()
    (run_dir / "namelist").write_text(
        "&namctl jpiglo = %d, jpjglo = %d, jphgr_msh = 0, nitend = %d, irecord = %d,\n"
        " rdt = 20.0, cbfr = 1.5d-4, visc = 0.1, dep_const = 100.0 /\n" % (
            jpiglo, jpjglo, nitend, irecord))
    (run_dir / "tmask_in.dat").write_text("".join(
        "%d %d %d\n" % (i + 1, j + 1, tm[j, i]) for j in range(jpjglo) for i in range(jpiglo)))
    (run_dir / "depth_in.dat").write_text("".join(
        "%d %d %.17g\n" % (i + 1, j + 1, ht[j, i]) for j in range(jpjglo)
        for i in range(jpiglo)))
    r = subprocess.run([EXE], cwd=run_dir, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr

    # the oracle on the same grid: mask past jpiglo x jpjglo is land, depths
    # extended by the last column / row, face depths the plain averages
    tm[:, jpiglo:] = 0
    tm[jpjglo:, :] = 0
    full = np.zeros((m.height, m.width))
    full[:jpjglo, :jpiglo] = ht
    full[:jpjglo, jpiglo:] = ht[:, -1:]
    full[jpjglo:, :] = full[jpjglo - 1:jpjglo, :]
    m.f["ht"][:] = full
    m.f["hu"][:, :-1] = 0.5 * (full[:, :-1] + full[:, 1:])
    m.f["hu"][:, -1] = full[:, -1]
    m.f["hv"][:-1] = 0.5 * (full[:-1] + full[1:])
    m.f["hv"][-1] = full[-1]
    exp_dir = tmp_path / "oracle"
    exp_dir.mkdir()
    xt = np.zeros((m.height, m.width))
    yt = np.zeros((m.height, m.width))
    xt[:] = (np.arange(m.width) - m.xs) * 1000.0 + 500.0
    yt[:] = ((np.arange(m.height) - m.ys) * 1000.0 + 500.0)[:, None]
    d = str(exp_dir).encode()

    def write(istp):
        assert gpulib.nl2d_model_write(d, istp, 0, m.width, m.xs, m.xe, m.ys, m.ye,
                                       T.dptr(xt), T.dptr(yt), T.dptr(m.f["ht"]),
                                       T.dptr(m.f["sshn_t"]), T.dptr(m.f["un"]),
                                       T.dptr(m.f["vn"])) == 0

    write(0)
    for istp in range(1, nitend + 1):
        T.run(oracle.oracle_invoke_time_step, m, 1, nit000=istp)
        if istp % irecord == 0:
            write(istp)
    for n in sorted(os.listdir(exp_dir)):
        assert (run_dir / n).read_bytes() == (exp_dir / n).read_bytes(), n
    assert np.abs(m.f["sshn_t"]).max() > 0  # the tide has entered the basin
    sums = T.model_checksums(m, oracle)
    assert "ua checksum = %s" % _fmt(gpulib, sums["ua"], 8) in r.stdout
