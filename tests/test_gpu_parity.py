"""GPU parity: the CUDA step, called through the C-ABI, against the CPU
oracle (and the golden fixtures made by the reference's own serial build).

Bar: bit-identical FP64 fields (both sides perform the same IEEE operations
in the same order; the oracle is built with -ffp-contract=off, the kernels
with -fmad=false).  Checksums are reduced in a different order on the GPU,
so they are compared to 10 significant digits (rtol 1e-10), the bar the
reference's E16.8 print-out cannot even resolve.
"""
import os

import numpy as np
import pytest

import nl2d_testlib as T
from test_oracle import CASES, bits_equal, load_case

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CHECKSUM_RTOL = 1e-10


def assert_fields_equal(got, want, tag=""):
    bad = [k for k in T.FIELDS if not bits_equal(got.f[k], want.f[k])]
    if bad:
        k = bad[0]
        diff = np.argwhere(got.f[k].view(np.int64) != want.f[k].view(np.int64))
        raise AssertionError("%s: fields differ %s; first %s at %s: %r vs %r" % (
            tag, bad, k, diff[0], got.f[k][tuple(diff[0])], want.f[k][tuple(diff[0])]))


@pytest.mark.parametrize("mode", [1, 0], ids=["reference_path", "fused_path"])
def test_cfg0_2000_steps_bitwise(gpulib, oracle, mode):
    """130x130 namelist (128x128 interior), 2000 steps through
    c_invoke_time_step: all 13 fields bit-identical to the oracle."""
    m = T.make_model(130, 130, 1, oracle=oracle)
    want = m.copy()
    T.run(oracle.oracle_invoke_time_step, want, 2000)
    paths = T.gpu_run_calls(gpulib, m, 2000, mode=mode)
    if mode == 0:
        # the rest start is what a step leaves: every step fused, the first too
        assert set(paths) == {2}, "fused path not taken"
    else:
        assert set(paths) == {1}
    assert_fields_equal(m, want, "mode %d" % mode)


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("mode", [1, 0], ids=["reference_path", "fused_path"])
def test_golden_fields_bitwise(gpulib, name, mode):
    """The reference serial build's final fields (tests/golden, made by
    make_golden.py) on small, odd and padded grids with jphgr_msh 1, 2, 3
    and a seeded bathymetry."""
    m, nsteps, want = load_case(name)
    T.gpu_run_calls(gpulib, m, nsteps, mode=mode)
    for k in T.FIELDS:
        assert bits_equal(m.f[k], want[k]), (name, k)


def test_graph_run_checksums_cfg0(gpulib, oracle):
    """nl2d_run_steps (CUDA graph, in-graph checksums every 100 steps) over
    2000 steps: checksums within 1e-10 of the reference's, fields bitwise."""
    want_sums = np.loadtxt(os.path.join(GOLDEN, "cfg0_checksums.txt"))
    m = T.make_model(130, 130, 1, oracle=oracle)
    want = m.copy()
    T.run(oracle.oracle_invoke_time_step, want, 2000)
    sums = T.gpu_run_graph(gpulib, m, 2000, every=100)
    np.testing.assert_allclose(sums, want_sums[:, :3], rtol=CHECKSUM_RTOL, atol=0)
    assert_fields_equal(m, want, "graph")


def test_graph_rerun_and_split(gpulib, oracle):
    """Two graph runs back to back (cached graph, both ping-pong phases) equal
    one long oracle run; so does a run split by per-step calls."""
    m = T.make_model(40, 33, 3, width=48, oracle=oracle)
    want = m.copy()
    T.run(oracle.oracle_invoke_time_step, want, 3 * 37 + 5)
    T.gpu_register(gpulib, m)
    import psyclonebench_gb300 as P
    out = np.zeros(3)
    for k in range(3):
        P.check(gpulib.nl2d_run_steps(1 + 37 * k, 37, 0, T.dptr(out)), "run")
    T.gpu_read_all(gpulib, m)
    # continue with per-step calls on the same registration
    for k in range(5):
        gpulib.c_invoke_time_step(*m.step_args(1 + 111 + k))
    T.gpu_read_all(gpulib, m)
    assert_fields_equal(m, want, "graph+calls")


def test_random_masks_and_bathymetry(gpulib, oracle):
    """Random land cells, random depths, padded widths: every step path."""
    rng = np.random.default_rng(11)
    for trial in range(4):
        nx, ny = (int(v) for v in rng.integers(9, 40, size=2))
        m = T.make_model(nx, ny, int(rng.integers(1, 4)),
                         width=nx + 1 + int(rng.integers(0, 9)), oracle=oracle)
        inner = m.grid["tmask"][m.ys + 1:m.ye, m.xs + 1:m.xe]
        inner[rng.random(inner.shape) < 0.08] = 0
        for k in ("ht", "hu", "hv"):
            m.f[k][:] = rng.uniform(50, 500, size=m.f[k].shape)
        want = m.copy()
        T.run(oracle.oracle_invoke_time_step, want, 60)
        got = m.copy()
        T.gpu_run_calls(gpulib, got, 60, mode=0)
        assert_fields_equal(got, want, "trial %d" % trial)


def test_benchmark_size_bitwise(gpulib, oracle):
    """The benchmark's 4096 x 4096 interior (4098 namelist, width padded to
    4104 as the bench lays it out) with random depths and a random initial
    state, 12 steps through c_invoke_time_step (the first on the reference
    path, since a random state is not what a step leaves; the rest fused):
    all 13 fields bit-identical to the oracle's OpenMP build."""
    rng = np.random.default_rng(5)
    m = T.make_model(4098, 4098, 1, width=4104, oracle=oracle)
    for k in ("ht", "hu", "hv"):
        m.f[k][:] = rng.uniform(50.0, 500.0, size=m.f[k].shape)
    for k, a in (("sshn_t", 0.1), ("un", 0.05), ("vn", 0.05)):
        m.f[k][:] = rng.uniform(-a, a, size=m.f[k].shape)
    want = m.copy()
    T.run(oracle.oracle_invoke_time_step_omp, want, 12)
    paths = T.gpu_run_calls(gpulib, m, 12, mode=0)
    assert paths[0] == 1 and set(paths[1:]) == {2}, paths
    assert_fields_equal(m, want, "4096^2")


def test_checkpoint_resume_is_bitwise(gpulib, oracle, tmp_path):
    """A run checkpointed after 40 steps and resumed from the file by a fresh
    registration (the model rebuilt from its set-up, so its host arrays hold
    the start state) ends with every field bit-identical to the
    uninterrupted run; a file of other extents or another kind is refused."""
    import ctypes
    import psyclonebench_gb300 as P
    rng = np.random.default_rng(8)
    m = T.make_model(61, 47, 1, width=64, oracle=oracle)
    for k in ("ht", "hu", "hv"):
        m.f[k][:] = rng.uniform(50.0, 500.0, size=m.f[k].shape)
    m.rdt = 5.0
    full = m.copy()
    T.gpu_run_calls(gpulib, full, 100, mode=0)
    gpulib.nl2d_finalize()
    a = m.copy()
    T.gpu_run_calls(gpulib, a, 40, mode=0)
    path = str(tmp_path / "ck.bin").encode()
    assert gpulib.nl2d_checkpoint_write(path, 41) == 0
    gpulib.nl2d_finalize()
    b = m.copy()
    T.gpu_register(gpulib, b)
    istep = ctypes.c_int(0)
    assert gpulib.nl2d_checkpoint_read(path, ctypes.byref(istep)) == 0
    assert istep.value == 41
    paths = T.gpu_run_calls(gpulib, b, 60, nit000=41, mode=0)
    assert paths[0] == 1 and set(paths[1:]) == {2}, paths
    assert_fields_equal(b, full, "resumed")
    # another problem's extents, and a file that is not a checkpoint
    gpulib.nl2d_finalize()
    c = T.make_model(40, 33, 1, oracle=oracle)
    T.gpu_register(gpulib, c)
    assert gpulib.nl2d_checkpoint_read(path, ctypes.byref(istep)) == P.NL2D_ERR_ARGS
    junk = tmp_path / "junk.bin"
    junk.write_bytes(b"not a checkpoint" * 8)
    assert gpulib.nl2d_checkpoint_read(str(junk).encode(), ctypes.byref(istep)) == \
        P.NL2D_ERR_PARSE
    buf = ctypes.create_string_buffer(256)
    assert gpulib.nl2d_last_error(buf, 256) == P.NL2D_ERR_PARSE  # the status, then cleared


def test_nan_in_a_field_is_reported_by_the_checksums(gpulib, oracle):
    """A NaN seeded into a host field before upload spreads through the
    steps (which still run); the checksums then report NL2D_ERR_NONFINITE
    instead of a number, and a clean problem registered afterwards runs
    normally."""
    import ctypes
    import psyclonebench_gb300 as P
    m = T.make_model(30, 26, 1, oracle=oracle)
    m.f["sshn_t"][10, 12] = np.nan
    T.gpu_register(gpulib, m)
    out = np.zeros(3)
    assert gpulib.nl2d_run_steps(1, 5, 0, T.dptr(out)) == 0
    assert gpulib.nl2d_checksums(T.dptr(out)) == P.NL2D_ERR_NONFINITE
    buf = ctypes.create_string_buffer(256)
    assert gpulib.nl2d_last_error(buf, 256) == P.NL2D_ERR_NONFINITE
    gpulib.nl2d_finalize()
    c = T.make_model(30, 26, 1, oracle=oracle)
    T.gpu_register(gpulib, c)
    assert gpulib.nl2d_run_steps(1, 5, 0, T.dptr(out)) == 0
    assert gpulib.nl2d_checksums(T.dptr(out)) == 0 and np.isfinite(out).all()


def test_varying_latitude_takes_the_reference_path(gpulib, oracle):
    """Latitudes that vary over the grid: the Coriolis sines are evaluated
    per point with the host libm, the fused path does not apply, and the
    reference-structured steps stay bit-identical to the oracle."""
    m = T.make_model(40, 33, 1, oracle=oracle)
    for k in ("gphiu", "gphiv"):
        m.grid[k][:] = 40.0 + 0.3 * np.arange(m.height)[:, None]
    want = m.copy()
    T.run(oracle.oracle_invoke_time_step, want, 30)
    paths = T.gpu_run_calls(gpulib, m, 30, mode=0)
    assert set(paths) == {1}, paths
    assert_fields_equal(m, want, "varying latitude")


def test_chained_flather_mask_uses_reference_path(gpulib, oracle):
    """A one-cell-wide wet column between two open columns makes a Flather
    face read another Flather face; the library then keeps to the ordered
    reference-structured step and still matches bit for bit."""
    m = T.make_model(16, 12, 1, oracle=oracle)
    t = m.grid["tmask"]
    t[m.ys:m.ye + 1, 5] = -1
    t[m.ys:m.ye + 1, 7] = -1
    want = m.copy()
    T.run(oracle.oracle_invoke_time_step, want, 50)
    paths = T.gpu_run_calls(gpulib, m, 50, mode=0)
    assert set(paths) == {1}
    assert_fields_equal(m, want, "chained")


def test_write_to_device_then_step(gpulib, oracle):
    """c_write_to_device of a perturbed sshn_t mid-run: the next step uses
    it (reference path), later steps fuse again; all bitwise."""
    m = T.make_model(30, 26, 1, oracle=oracle)
    want = m.copy()
    T.run(oracle.oracle_invoke_time_step, want, 20)
    T.gpu_run_calls(gpulib, m, 20, mode=0)
    pert = np.random.default_rng(5).normal(0, 1e-3, size=m.f["sshn_t"].shape)
    for mm in (m, want):
        mm.f["sshn_t"] += pert
    gpulib.c_write_to_device(m.f["sshn_t"].ctypes.data, m.f["sshn_t"].ctypes.data, 1, 1,
                             m.width, m.height, True)
    T.run(oracle.oracle_invoke_time_step, want, 30, nit000=21)
    paths = T.gpu_run_calls(gpulib, m, 30, nit000=21, mode=0)
    assert paths[0] == 1 and paths[-1] == 2
    assert_fields_equal(m, want, "after write")


@pytest.mark.parametrize("breach", ["ssha_t", "ua", "va", "sshn_u", "sshn_v"])
def test_first_step_after_upload_checks_step_consistency(gpulib, oracle, breach):
    """The rest start satisfies what a step leaves (ua == un, va == vn,
    ssha_t == sshn_t on the copy region; sshn_u / sshn_v as next_ssh makes
    them), so its first step is fused.  One cell breaking it sends the first
    step down the reference-structured path; either way 10 steps are bit-
    identical to the oracle."""
    m = T.make_model(37, 29, 3, width=40, oracle=oracle)
    rng = np.random.default_rng(13)
    for k in ("ht", "hu", "hv"):
        m.f[k][:] = rng.uniform(50.0, 500.0, size=m.f[k].shape)
    # a ring cell of the copy region (column xs-1) or an interior face
    j = m.ys + 3
    cell = {"ssha_t": (j, m.xs - 1), "ua": (j, m.xs - 1), "va": (m.ys - 1, m.xs + 4),
            "sshn_u": (j, m.xs + 2), "sshn_v": (j, m.xs + 2)}[breach]
    m.f[breach][cell] = 1e-3
    want = m.copy()
    T.run(oracle.oracle_invoke_time_step, want, 10)
    paths = T.gpu_run_calls(gpulib, m, 10, mode=0)
    assert paths[0] == 1 and set(paths[1:]) == {2}, (breach, paths)
    assert_fields_equal(m, want, breach)
    gpulib.nl2d_finalize()
    clean = T.make_model(37, 29, 3, width=40, oracle=oracle)
    paths = T.gpu_run_calls(gpulib, clean, 3, mode=0)
    assert set(paths) == {2}


def test_transfer_bytes_and_direct_state_read(gpulib, oracle):
    """Registration copies the 25 arrays once; reading sshn_t, un and vn back
    after fused steps copies exactly those fields and needs no other work;
    every field read back equals the oracle."""
    import ctypes
    m = T.make_model(50, 41, 1, oracle=oracle)
    want = m.copy()
    T.run(oracle.oracle_invoke_time_step, want, 8)
    n = m.width * m.height
    for k in range(8):
        gpulib.c_invoke_time_step(*m.step_args(1 + k))
        assert gpulib.nl2d_last_path() == 2
    nb = (ctypes.c_longlong * 2)()
    assert gpulib.nl2d_transfer_bytes(nb) == 0
    assert nb[0] == 24 * n * 8 + n * 4 and nb[1] == 0
    for k in ("sshn_t", "un", "vn"):
        a = m.f[k]
        gpulib.c_read_from_device(a.ctypes.data, a.ctypes.data, 1, 1, m.width, m.height, True)
        assert bits_equal(a, want.f[k]), k
    assert gpulib.nl2d_transfer_bytes(nb) == 0
    assert nb[0] == 24 * n * 8 + n * 4 and nb[1] == 3 * n * 8
    T.gpu_read_all(gpulib, m)
    assert_fields_equal(m, want, "all fields")


def test_partial_read(gpulib, oracle):
    m = T.make_model(20, 20, 1, oracle=oracle)
    T.gpu_run_calls(gpulib, m, 10, mode=0)
    full = m.f["un"].copy()
    dst = np.full_like(full, 7.0)
    gpulib.c_read_from_device(m.f["un"].ctypes.data, dst.ctypes.data, 3, 4, 5, 6, True)
    T.gpu_check(gpulib, "partial read")
    assert bits_equal(dst[3:9, 2:7], full[3:9, 2:7])
    dst[3:9, 2:7] = 7.0
    assert (dst == 7.0).all()


def test_partial_writes(gpulib, oracle):
    """A write of whole rows (one linear copy) and a write of a rectangle (a
    2-D copy) change exactly the cells asked for."""
    m = T.make_model(20, 20, 1, oracle=oracle)
    T.gpu_run_calls(gpulib, m, 5, mode=0)
    before = np.zeros_like(m.f["un"])
    gpulib.c_read_from_device(m.f["un"].ctypes.data, before.ctypes.data, 1, 1, m.width,
                              m.height, True)
    src = np.full_like(before, 1.5)
    src[10:13, 3:9] = -2.5
    gpulib.c_write_to_device(src.ctypes.data, m.f["un"].ctypes.data, 1, 5, m.width, 4, True)
    gpulib.c_write_to_device(src.ctypes.data, m.f["un"].ctypes.data, 4, 11, 6, 3, True)
    got = np.zeros_like(before)
    gpulib.c_read_from_device(m.f["un"].ctypes.data, got.ctypes.data, 1, 1, m.width, m.height,
                              True)
    T.gpu_check(gpulib, "partial writes")
    want = before.copy()
    want[4:8, :] = 1.5
    want[10:13, 3:9] = -2.5
    assert bits_equal(got, want)


def test_errors_are_reported_not_fatal(gpulib, oracle):
    import psyclonebench_gb300 as P
    m = T.make_model(12, 12, 1, oracle=oracle)
    args = m.step_args(1)
    args[26] = 0  # internal_xstart = 0 leaves no ring
    gpulib.c_invoke_time_step(*args)
    with pytest.raises(P.Nl2dError):
        P.check(None, "bad bounds")
    junk = np.zeros(4)
    gpulib.c_read_from_device(junk.ctypes.data, junk.ctypes.data, 1, 1, 2, 2, True)
    with pytest.raises(P.Nl2dError):
        P.check(None, "unknown field")
    # the library still works afterwards
    m2 = T.make_model(12, 12, 1, oracle=oracle)
    want = m2.copy()
    T.run(oracle.oracle_invoke_time_step, want, 5)
    T.gpu_run_calls(gpulib, m2, 5)
    assert_fields_equal(m2, want)


def test_deterministic(gpulib, oracle):
    a = T.make_model(64, 48, 1, oracle=oracle)
    b = a.copy()
    sa = T.gpu_run_graph(gpulib, a, 200, every=50)
    sb = T.gpu_run_graph(gpulib, b, 200, every=50)
    assert bits_equal(sa, sb)
    assert_fields_equal(a, b, "determinism")


@pytest.mark.parametrize("d", [1.0e6, 1.0e3, 2.0e3, 1.0 + 1.5e-4 * 20.0, 100.0, 57.3,
                               3.0, 0.7, 1.0e-30, 4.0e25])
def test_exact_helpers_match_ieee(gpulib, d):
    """The fused step's Markstein division, integer halving and integer
    upwind pick give the IEEE results bit for bit on 2^24 sampled inputs
    per divisor (zeros, subnormals, non-finite and normal values)."""
    import ctypes
    out = (ctypes.c_longlong * 3)()
    assert gpulib.nl2d_selftest_exact(1 << 24, 12345, d, out) == 0
    assert list(out) == [0, 0, 0], list(out)


@pytest.mark.parametrize("seed", [1, 0xC0FFEE])
def test_integer_pipe_add_and_multiply_match_ieee(gpulib, seed):
    """dadd_i / dmul_i (exact IEEE add and multiply done on the integer
    pipes) give the FP64 instructions' bits on 2^27 sampled pairs:
    alignment shifts of 0..70 bits with either sign, near cancellations,
    products at both ends of the normal range, zeros, subnormals,
    infinities and NaNs."""
    import ctypes
    out = (ctypes.c_longlong * 2)()
    assert gpulib.nl2d_selftest_intfp(1 << 27, seed, out) == 0
    assert list(out) == [0, 0], list(out)
