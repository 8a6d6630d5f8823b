"""The FP64-equivalent form (nl2d_set_precision(2)): interior cells in
double-float arithmetic on the FP32 pipe, the other cells in exact FP64.
Not bit-identical; held to the FP64-equivalent contract against the
reference: relative L2 <= 1e-10 per field and checksums agreeing
to 10 significant digits (relative 1e-10) after 2000 steps of the parity
namelist, and the same bar on bathymetry, random starts and land."""
import os

import numpy as np
import pytest

import nl2d_testlib as T

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
REL_L2 = 1e-10
CHECKSUM_RTOL = 1e-10


def run_df(gpulib, m, nsteps, nit000=1, every=0):
    """nsteps of the FP64-equivalent form through c_invoke_time_step; returns
    the step paths and, with `every`, the checksums after every every-th
    step."""
    import psyclonebench_gb300 as P
    gpulib.nl2d_set_precision(2)
    paths, sums = [], []
    out = np.zeros(3)
    for k in range(nsteps):
        gpulib.c_invoke_time_step(*m.step_args(nit000 + k))
        paths.append(gpulib.nl2d_last_path())
        if every and (k + 1) % every == 0:
            P.check(gpulib.nl2d_checksums(T.dptr(out)), "checksums")
            sums.append(out.copy())
    P.check(None, "c_invoke_time_step")
    T.gpu_read_all(gpulib, m)
    gpulib.nl2d_set_precision(0)
    return paths, sums


def assert_close_fields(got, want, fields=T.FIELDS, tag=""):
    worst = {}
    for k in fields:
        assert np.isfinite(got.f[k]).all(), (tag, k)
        worst[k] = T.rel_l2(got.f[k], want.f[k])
    print(tag, "relative L2 per field:", {k: "%.2e" % v for k, v in worst.items()})
    bad = {k: v for k, v in worst.items() if not v <= REL_L2}
    assert not bad, (tag, bad)


def test_df_cfg0_2000_steps(gpulib, oracle):
    """The parity namelist (128x128 interior, rest start, 0.2 m tide) over
    2000 steps: every field within relative L2 1e-10 of the oracle (itself
    bit-identical to the reference's serial build), and the ssh / u / v
    checksums every 100 steps within 1e-10 of the reference build's."""
    want_sums = np.loadtxt(os.path.join(GOLDEN, "cfg0_checksums.txt"))
    m = T.make_model(130, 130, 1, oracle=oracle)
    want = m.copy()
    T.run(oracle.oracle_invoke_time_step, want, 2000)
    paths, sums = run_df(gpulib, m, 2000, every=100)
    assert set(paths) == {2}, "the FP64-equivalent form did not run"
    assert_close_fields(m, want, tag="cfg0")
    got = np.array(sums)
    np.testing.assert_allclose(got, want_sums[:, :3], rtol=CHECKSUM_RTOL, atol=0)


@pytest.mark.parametrize("case", ["bathymetry_active", "random_land", "open_east_south"])
def test_df_against_oracle(gpulib, oracle, case):
    """Bathymetry with every cell in motion from a random start (the first
    step reference-structured, as after any such upload), 8 % random land
    (cells next to land go to the exact FP64 part), and open east and south
    sides: 300 steps within relative L2 1e-10 of the oracle per field."""
    rng = np.random.default_rng({"bathymetry_active": 1, "random_land": 2,
                                 "open_east_south": 3}[case])
    if case == "open_east_south":
        m = T.make_model(97, 75, 3, width=104, oracle=oracle)
    else:
        m = T.make_model(130, 98, 1, width=136, oracle=oracle)
    from psyclonebench_gb300.workloads import fourier_depth
    ht, hu, hv = fourier_depth(m.width, m.height, 9)
    m.f["ht"][:], m.f["hu"][:], m.f["hv"][:] = ht, hu, hv
    m.rdt = 5.0
    if case == "bathymetry_active":
        for k, a in (("sshn_t", 0.05), ("un", 0.02), ("vn", 0.02)):
            m.f[k][:] = rng.uniform(-a, a, size=m.f[k].shape)
    if case == "random_land":
        inner = m.grid["tmask"][m.ys + 1:m.ye, m.xs + 1:m.xe]
        inner[rng.random(inner.shape) < 0.08] = 0
    want = m.copy()
    T.run(oracle.oracle_invoke_time_step, want, 300)
    paths, _ = run_df(gpulib, m, 300)
    assert set(paths[1:]) == {2}
    assert_close_fields(m, want, tag=case)


def test_df_graph_run_matches_calls(gpulib, oracle):
    """The captured multi-step run of the form (nl2d_run_steps) equals the
    same steps taken one call at a time, bit for bit (same kernels, same
    inputs)."""
    import psyclonebench_gb300 as P
    a = T.make_model(70, 55, 1, oracle=oracle)
    b = a.copy()
    run_df(gpulib, a, 60)
    gpulib.nl2d_finalize()
    T.gpu_register(gpulib, b)
    gpulib.nl2d_set_precision(2)
    out = np.zeros(6)
    P.check(gpulib.nl2d_run_steps(1, 60, 30, T.dptr(out)), "run_steps")
    T.gpu_read_all(gpulib, b)
    gpulib.nl2d_set_precision(0)
    for k in T.FIELDS:
        assert np.array_equal(a.f[k].view(np.int64), b.f[k].view(np.int64)), k


def test_df_bit_conversions(gpulib):
    """split_bits / join_bits / widen_bits (the march's conversions done on
    the integer and FP32 pipes) on values across every range boundary and
    on random values: 47 significant bits kept in range, normalised pairs,
    the stated flushes, infinities and NaN carried through; the join equals
    the FP64 sum of the exactly widened halves, the widening equals the
    exact FP32 -> FP64 conversion (subnormal floats flushed)."""
    rng = np.random.default_rng(5)
    edges = [0.0, -0.0, 1.0, -1.0, np.pi, 2.0 ** -80, -(2.0 ** -80),
             np.nextafter(2.0 ** -80, 0), 2.0 ** -126, np.nextafter(2.0 ** -126, 0),
             2.0 ** -127, 5e-324, -1e-310, np.nextafter(2.0 ** 128, 0), 2.0 ** 128, np.nextafter(2.0 ** 127, 0),
             2.0 ** 127, -1e300,
             np.inf, -np.inf, np.nan, 0.1, -0.2, 3.4e38, 1.0 + 2.0 ** -30, 1.0 - 2.0 ** -40]
    rand = rng.standard_normal(200000) * np.exp(rng.uniform(-60, 60, 200000))
    x = np.concatenate([np.array(edges), rand, rng.uniform(-0.5, 0.5, 50000)])
    n = x.size
    hi, lo = np.zeros(n, np.float32), np.zeros(n, np.float32)
    joined, widened = np.zeros(n), np.zeros(n)
    assert gpulib.nl2d_selftest_df(T.dptr(x), n, hi.ctypes.data, lo.ctypes.data,
                                   T.dptr(joined), T.dptr(widened)) == 0
    ax = np.abs(x)
    fin = np.isfinite(x)
    full = fin & (ax >= 2.0 ** -80) & (ax < 2.0 ** 127)
    pair = hi[full].astype(np.float64) + lo[full].astype(np.float64)
    assert np.all(np.abs(pair - x[full]) <= 2.0 ** -46 * ax[full])
    # normalised: hi is the FP32 rounding of hi + lo
    assert np.array_equal((hi[full] + lo[full]).view(np.int32), hi[full].view(np.int32))
    mid = fin & (ax >= 2.0 ** -126) & (ax < 2.0 ** -80)
    assert np.all(np.abs(hi[mid] - x[mid]) <= 2.0 ** -23 * ax[mid]) and np.all(lo[mid] == 0)
    tiny = fin & (ax < 2.0 ** -126)
    assert np.all(hi[tiny] == 0) and np.all(lo[tiny] == 0)
    assert np.array_equal(np.signbit(hi[tiny]), np.signbit(x[tiny]))
    big = ~np.isnan(x) & (ax >= 2.0 ** 127)
    assert np.array_equal(hi[big], np.where(x[big] > 0, np.inf, -np.inf).astype(np.float32))
    assert np.all(np.isnan(hi[np.isnan(x)]))
    # join: the FP64 sum of the halves, exactly widened
    want = hi[full].astype(np.float64) + lo[full].astype(np.float64)
    assert np.array_equal(joined[full].view(np.int64), want.view(np.int64))
    # widen: exact FP32 -> FP64 for normal floats, signed zero for subnormals
    with np.errstate(over="ignore"):
        f = x.astype(np.float32)
    normal = np.isfinite(f) & (np.abs(f) >= np.float32(2.0 ** -126))
    assert np.array_equal(widened[normal].view(np.int64),
                          f[normal].astype(np.float64).view(np.int64))
    sub = np.isfinite(f) & (np.abs(f) < np.float32(2.0 ** -126))
    assert np.all(widened[sub] == 0)
    assert np.array_equal(np.signbit(widened[sub]), np.signbit(f[sub]))
    inf = np.isinf(f)
    assert np.array_equal(widened[inf], f[inf].astype(np.float64))
    assert np.all(np.isnan(widened[np.isnan(f)]))


@pytest.mark.parametrize("case", ["cfg0", "random_land", "open_east_south"])
def test_df_exact_cells_equal_fp64_step(gpulib, oracle, case):
    """One step of the form from a state both paths share: every copy-region
    cell the double-float march does not write (the exact cells: the edge
    rows, the side columns, the cells next to land) is bit-identical
    to the FP64 step's, so no such cell is left unwritten; the march's cells
    agree to 1e-12 relative to the field's size."""
    rng = np.random.default_rng({"cfg0": 7, "random_land": 8, "open_east_south": 9}[case])
    if case == "open_east_south":
        m = T.make_model(97, 75, 3, width=104, oracle=oracle)
    else:
        m = T.make_model(262, 140, 1, width=264, oracle=oracle)
    from psyclonebench_gb300.workloads import fourier_depth
    if case != "cfg0":
        ht, hu, hv = fourier_depth(m.width, m.height, 4)
        m.f["ht"][:], m.f["hu"][:], m.f["hv"][:] = ht, hu, hv
        m.rdt = 5.0
        for k, a in (("sshn_t", 0.05), ("un", 0.02), ("vn", 0.02)):
            m.f[k][:] = rng.uniform(-a, a, size=m.f[k].shape)
    if case == "random_land":
        inner = m.grid["tmask"][m.ys + 1:m.ye, m.xs + 1:m.xe]
        inner[rng.random(inner.shape) < 0.05] = 0
    # two steps of the FP64 path: the state is then what a step leaves
    T.gpu_run_calls(gpulib, m, 2)
    gpulib.nl2d_finalize()
    a, b = m.copy(), m.copy()
    T.gpu_run_calls(gpulib, a, 1, nit000=3)
    gpulib.nl2d_finalize()
    T.gpu_register(gpulib, b)
    paths, _ = run_df(gpulib, b, 1, nit000=3)
    gpulib.nl2d_finalize()
    assert paths == [2]
    # the march's cells: interior one inside next_ssh's ranges, 3x3 wet
    tm = m.grid["tmask"]
    H, W = tm.shape
    march = np.zeros((H, W), bool)
    wet = np.ones((m.ye - m.ys - 1, m.xe - m.xs - 1), bool)
    for dj in (-1, 0, 1):
        for di in (-1, 0, 1):
            wet &= tm[m.ys + 1 + dj:m.ye + dj, m.xs + 1 + di:m.xe + di] > 0
    march[m.ys + 1:m.ye, m.xs + 1:m.xe] = wet
    copy = np.zeros((H, W), bool)
    copy[m.ys - 1:m.ye + 1, m.xs - 1:m.xe + 2] = True
    exact = copy & ~march
    assert exact.sum() > 0 and march.sum() > 0
    for k in ("sshn_t", "un", "vn"):
        ga, gb = a.f[k], b.f[k]
        assert np.array_equal(ga[exact].view(np.int64), gb[exact].view(np.int64)), k
        scale = max(np.abs(ga[copy]).max(), 1e-30)
        assert np.abs(ga[march] - gb[march]).max() <= 1e-12 * scale, k
