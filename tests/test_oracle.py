"""CPU tests: the oracle restatement against the reference's own compiled
step (where it was built here) and against the committed golden fixtures."""
import os

import numpy as np
import pytest

import nl2d_testlib as T

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ["small_s_open", "small_e_open", "small_se_open", "small_bathy"]


def load_case(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    nx, ny, jphgr, nsteps, width, height = (int(v) for v in z["meta"])
    m = T.make_model(nx, ny, jphgr, width=width, height=height)
    for k in ("ht", "hu", "hv"):
        m.f[k][:] = z["init_" + k]
    return m, nsteps, {k: z["final_" + k] for k in T.FIELDS}


def bits_equal(a, b):
    return np.array_equal(np.asarray(a).view(np.int64), np.asarray(b).view(np.int64))


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_golden_fields(oracle, name):
    m, nsteps, want = load_case(name)
    T.run(oracle.oracle_invoke_time_step, m, nsteps)
    for k in T.FIELDS:
        assert bits_equal(m.f[k], want[k]), k


@pytest.mark.parametrize("name", CASES[:2])
def test_oracle_omp_matches_serial(oracle, name):
    m, nsteps, want = load_case(name)
    T.run(oracle.oracle_invoke_time_step_omp, m, nsteps)
    for k in T.FIELDS:
        assert bits_equal(m.f[k], want[k]), k


def test_oracle_cfg0_checksums(oracle):
    """128x128 interior, 2000 steps: checksums every 100 steps agree with the
    reference serial build's to 1e-12 relative (same serial summation, so in
    practice bit for bit)."""
    want = np.loadtxt(os.path.join(GOLDEN, "cfg0_checksums.txt"))
    m = T.make_model(130, 130, 1, oracle=oracle)
    sums = []
    T.run(oracle.oracle_invoke_time_step, m, 2000, every=100, checksums=sums)
    got = np.array([[s[k] for k in ("sshn_t", "un", "vn", "ua", "va")] for s in sums])
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=0)


def test_oracle_matches_reference_build_random_masks(oracle):
    """Where the reference's own step was compiled here (oracle/_ref), the
    restatement is bit-identical to it on random masks, including masks
    with open cells inside the domain."""
    ref = T.load_ref("serial")
    if ref is None:
        pytest.skip("reference not built here (oracle/_ref)")
    rng = np.random.default_rng(3)
    for trial in range(6):
        nx, ny = rng.integers(8, 30, size=2)
        m = T.make_model(int(nx), int(ny), int(rng.integers(1, 4)),
                         width=int(nx) + 1 + int(rng.integers(0, 4)), oracle=oracle)
        inner = m.grid["tmask"][m.ys + 1:m.ye, m.xs + 1:m.xe]
        land = rng.random(inner.shape) < 0.1
        inner[land] = 0
        for k in ("ht", "hu", "hv"):
            m.f[k][:] = rng.uniform(50, 500, size=m.f[k].shape)
        m2 = m.copy()
        T.run(oracle.oracle_invoke_time_step, m, 40)
        T.run(ref.c_invoke_time_step, m2, 40)
        for k in T.FIELDS:
            assert bits_equal(m.f[k], m2.f[k]), (trial, k)


@pytest.mark.parametrize("kind,port", [("omp", "oracle_invoke_time_step_omp"),
                                       ("ompopt", "oracle_invoke_time_step_ompopt")])
def test_openmp_ports_match_reference_builds(oracle, kind, port):
    """The two OpenMP ports timed as CPU baselines (the worksharing layer and
    the partially fused one) are bit-identical to the reference's own
    time_step_omp.cpp / time_step_ompopt.cpp compiled here, on the parity
    namelist and on a random-mask case with open east and south sides."""
    ref = T.load_ref(kind)
    if ref is None:
        pytest.skip("reference not built here (oracle/_ref)")
    rng = np.random.default_rng(5)
    cases = [T.make_model(40, 33, 1, oracle=oracle),
             T.make_model(29, 37, 3, width=33, oracle=oracle)]
    inner = cases[1].grid["tmask"][2:-4, 2:-4]
    inner[rng.random(inner.shape) < 0.08] = 0
    for k in ("ht", "hu", "hv"):
        cases[1].f[k][:] = rng.uniform(50, 500, size=cases[1].f[k].shape)
    for m in cases:
        m2 = m.copy()
        T.run(getattr(oracle, port), m, 60)
        T.run(ref.c_invoke_time_step, m2, 60)
        for k in T.FIELDS:
            assert bits_equal(m.f[k], m2.f[k]), (kind, k)


def test_ompopt_layer_skips_the_east_column_of_next_sshv(oracle):
    """The reference's partially fused layer runs next_sshv over next_sshu's
    range, [xs, xe-1] x [ys, ye] (time_step_ompopt.cpp:141-147), where the
    serial layer uses [xs, xe] x [ys, ye-1] (time_step.cpp:131-136): column
    xe of sshn_v keeps its initial value and row ye is written.  So the
    fields differ from the serial step's; the CPU baseline that times it
    does the same amount of work on a slightly different computation."""
    m = T.make_model(40, 33, 1, oracle=oracle)
    m2 = m.copy()
    T.run(oracle.oracle_invoke_time_step_ompopt, m, 80)
    T.run(oracle.oracle_invoke_time_step, m2, 80)
    assert (m.f["sshn_v"][m.ys:m.ye, m.xe] == 0).all()
    assert (m2.f["sshn_v"][m.ys:m.ye, m.xe] != 0).any()
    assert (m.f["sshn_v"][m.ye, m.xs:m.xe] != 0).any()
    assert (m2.f["sshn_v"][m.ye, :] == 0).all()
    assert 0 < T.rel_l2(m.f["sshn_t"], m2.f["sshn_t"]) < 1e-3


def test_tmask_builder(oracle):
    """model_mod.f90:94-249 for one rank: walls west/north, open south
    (jphgr 1), east (2) or both (3); southern row wins at the corners."""
    for jphgr, s_val, e_val in ((1, -1, 0), (2, 0, -1), (3, -1, -1)):
        m = T.make_model(10, 8, jphgr, width=13, oracle=oracle)
        t = m.grid["tmask"]
        assert (t[m.ys:m.ye + 1, m.xs:m.xe + 1] == 1).all()
        assert (t[:, 0] == np.where(np.arange(m.height) < m.ys, s_val, 0)).all()
        # east (assigned after north) wins at the NE corner, south at the S corners
        assert (t[m.ye + 1:, :m.xe + 1] == 0).all()
        assert (t[m.ys:, m.xe + 1:] == e_val).all()
        assert (t[m.ys:m.ye + 1, m.xe + 1:] == e_val).all()
        assert (t[0, :] == s_val).all()
    assert oracle.oracle_setup_tmask(0, 5, 5, 1, 3, 1, 3, T.iptr(np.zeros((5, 5), np.int32))) == -1


def test_namelist_reader(oracle, tmp_path):
    import ctypes
    p = tmp_path / "namelist"
    p.write_text("!---\n&namctl   ! example\n   jpiglo = 66 ! cols\n  JPJGLO=34\n"
                 "  jphgr_msh = 3\n dx = 250.0\n dy = 5.0d2\n dep_const = 40.0\n"
                 " nit000 = 3\n nitend = 77\n irecord = 1000\n rdt = 12.5\n"
                 " cbfr = 0.0002\n visc = 0.5\n/\n")
    ints = np.zeros(6, np.int32)
    dbls = np.zeros(6, np.float64)
    rc = oracle.oracle_read_namelist(str(p).encode(), T.iptr(ints), T.dptr(dbls))
    assert rc == 0
    assert list(ints) == [66, 34, 3, 3, 77, 1000]
    assert list(dbls) == [250.0, 500.0, 40.0, 12.5, 0.0002, 0.5]
    p.write_text("&namctl\n bogus = 1\n/\n")
    assert oracle.oracle_read_namelist(str(p).encode(), T.iptr(ints), T.dptr(dbls)) == -2
    assert oracle.oracle_read_namelist(b"/nonexistent/namelist", T.iptr(ints),
                                       T.dptr(dbls)) == -1
    del ctypes
