"""The first c_invoke_time_step over pinned arrays uploads the arrays a
fused step reads, starts fused steps and lets the other arrays and the
registration scan follow on a second stream; a later call keeps those
steps or restores the uploaded state and takes them again by the path
rules the scan decides.  Every outcome is bit-identical to the oracle (the
reference's serial step)."""
import ctypes

import numpy as np
import pytest

import nl2d_testlib as T
from test_oracle import bits_equal

pytestmark = pytest.mark.gpu


def assert_fields_equal(got, want, tag=""):
    bad = [k for k in T.FIELDS if not bits_equal(got.f[k], want.f[k])]
    assert not bad, (tag, bad)


def counts(gpulib):
    out = (ctypes.c_int * 2)()
    assert gpulib.nl2d_speculation_counts(out) == 0
    return out[0], out[1]


def run_pinned(gpulib, m, nsteps, read_after=None, verdict=None, istep0=1):
    """nsteps calls (isteps istep0 ...) over m's arrays pinned; with
    read_after = k, sshn_t is read back right after step k (before the next
    call).  verdict "kept" or "redone": the speculation must have ended that
    way."""
    before = counts(gpulib)
    held = T.pin_model(gpulib, m)
    try:
        paths = []
        for k in range(nsteps):
            gpulib.c_invoke_time_step(*m.step_args(istep0 + k))
            paths.append(gpulib.nl2d_last_path())
            if read_after == k + 1:
                a = m.f["sshn_t"]
                gpulib.c_read_from_device(a.ctypes.data, a.ctypes.data, 1, 1, m.width,
                                          m.height, True)
                paths.append(("read", a.copy()))
        T.gpu_check(gpulib, "pinned run")
        T.gpu_read_all(gpulib, m)
        gpulib.nl2d_finalize()
        after = counts(gpulib)
        if verdict:
            want = (1, 0) if verdict == "kept" else (0, 1)
            assert (after[0] - before[0], after[1] - before[1]) == want, (verdict, before, after)
        return paths
    finally:
        T.unpin_model(gpulib, held)


def big_model(oracle, seed):
    """1024 x 1024 interior: the late arrays' copies outlast a few steps."""
    m = T.make_model(1026, 1026, 1, width=1032, oracle=oracle)
    rng = np.random.default_rng(seed)
    return m, rng


def test_speculation_kept_rest_start(gpulib, oracle):
    """The reference's rest start: every step fused from the first, the
    speculation kept, 40 steps bit-identical to the oracle."""
    m, _ = big_model(oracle, 1)
    want = m.copy()
    T.run(oracle.oracle_invoke_time_step, want, 40)
    paths = run_pinned(gpulib, m, 40, verdict="kept")
    assert set(paths) == {2}, paths
    assert_fields_equal(m, want, "kept")


def test_speculation_rolled_back_metric(gpulib, oracle):
    """One interior point of area_t differs: the fused path does not apply.
    The steps taken before the scan answered are undone and taken again on
    the reference-structured path; 12 steps bit-identical to the oracle."""
    m, _ = big_model(oracle, 2)
    m.grid["area_t"][m.ys + 500, m.xs + 300] *= 1.0000001
    want = m.copy()
    T.run(oracle.oracle_invoke_time_step, want, 12)
    paths = run_pinned(gpulib, m, 12, verdict="redone")
    assert paths[-1] == 1, paths
    assert_fields_equal(m, want, "metric")


def test_speculation_rolled_back_state(gpulib, oracle):
    """A random start is not what a step leaves: the first step must be
    reference-structured, the later ones fused; the speculative fused steps
    are undone and taken again that way, bit-identical to the oracle."""
    m, rng = big_model(oracle, 3)
    for k, a in (("sshn_t", 0.05), ("un", 0.02), ("vn", 0.02)):
        m.f[k][:] = rng.uniform(-a, a, size=m.f[k].shape)
    want = m.copy()
    T.run(oracle.oracle_invoke_time_step, want, 12)
    paths = run_pinned(gpulib, m, 12, verdict="redone")
    assert paths[-1] == 2, paths
    assert_fields_equal(m, want, "state")


def test_read_during_speculation(gpulib, oracle):
    """A read right after the first step waits for the verdict and returns
    the oracle's field after one step; the run then carries on."""
    m, rng = big_model(oracle, 4)
    for k, a in (("un", 0.02), ("vn", 0.02)):
        m.f[k][:] = rng.uniform(-a, a, size=m.f[k].shape)
    one = m.copy()
    T.run(oracle.oracle_invoke_time_step, one, 1)
    want = m.copy()
    T.run(oracle.oracle_invoke_time_step, want, 6)
    paths = run_pinned(gpulib, m, 6, read_after=1, verdict="redone")
    got1 = [p for p in paths if isinstance(p, tuple)][0][1]
    assert bits_equal(got1, one.f["sshn_t"])
    assert_fields_equal(m, want, "read")


@pytest.mark.parametrize("jpiglo,jpjglo", [(32, 14), (64, 52), (302, 132), (1026, 1026)])
def test_banded_first_step(gpulib, oracle, jpiglo, jpjglo):
    """The step arrays go up in row bands (1, 4, 8 and 8 bands of the fused
    step's tile rows here) and the first fused step runs band by band behind
    them.  From a state the oracle's own steps left (so the speculation is
    kept and every field is in motion), 20 steps bit-identical to the
    oracle's next 20."""
    m = T.make_model(jpiglo, jpjglo, 1, oracle=oracle)
    T.run(oracle.oracle_invoke_time_step, m, 30)
    assert np.abs(m.f["un"]).max() > 0
    want = m.copy()
    T.run(oracle.oracle_invoke_time_step, want, 20, nit000=31)
    paths = run_pinned(gpulib, m, 20, verdict="kept", istep0=31)
    assert set(paths) == {2}, paths
    assert_fields_equal(m, want, "banded")
