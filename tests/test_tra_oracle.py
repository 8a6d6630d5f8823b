"""The tracer-advection oracle (oracle/tra_adv_oracle.c) against an
independent numpy restatement of tra_adv.F90: bit-identical fields and work
arrays after several iterations, from the benchmark's own initial values and
from random inputs; the OpenMP form equals the serial one."""
import ctypes

import numpy as np
import pytest

import tra_adv_numpy as TN
from nl2d_testlib import load_oracle

_DP = ctypes.POINTER(ctypes.c_double)
IN3 = ("mydomain", "tsn", "pun", "pvn", "pwn", "umask", "vmask", "tmask")
IN2 = ("ztfreez", "rnfmsk", "upsmsk")
WORK = ("zwx", "zwy", "zslpx", "zslpy", "zind")


def tra_lib():
    lib = load_oracle()
    for name in ("tra_oracle_step", "tra_oracle_step_omp"):
        fn = getattr(lib, name)
        fn.argtypes = [ctypes.c_int] * 3 + [_DP] * 17
        fn.restype = None
    lib.tra_oracle_init.argtypes = [ctypes.c_int] * 3 + [_DP] * 12
    lib.tra_oracle_init.restype = None
    lib.tra_oracle_checksum.argtypes = [ctypes.c_int] * 3 + [_DP]
    lib.tra_oracle_checksum.restype = ctypes.c_double
    return lib


def _p(a):
    return a.ctypes.data_as(_DP)


def oracle_run(lib, f, w, niter, omp=False):
    """Advances f (mydomain in place) and the work arrays w by niter oracle
    iterations."""
    K, J, I = f["mydomain"].shape
    fn = lib.tra_oracle_step_omp if omp else lib.tra_oracle_step
    for _ in range(niter):
        fn(I, J, K, _p(f["mydomain"]), _p(f["tsn"]), _p(f["pun"]), _p(f["pvn"]), _p(f["pwn"]),
           _p(f["umask"]), _p(f["vmask"]), _p(f["tmask"]), _p(f["ztfreez"]), _p(f["rnfmsk"]),
           _p(f["upsmsk"]), _p(f["rnfmsk_z"]), *[_p(w[n]) for n in WORK])


def random_inputs(jpi, jpj, jpk, seed):
    rng = np.random.default_rng(seed)
    f = {n: rng.uniform(-1.0, 1.0, size=(jpk, jpj, jpi)) for n in IN3}
    for n in ("umask", "vmask", "tmask"):
        f[n] = rng.uniform(0.0, 1.0, size=(jpk, jpj, jpi))
    f.update({n: rng.uniform(0.0, 1.0, size=(jpj, jpi)) for n in IN2})
    f["rnfmsk_z"] = rng.uniform(0.0, 1.0, size=jpk)
    return f


def quantized_inputs(jpi, jpj, jpk, seed):
    """Fields drawn from a few values, signed zeros included, so that zero
    differences, signed-zero products, ties in the limiter and zero
    velocities are frequent."""
    rng = np.random.default_rng(seed)
    vals = np.array([-2.0, -1.0, -0.5, -0.0, 0.0, 0.5, 1.0, 2.0])
    f = {n: rng.choice(vals, size=(jpk, jpj, jpi)) for n in IN3}
    for n in ("umask", "vmask", "tmask"):
        f[n] = rng.choice(np.array([0.0, 0.5, 1.0]), size=(jpk, jpj, jpi))
    f.update({n: rng.choice(np.array([0.0, 0.25, 1.0]), size=(jpj, jpi)) for n in IN2})
    f["rnfmsk_z"] = rng.choice(np.array([0.0, 1.0]), size=jpk)
    return f


def zero_work(shape):
    return {n: np.zeros(shape) for n in WORK}


def test_init_is_the_benchmarks(oracle):
    lib = tra_lib()
    I, J, K = 7, 5, 4
    f = {n: np.zeros((K, J, I)) for n in IN3}
    f.update({n: np.zeros((J, I)) for n in IN2})
    f["rnfmsk_z"] = np.zeros(K)
    lib.tra_oracle_init(I, J, K, *[_p(f[n]) for n in IN3 + IN2 + ("rnfmsk_z",)])
    want = TN.init(I, J, K)
    for n in f:
        np.testing.assert_array_equal(f[n], want[n], err_msg=n)
    assert list(f["rnfmsk_z"]) == [0.0, 0.0, 0.0, 1.0]  # jk / jpk is an integer division


@pytest.mark.parametrize("dims,kind,niter", [
    ((12, 9, 6), "benchmark", 4),
    ((16, 11, 7), "random", 3),
    ((9, 8, 2), "random", 3),      # a single active level
    ((20, 14, 5), "benchmark", 6),
    ((18, 13, 6), "quantized", 5),
])
def test_c_oracle_equals_numpy_restatement(oracle, dims, kind, niter):
    lib = tra_lib()
    I, J, K = dims
    f = {"benchmark": lambda: TN.init(I, J, K),
         "random": lambda: random_inputs(I, J, K, seed=I * J + K),
         "quantized": lambda: quantized_inputs(I, J, K, seed=I * J + K)}[kind]()
    g = {n: v.copy() for n, v in f.items()}
    w, wn = zero_work((K, J, I)), zero_work((K, J, I))
    oracle_run(lib, f, w, niter)
    for _ in range(niter):
        TN.step(g, wn)
    np.testing.assert_array_equal(f["mydomain"].view(np.int64), g["mydomain"].view(np.int64))
    for n in WORK:
        np.testing.assert_array_equal(w[n].view(np.int64), wn[n].view(np.int64), err_msg=n)
    assert lib.tra_oracle_checksum(I, J, K, _p(f["mydomain"])) == TN.checksum(g["mydomain"])
    assert np.isfinite(f["mydomain"]).all()


def test_openmp_form_equals_serial(oracle):
    lib = tra_lib()
    f = random_inputs(40, 30, 9, seed=3)
    g = {n: v.copy() for n, v in f.items()}
    w, w2 = zero_work((9, 30, 40)), zero_work((9, 30, 40))
    oracle_run(lib, f, w, 3)
    oracle_run(lib, g, w2, 3, omp=True)
    np.testing.assert_array_equal(f["mydomain"], g["mydomain"])
