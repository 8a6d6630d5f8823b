"""The tracer-advection iteration on the GPU (tra_adv_compute through the
C-ABI) against the oracle: mydomain bit-identical after several iterations,
from the benchmark's own initial values and from random inputs, across a
re-registration, through the timed run, and the benchmark's checksum."""
import ctypes

import numpy as np
import pytest

import tra_adv_numpy as TN
from test_tra_oracle import oracle_run, quantized_inputs, random_inputs, tra_lib, zero_work

pytestmark = pytest.mark.gpu
_DP = ctypes.POINTER(ctypes.c_double)


def _p(a):
    return a.ctypes.data_as(_DP)


def gpu_compute(lib, f, niter):
    K, J, I = f["mydomain"].shape
    for _ in range(niter):
        lib.tra_adv_compute(_p(f["ztfreez"]), _p(f["pun"]), _p(f["pvn"]), _p(f["pwn"]),
                            _p(f["umask"]), _p(f["vmask"]), _p(f["tmask"]), _p(f["rnfmsk"]),
                            _p(f["rnfmsk_z"]), _p(f["upsmsk"]), _p(f["mydomain"]), _p(f["tsn"]),
                            I, J, K)
    buf = ctypes.create_string_buffer(256)
    assert lib.tra_adv_last_error(buf, 256) == 0, buf.value


def gpu_field(lib, shape):
    out = np.full(shape, np.nan)
    assert lib.tra_adv_read(_p(out)) == 0
    return out


def oracle_field(f, niter):
    g = {n: v.copy() for n, v in f.items()}
    oracle_run(tra_lib(), g, zero_work(g["mydomain"].shape), niter)
    return g["mydomain"]


@pytest.mark.parametrize("dims,kind,niter", [
    ((20, 14, 6), "benchmark", 5),
    ((33, 17, 7), "random", 6),
    ((130, 70, 9), "random", 4),     # several blocks in i and j
    ((9, 8, 2), "random", 3),        # a single active level
    ((47, 35, 6), "quantized", 5),   # signed zeros, zero differences, limiter ties
])
def test_gpu_iteration_is_bit_identical(gpulib, oracle, dims, kind, niter):
    I, J, K = dims
    f = {"benchmark": lambda: TN.init(I, J, K),
         "random": lambda: random_inputs(I, J, K, seed=I + J + K),
         "quantized": lambda: quantized_inputs(I, J, K, seed=I + J + K)}[kind]()
    want = oracle_field(f, niter)
    before = f["mydomain"].copy()
    gpu_compute(gpulib, f, niter)
    got = gpu_field(gpulib, want.shape)
    np.testing.assert_array_equal(got.view(np.int64), want.view(np.int64))  # every bit
    # the host array stays as it was until the caller reads the result back
    np.testing.assert_array_equal(f["mydomain"], before)
    s = ctypes.c_double(0.0)
    assert gpulib.tra_adv_checksum(ctypes.byref(s)) == 0
    assert s.value == tra_lib().tra_oracle_checksum(I, J, K, _p(want))
    gpulib.tra_adv_finalize()


def test_benchmark_size_is_bit_identical(gpulib, oracle):
    """The benchmark's own case, 512 x 512 x 75 from its initial values:
    three iterations through tra_adv_compute and three through the timed
    run, every bit of the field against the (OpenMP) oracle."""
    I, J, K = 512, 512, 75
    f = TN.init(I, J, K)
    g = {n: v.copy() for n, v in f.items()}
    oracle_run(tra_lib(), g, zero_work((K, J, I)), 6, omp=True)
    gpu_compute(gpulib, f, 3)
    ms = ctypes.c_double(0.0)
    assert gpulib.tra_adv_run(3, ctypes.byref(ms)) == 0
    got = gpu_field(gpulib, (K, J, I))
    np.testing.assert_array_equal(got.view(np.int64), g["mydomain"].view(np.int64))
    s = ctypes.c_double(0.0)
    assert gpulib.tra_adv_checksum(ctypes.byref(s)) == 0
    assert s.value == tra_lib().tra_oracle_checksum(I, J, K, _p(g["mydomain"]))
    gpulib.tra_adv_finalize()


def test_new_arrays_start_a_new_run_and_run_continues(gpulib, oracle):
    """Other arrays register afresh (work arrays zeroed again); the timed
    run continues the registered state."""
    f = random_inputs(24, 18, 5, seed=9)
    gpu_compute(gpulib, f, 2)
    g = {n: v.copy() for n, v in f.items()}  # new host arrays, same values
    gpu_compute(gpulib, g, 2)
    ms = ctypes.c_double(0.0)
    assert gpulib.tra_adv_run(3, ctypes.byref(ms)) == 0 and ms.value > 0
    np.testing.assert_array_equal(gpu_field(gpulib, f["mydomain"].shape), oracle_field(f, 5))
    gpulib.tra_adv_finalize()


def test_bad_extents_are_reported(gpulib):
    f = random_inputs(5, 5, 3, seed=1)
    lib = gpulib
    lib.tra_adv_compute(_p(f["ztfreez"]), _p(f["pun"]), _p(f["pvn"]), _p(f["pwn"]),
                        _p(f["umask"]), _p(f["vmask"]), _p(f["tmask"]), _p(f["rnfmsk"]),
                        _p(f["rnfmsk_z"]), _p(f["upsmsk"]), _p(f["mydomain"]), _p(f["tsn"]),
                        2, 5, 3)
    buf = ctypes.create_string_buffer(256)
    assert lib.tra_adv_last_error(buf, 256) == 2 and b"extents" in buf.value
    assert lib.tra_adv_last_error(buf, 256) == 0
