"""The allocation-free checksum entry point (nl2d_field_checksum_noalloc).

It exists for callers that cannot call cudaMalloc — a host model whose own
memory manager owns every device buffer, or a time loop that must not
trigger the synchronisation an allocation can cause — and keeps its partial
sums in a fixed device array inside the library.  This file is collected
last so that a stop-at-first-failure run has already run every other test.
"""
import numpy as np
import pytest

import nl2d_testlib as T

pytestmark = pytest.mark.gpu

CHECKSUM_RTOL = 1e-10  # the tolerance the other checksum tests use
LIMIT_CELLS = 8192 * 8192  # 16384 partials of 4096 cells


def host_sum(a, x0, x1, y0, y1):
    return float(np.abs(a[y0:y1 + 1, x0:x1 + 1]).sum())


def test_noalloc_checksum_matches_library_checksum(gpulib, oracle):
    import psyclonebench_gb300 as P
    import torch

    m = T.make_model(203, 151, 3, width=208, oracle=oracle)
    rng = np.random.default_rng(2)
    for k in ("ht", "hu", "hv"):
        m.f[k][:] = rng.uniform(50, 500, size=m.f[k].shape)
    T.gpu_register(gpulib, m)
    out = np.zeros(3)
    P.check(gpulib.nl2d_run_steps(1, 40, 0, T.dptr(out)), "run")
    T.gpu_read_all(gpulib, m)

    d_out = torch.zeros(1, dtype=torch.float64, device="cuda")
    rects = {"sshn_t": (m.xs, m.xe, m.ys, m.ye), "un": (m.xs, m.xe - 1, m.ys, m.ye)}
    # Two calls in a row, each checked against the allocating entry point
    # and against a host sum of the same field.
    for name in ("sshn_t", "un"):
        x0, x1, y0, y1 = rects[name]
        want = np.zeros(1)
        P.check(gpulib.nl2d_field_checksum(m.f[name].ctypes.data, x0, x1, y0, y1,
                                           T.dptr(want)), "nl2d_field_checksum")
        dptr = gpulib.nl2d_device_ptr(m.f[name].ctypes.data)
        assert dptr
        P.check(gpulib.nl2d_sync(), "sync")
        rc = gpulib.nl2d_field_checksum_noalloc(dptr, m.width, x0, x1, y0, y1,
                                                d_out.data_ptr(), None)
        assert rc == P.NL2D_OK
        torch.cuda.synchronize()
        got = float(d_out.item())
        assert want[0] > 0
        np.testing.assert_allclose(got, want[0], rtol=CHECKSUM_RTOL, atol=0)
        np.testing.assert_allclose(got, host_sum(m.f[name], x0, x1, y0, y1),
                                   rtol=CHECKSUM_RTOL, atol=0)

    # Queued on a side stream (the caller's cudaStream_t).
    side = torch.cuda.Stream()
    x0, x1, y0, y1 = rects["sshn_t"]
    dptr = gpulib.nl2d_device_ptr(m.f["sshn_t"].ctypes.data)
    with torch.cuda.stream(side):
        d_side = torch.zeros(1, dtype=torch.float64, device="cuda")
        rc = gpulib.nl2d_field_checksum_noalloc(dptr, m.width, x0, x1, y0, y1,
                                                d_side.data_ptr(), side.cuda_stream)
    assert rc == P.NL2D_OK
    side.synchronize()
    np.testing.assert_allclose(float(d_side.item()), host_sum(m.f["sshn_t"], x0, x1, y0, y1),
                               rtol=CHECKSUM_RTOL, atol=0)
    gpulib.nl2d_finalize()


def test_noalloc_checksum_capacity_boundary(gpulib):
    """Exactly 8192 x 8192 cells fit the fixed array and give the host sum;
    one column more is rejected on the host before any launch."""
    import psyclonebench_gb300 as P
    import torch

    n = 8192
    g = torch.Generator(device="cuda").manual_seed(5)
    f = torch.rand(n, n, dtype=torch.float64, device="cuda", generator=g) - 0.5
    d_out = torch.zeros(1, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    assert n * n == LIMIT_CELLS
    rc = gpulib.nl2d_field_checksum_noalloc(f.data_ptr(), n, 0, n - 1, 0, n - 1,
                                            d_out.data_ptr(), None)
    assert rc == P.NL2D_OK
    torch.cuda.synchronize()
    want = float(np.abs(f.cpu().numpy()).sum())
    np.testing.assert_allclose(float(d_out.item()), want, rtol=CHECKSUM_RTOL, atol=0)
    # 8193 x 8192 cells: one partial too many (never launched, so the
    # rectangle may exceed the allocation).
    rc = gpulib.nl2d_field_checksum_noalloc(f.data_ptr(), n + 1, 0, n, 0, n - 1,
                                            d_out.data_ptr(), None)
    assert rc == P.NL2D_ERR_TOO_LARGE
    rc = gpulib.nl2d_field_checksum_noalloc(f.data_ptr(), 10000, 0, 9999, 0, 9999,
                                            d_out.data_ptr(), None)
    assert rc == P.NL2D_ERR_TOO_LARGE
    del f
