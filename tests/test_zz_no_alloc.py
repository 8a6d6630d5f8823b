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

    d_out = torch.zeros(1, dtype=torch.float64, device="cuda")
    rects = {"sshn_t": (m.xs, m.xe, m.ys, m.ye), "un": (m.xs, m.xe - 1, m.ys, m.ye)}
    # Two calls in a row, each checked against the allocating entry point.
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

    # Beyond the fixed capacity (more than 8192 x 8192 cells): rejected on
    # the host before any launch.
    dptr = gpulib.nl2d_device_ptr(m.f["sshn_t"].ctypes.data)
    rc = gpulib.nl2d_field_checksum_noalloc(dptr, 10000, 0, 9999, 0, 9999,
                                            d_out.data_ptr(), None)
    assert rc == P.NL2D_ERR_TOO_LARGE
    gpulib.nl2d_finalize()
