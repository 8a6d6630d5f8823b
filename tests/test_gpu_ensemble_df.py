"""The ensemble's FP64-equivalent form (precision 2): the FP64 state, every
domain's interior by the double-float column march, every other cell by the
fused step's general per-cell code in exact FP64.  Held to the FP64-equivalent contract
against the FP64 ensemble (itself bit-identical to the reference's step with
each domain's tide): relative L2 <= 1e-10 per field and checksums to 10
significant digits; the cells the march does not write are bit-identical
to the FP64 form's after one step from the same state."""
import numpy as np
import pytest

from test_gpu_ensemble import config3_sample, small_specs
from test_oracle import bits_equal
import nl2d_testlib as T

pytestmark = pytest.mark.gpu

REL_L2 = 1e-10
CHECKSUM_RTOL = 1e-10


@pytest.fixture(scope="module")
def domains():
    from psyclonebench_gb300.ensemble import build_domain
    return [build_domain(s) for s in small_specs()]


def copy_region(d, a):
    w, h, xs, xe, ys, ye = d["dims"]
    return a[ys - 1:ye + 1, xs - 1:xe + 2]


def march_cells(d):
    """Cells the double-float march writes: interior cells one inside the
    interior's edge whose 3x3 mask neighbourhood is wet."""
    w, h, xs, xe, ys, ye = d["dims"]
    m = d["tmask"]
    reg = np.zeros((h, w), bool)
    wet = m > 0
    for j in range(ys + 1, ye):
        for i in range(xs + 1, xe):
            reg[j, i] = wet[j - 1:j + 2, i - 1:i + 2].all()
    return reg


def run_pair(gpulib, doms, nsteps, every=0):
    """FP64 ensemble, then the FP64-equivalent form from rest: (reads,
    checksums) of both."""
    from psyclonebench_gb300.ensemble import Ensemble
    ens = Ensemble(doms, lib=gpulib)
    _, s64 = ens.run(1, nsteps, checksum_every=every)
    ref = [ens.read(k) for k in range(len(doms))]
    ens.set_precision(2)
    _, sdf = ens.run(1, nsteps, checksum_every=every)
    got = [ens.read(k) for k in range(len(doms))]
    ens.close()
    return ref, s64, got, sdf


def worst_rel_l2(doms, ref, got):
    worst = 0.0
    for k, d in enumerate(doms):
        for f in range(3):
            a, b = copy_region(d, got[k][f]), copy_region(d, ref[k][f])
            assert np.isfinite(a).all(), (k, f)
            if np.abs(b).max() > 0:
                worst = max(worst, T.rel_l2(a, b))
            else:
                assert np.abs(a).max() == 0, (k, f)
    return worst


def test_df_ensemble_vs_fp64(gpulib, domains):
    """Eight domains (all four open sides, their own tides), 300 steps:
    every field of every domain within relative L2 1e-10 of the FP64
    ensemble, checksums every 100 steps within 1e-10."""
    ref, s64, got, sdf = run_pair(gpulib, domains, 300, every=100)
    worst = worst_rel_l2(domains, ref, got)
    print("FP64-equivalent ensemble worst per-field relative L2:", worst)
    assert worst <= REL_L2
    np.testing.assert_allclose(sdf, s64, rtol=CHECKSUM_RTOL, atol=1e-300)


def test_df_ensemble_strip_heights_agree(gpulib, domains):
    """Every strip height the autotuner searches gives the same bits (each
    cell's arithmetic does not depend on it)."""
    from psyclonebench_gb300.ensemble import Ensemble
    ens = Ensemble(domains, lib=gpulib)
    ens.set_precision(2)
    got = []
    for mr in (8, 16, 32, 64):
        ens.schedule(2, 0, 4.0, (32, 16), mr)
        ens.reset()
        ens.run(1, 60)
        got.append([ens.read(k) for k in range(len(domains))])
    ens.close()
    for k in range(len(domains)):
        for f in range(3):
            assert all(bits_equal(got[0][k][f], g[k][f]) for g in got[1:]), (k, f)


def test_df_ensemble_exact_cells_bitwise(gpulib):
    """From one state (100 FP64 steps, handed over through the interior
    import), one step in each form: every cell the march does not write is
    bit-identical to the FP64 form's, and the march's cells agree to
    relative L2 1e-12."""
    import ctypes

    import torch
    from psyclonebench_gb300.ensemble import Ensemble, build_domain
    # the import and export take domains of one interior size
    spec = small_specs()[0]
    doms = [build_domain(dict(spec, open_side=s, depth_seed=40 + k))
            for k, s in enumerate("SNEW")]
    w, h, xs, xe, ys, ye = doms[0]["dims"]
    nx, ny = xe - xs + 1, ye - ys + 1
    buf = torch.zeros((len(doms), ny, nx, 3), dtype=torch.float32, device="cuda")
    ptr = ctypes.c_void_p(buf.data_ptr())
    ens = Ensemble(doms, lib=gpulib)
    ens.run(1, 100)
    assert gpulib.nl2d_ens_export_interior(ptr) == 0
    torch.cuda.synchronize()
    assert float(buf.abs().max()) > 0
    results = []
    for precision in (0, 2):
        ens.set_precision(precision)
        ens.reset()
        ens.run(1, 0)  # builds the form
        assert gpulib.nl2d_ens_import_interior(ptr) == 0
        ens.run(101, 1)
        results.append([ens.read(k) for k in range(len(doms))])
    ens.close()
    for k, d in enumerate(doms):
        reg = march_cells(d)
        for f in range(3):
            a, b = results[1][k][f], results[0][k][f]
            exact = copy_region(d, ~reg)
            assert bits_equal(copy_region(d, a)[exact], copy_region(d, b)[exact]), (k, f)
            assert reg.any()
            if np.abs(b[reg]).max() > 0:
                assert T.rel_l2(a[reg], b[reg]) <= 1e-12, (k, f)


def test_df_ensemble_with_differing_grids(gpulib, domains):
    """Domains with their own grid spacing and latitude: each march warp
    takes its domain's constants.  300 steps within relative L2 1e-10 of the
    FP64 ensemble (itself bit-identical to the reference step of each
    domain's grid)."""
    doms = [dict(d) for d in domains[:4]]
    doms[1]["geo"] = (900.0, 1100.0, 45.0)
    doms[3]["geo"] = (1200.0, 800.0, 30.0)
    ref, s64, got, sdf = run_pair(gpulib, doms, 300, every=100)
    worst = worst_rel_l2(doms, ref, got)
    print("FP64-equivalent ensemble, differing grids, worst relative L2:", worst)
    assert worst <= REL_L2
    np.testing.assert_allclose(sdf, s64, rtol=CHECKSUM_RTOL, atol=1e-300)


def test_df_ensemble_bench_sample_2000_steps(gpulib):
    """24 domains of the benchmark's 512-domain draw (up to 1016 cells wide,
    all four open sides, their own tides), 2000 steps: every field within
    relative L2 1e-10 of the FP64 ensemble, checksums every 500 steps within
    1e-10."""
    from psyclonebench_gb300.ensemble import build_domain
    doms = [build_domain(s) for s in config3_sample()]
    ref, s64, got, sdf = run_pair(gpulib, doms, 2000, every=500)
    worst = worst_rel_l2(doms, ref, got)
    print("bench-sample FP64-equivalent ensemble worst relative L2 after 2000 steps:", worst)
    assert worst <= REL_L2
    np.testing.assert_allclose(sdf, s64, rtol=CHECKSUM_RTOL, atol=1e-300)


def test_df_ensemble_with_interior_land(gpulib, domains):
    """Blocks of land inside every domain: the cells beside them join the
    exact cells (the march takes only cells whose 3x3 neighbourhood is
    wet).  200 steps within relative L2 1e-10 of the FP64 ensemble."""
    rng = np.random.default_rng(9)
    doms = []
    for d in domains:
        d = dict(d)
        m = d["tmask"].copy()
        w, h, xs, xe, ys, ye = d["dims"]
        for _ in range(3):
            i = int(rng.integers(xs + 3, max(xs + 4, xe - 5)))
            j = int(rng.integers(ys + 3, max(ys + 4, ye - 4)))
            m[j:j + 2, i:i + 3] = 0
        d["tmask"] = m
        doms.append(d)
    ref, s64, got, sdf = run_pair(gpulib, doms, 200, every=100)
    worst = worst_rel_l2(doms, ref, got)
    print("FP64-equivalent ensemble with land, worst relative L2:", worst)
    assert worst <= REL_L2
    np.testing.assert_allclose(sdf, s64, rtol=CHECKSUM_RTOL, atol=1e-300)
