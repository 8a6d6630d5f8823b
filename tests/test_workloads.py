"""CPU tests of the synthetic workloads against the configurations they
stand for: the Fourier bathymetry of the mixed-precision case (depths
clipped to [50, 500] m, U / V depths the same function half a cell east /
north), and the seeded ensemble of independent domains (sizes log-uniform
in [64, 1024] per axis, tide amplitude U(0.05, 0.5) m, period U(10, 14) h,
one open side of four), with their array layout and open-side masks."""
import math

import numpy as np

from psyclonebench_gb300.ensemble import build_domain, domain_layout, open_side_mask
from psyclonebench_gb300.workloads import ensemble_domains, fourier_depth


def test_fourier_depth_range_staggering_and_seed():
    ht, hu, hv = fourier_depth(96, 64, seed=7)
    for a in (ht, hu, hv):
        assert a.shape == (64, 96) and a.dtype == np.float64
        assert a.min() >= 50.0 and a.max() <= 500.0
    assert not np.array_equal(ht, hu) and not np.array_equal(ht, hv)
    # the same seed gives the same arrays, another seed other arrays
    again = fourier_depth(96, 64, seed=7)
    assert all(np.array_equal(x, y) for x, y in zip((ht, hu, hv), again))
    assert not np.array_equal(ht, fourier_depth(96, 64, seed=8)[0])
    # U points: the T-point function half a cell east.  On a domain twice as
    # wide with half the cell size the T points at odd columns are those U
    # points of the coarse domain (same physical size, same modes).
    fine = fourier_depth(192, 64, seed=7, dx=500.0)[0]
    interior = (ht > 50.0) & (ht < 500.0) & (hu > 50.0) & (hu < 500.0)
    np.testing.assert_allclose(fine[:, 1::2][interior], hu[interior], rtol=1e-12)


def test_ensemble_domains_follow_the_spec():
    specs = ensemble_domains(512, seed=7)
    assert len(specs) == 512
    nx = np.array([s["nx"] for s in specs])
    ny = np.array([s["ny"] for s in specs])
    assert nx.min() >= 64 and nx.max() <= 1024 and ny.min() >= 64 and ny.max() <= 1024
    # log-uniform: the median of log2(size) near the middle of [6, 10]
    assert abs(np.median(np.log2(np.concatenate([nx, ny]))) - 8.0) < 0.3
    amp = np.array([s["tide_amp"] for s in specs])
    per = np.array([s["tide_period_h"] for s in specs])
    assert amp.min() >= 0.05 and amp.max() <= 0.5
    assert per.min() >= 10.0 and per.max() <= 14.0
    assert {s["open_side"] for s in specs} == set("SNEW")
    assert ensemble_domains(512, seed=7) == specs
    assert ensemble_domains(512, seed=8) != specs


def test_domain_layout_and_open_side_masks():
    for nx, ny in ((64, 64), (100, 333), (1023, 65)):
        width, height, xs, xe, ys, ye = domain_layout(nx, ny)
        assert (xe - xs + 1, ye - ys + 1) == (nx, ny)
        assert width % 8 == 0 and width >= nx + 3 and height == ny + 3
        for side in "SNEW":
            m = open_side_mask(side, width, height, xs, xe, ys, ye)
            assert (m[ys:ye + 1, xs:xe + 1] == 1).all()
            open_cells = {"W": m[ys:ye + 1, xs - 1], "E": m[ys:ye + 1, xe + 1],
                          "S": m[ys - 1, xs:xe + 1], "N": m[ye + 1, xs:xe + 1]}
            for s, cells in open_cells.items():
                assert (cells == (-1 if s == side else 0)).all(), (side, s)


def test_build_domain_carries_the_spec():
    spec = ensemble_domains(3, seed=11)[1]
    d = build_domain(spec)
    width, height, xs, xe, ys, ye = d["dims"]
    assert (xe - xs + 1, ye - ys + 1) == (spec["nx"], spec["ny"])
    assert d["tmask"].shape == d["ht"].shape == (height, width)
    assert d["tide"] == (spec["tide_amp"], spec["tide_period_h"])
    assert math.isfinite(float(d["hu"].sum()))
