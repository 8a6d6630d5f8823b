"""The ensemble form: many domains, one persistent launch per step.  Every
domain must be bit-identical to the oracle's step with that domain's tide
(which is the reference's step when amplitude 0.2 m and period 12.42 h)."""
import numpy as np
import pytest

import nl2d_testlib as T
from test_oracle import bits_equal

pytestmark = pytest.mark.gpu


def small_specs():
    specs = []
    rng = np.random.default_rng(17)
    for k, side in enumerate("SNEWSNEW"):
        specs.append({"nx": int(rng.integers(12, 45)), "ny": int(rng.integers(12, 45)),
                      "depth_seed": 100 + k, "tide_amp": float(rng.uniform(0.05, 0.5)),
                      "tide_period_h": float(rng.uniform(10.0, 14.0)), "open_side": side})
    specs[0]["tide_amp"], specs[0]["tide_period_h"] = 0.2, 12.42  # the reference's tide
    return specs


@pytest.fixture(scope="module")
def domains():
    from psyclonebench_gb300.ensemble import build_domain
    return [build_domain(s) for s in small_specs()]


@pytest.mark.parametrize("cps,policy,tile", [(2, 0, (32, 16)), (1, 1, (32, 16)),
                                             (2, 2, (32, 16)), (2, 0, (32, 8)),
                                             (2, 1, (16, 16)), (1, 0, (64, 8)),
                                             (2, 2, (32, 32))])
def test_ensemble_matches_oracle(gpulib, oracle, domains, cps, policy, tile):
    """Bit-identical under every schedule and every tile shape."""
    from psyclonebench_gb300.ensemble import Ensemble
    ens = Ensemble(domains, lib=gpulib)
    ens.schedule(cps, policy, 4.0, tile)
    ms, sums = ens.run(1, 90, checksum_every=30)
    assert sums.shape == (3, len(domains), 3)
    for k, d in enumerate(domains):
        want, want_sums = T.ensemble_oracle_run(d, 90, oracle=oracle, every=30)
        sn, un, vn = ens.read(k)
        for name, got in (("sshn_t", sn), ("un", un), ("vn", vn)):
            x0, x1, y0, y1 = T.regions(want)["t"]
            assert bits_equal(got[y0 - 1:y1 + 1, x0 - 1:x1 + 2],
                              want.f[name][y0 - 1:y1 + 1, x0 - 1:x1 + 2]), (k, name)
        w = np.array([[s["sshn_t"], s["un"], s["vn"]] for s in want_sums])
        np.testing.assert_allclose(sums[:, k, :], w, rtol=1e-10, atol=1e-300)
    ens.close()


def test_autotuner_picks_a_schedule(gpulib, domains, tmp_path, monkeypatch):
    from psyclonebench_gb300 import autotune
    from psyclonebench_gb300.ensemble import Ensemble
    monkeypatch.setenv("NL2D_TUNE_CACHE", str(tmp_path))
    ens = Ensemble(domains, lib=gpulib)
    choice = autotune.tune(ens, steps=2)
    n = len(autotune.SCHEDULES) + 2 * (len(autotune.SHAPES) - 1)
    assert not choice["cached"] and len(choice["timings"]) == n
    assert choice["ms_per_step"] == min(t["ms_per_step"] for t in choice["timings"])
    print("autotuner timings (cps, policy, weight, tile: ms/step):",
          [(t["ctas_per_sm"], t["policy"], t["boundary_weight"], t["tile"],
            round(t["ms_per_step"], 4)) for t in choice["timings"]])
    again = autotune.tune(ens, steps=2)
    assert again["cached"] and again["policy"] == choice["policy"]
    # the tuned schedule gives the same bits as any other
    a_ms, a = ens.run(1, 20, checksum_every=20)
    ens.reset()
    ens.schedule(1, 0, 0.0, (64, 8))
    b_ms, b = ens.run(1, 20, checksum_every=20)
    assert bits_equal(a, b)
    ens.close()


def test_mixed_march_strip_heights_agree(gpulib, domains):
    """The mixed form's column march gives the same result for every strip
    height the autotuner searches (each cell's arithmetic is the same)."""
    from psyclonebench_gb300.ensemble import Ensemble
    ens = Ensemble(domains, lib=gpulib)
    ens.set_precision(1)
    got = []
    for mr in (8, 16, 32, 64):
        ens.schedule(2, 0, 4.0, (32, 16), mr)
        ens.reset()
        ens.run(1, 50)
        assert ens.uses_march()
        got.append([ens.read(k)[0] for k in range(len(domains))])
    for k in range(len(domains)):
        assert all(bits_equal(got[0][k], g[k]) for g in got[1:]), k
    ens.close()


def test_mixed_ensemble_error_vs_fp64(gpulib, domains):
    """The FP32 form of the ensemble stays within 1e-6 m ssh RMS of the
    FP64 ensemble (itself bit-identical to the reference) after 300 steps."""
    from psyclonebench_gb300.ensemble import Ensemble
    ens = Ensemble(domains, lib=gpulib)
    ens.run(1, 300)
    ref = [ens.read(k) for k in range(len(domains))]
    ens.set_precision(1)
    _, sums = ens.run(1, 300, checksum_every=300)
    assert ens.uses_march()  # every domain shares the step's constants
    worst = 0.0
    for k, d in enumerate(domains):
        w, h, xs, xe, ys, ye = d["dims"]
        got = ens.read(k)
        diff = got[0][ys:ye + 1, xs:xe + 1] - ref[k][0][ys:ye + 1, xs:xe + 1]
        worst = max(worst, float(np.sqrt(np.mean(diff * diff))))
        assert np.isfinite(got[1]).all() and np.isfinite(got[2]).all()
        np.testing.assert_allclose(sums[0, k, 0], np.abs(got[0][ys:ye + 1, xs:xe + 1]).sum(),
                                   rtol=1e-10)
    print("mixed ensemble worst per-domain ssh RMS error:", worst)
    assert worst <= 1e-6
    ens.close()


def test_mixed_ensemble_with_differing_grids(gpulib, domains):
    """Domains with their own grid spacing and latitude do not share the
    step's constants, so each march warp takes its own domain's; the mixed
    ensemble stays within the same bar against the FP64 ensemble."""
    from psyclonebench_gb300.ensemble import Ensemble
    doms = [dict(d) for d in domains[:4]]
    doms[1]["geo"] = (900.0, 1100.0, 45.0)
    doms[3]["geo"] = (1200.0, 800.0, 30.0)
    ens = Ensemble(doms, lib=gpulib)
    ens.run(1, 300)
    ref = [ens.read(k) for k in range(len(doms))]
    ens.set_precision(1)
    ens.run(1, 300)
    assert ens.uses_march()
    worst = 0.0
    for k, d in enumerate(doms):
        w, h, xs, xe, ys, ye = d["dims"]
        got = ens.read(k)
        diff = got[0][ys:ye + 1, xs:xe + 1] - ref[k][0][ys:ye + 1, xs:xe + 1]
        worst = max(worst, float(np.sqrt(np.mean(diff * diff))))
        assert np.isfinite(got[1]).all() and np.isfinite(got[2]).all()
    print("mixed ensemble, differing grids, worst per-domain ssh RMS error:", worst)
    assert worst <= 1e-6
    ens.close()


# ---- a sample of the benchmark's own 512-domain draw ----------------------

BENCH_ENSEMBLE_SEED = 7  # bench.py's run_ensemble draw


def config3_sample():
    """24 domains of workloads.ensemble_domains(512, 7): the widest and the
    tallest, the two largest by cells, and five more per open side; every
    tide is the domain's own (amplitudes 0.05-0.5 m, periods 10-14 h)."""
    from psyclonebench_gb300.workloads import ensemble_domains
    specs = ensemble_domains(512, BENCH_ENSEMBLE_SEED)
    cells = [s["nx"] * s["ny"] for s in specs]
    pick = [max(range(512), key=lambda k: specs[k]["nx"]),
            max(range(512), key=lambda k: specs[k]["ny"])]
    for k in sorted(range(512), key=lambda k: -cells[k]):
        if len(pick) == 4:
            break
        if k not in pick:
            pick.append(k)
    rng = np.random.default_rng(29)
    for side in "SNEW":
        cand = [k for k in range(512) if specs[k]["open_side"] == side and k not in pick]
        pick += [int(k) for k in rng.choice(cand, size=5, replace=False)]
    return [specs[k] for k in pick]


def _oracle_job(args):
    """Runs in a spawned worker: the oracle's tide-parametrised step of one
    domain; returns its (sshn_t, un, vn)."""
    spec, nsteps = args
    import nl2d_testlib as T
    from psyclonebench_gb300.ensemble import build_domain
    m, _ = T.ensemble_oracle_run(build_domain(spec), nsteps)
    return m.f["sshn_t"], m.f["un"], m.f["vn"]


def test_ensemble_bench_sample_matches_oracle(gpulib):
    """24 domains of the benchmark's 512-domain ensemble (up to 1016 cells
    wide, all four open sides, their own tides), 60 FP64 steps in one
    persistent launch per step: every domain bit-identical to the oracle's
    step with that domain's tide."""
    import multiprocessing as mp

    from psyclonebench_gb300.ensemble import Ensemble, build_domain
    specs = config3_sample()
    assert max(s["nx"] for s in specs) >= 1000 and {s["open_side"] for s in specs} == set("SNEW")
    assert all((s["tide_amp"], s["tide_period_h"]) != (0.2, 12.42) for s in specs)
    nsteps = 60
    with mp.get_context("spawn").Pool(min(8, mp.cpu_count())) as pool:
        pending = pool.map_async(_oracle_job, [(s, nsteps) for s in specs])
        doms = [build_domain(s) for s in specs]
        ens = Ensemble(doms, lib=gpulib)
        ens.run(1, nsteps)
        got = [ens.read(k) for k in range(len(doms))]
        ens.close()
        want = pending.get(timeout=900)
    for k, d in enumerate(doms):
        w, h, xs, xe, ys, ye = d["dims"]
        for f, name in enumerate(("sshn_t", "un", "vn")):
            a = got[k][f][ys - 1:ye + 1, xs - 1:xe + 2]
            b = want[k][f][ys - 1:ye + 1, xs - 1:xe + 2]
            assert bits_equal(a, b), (k, specs[k], name)
        assert np.abs(want[k][0]).max() > 0  # the tide has entered


def test_mixed_ensemble_bench_sample_2000_steps(gpulib):
    """The same 24 domains over 2000 steps: the mixed-precision ensemble
    stays within 1e-6 m ssh RMS of the FP64 ensemble (bit-identical to the
    reference step, previous test) on every domain."""
    from psyclonebench_gb300.ensemble import Ensemble, build_domain
    doms = [build_domain(s) for s in config3_sample()]
    ens = Ensemble(doms, lib=gpulib)
    ens.run(1, 2000)
    ref = [ens.read(k) for k in range(len(doms))]
    ens.set_precision(1)
    ens.run(1, 2000)
    assert ens.uses_march()
    worst = 0.0
    for k, d in enumerate(doms):
        w, h, xs, xe, ys, ye = d["dims"]
        got = ens.read(k)
        assert all(np.isfinite(ref[k][f]).all() for f in range(3))
        diff = got[0][ys:ye + 1, xs:xe + 1] - ref[k][0][ys:ye + 1, xs:xe + 1]
        worst = max(worst, float(np.sqrt(np.mean(diff * diff))))
    ens.close()
    print("bench-sample mixed ensemble worst per-domain ssh RMS error after 2000 steps:", worst)
    assert worst <= 1e-6
