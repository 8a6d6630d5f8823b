"""CPU tests of the ensemble schedule autotuner's host logic with a stand-in
ensemble: it times every candidate schedule, applies the fastest, leaves
the ensemble at rest after each trial, caches the choice per domain-size
signature and reuses it without timing again."""
import pytest

from psyclonebench_gb300 import autotune


class FakeEnsemble:
    """The calls tune() makes on an Ensemble: schedule, run, reset."""

    def __init__(self, domains, cost):
        self.domains = domains
        self.cost = cost          # ms per step of a (ctas_per_sm, policy, weight)
        self.cur = None
        self.resets = 0

    def schedule(self, cps, pol, bw):
        self.cur = (cps, pol, bw)

    def run(self, every, steps):
        return self.cost(self.cur) * steps, None

    def reset(self):
        self.resets += 1


def dom(nx, ny):
    return {"dims": (nx + 2, ny + 2, 1, nx, 1, ny)}


def test_tune_picks_the_fastest_and_reuses_the_cache(tmp_path, monkeypatch):
    monkeypatch.setenv("NL2D_TUNE_CACHE", str(tmp_path))
    best = (2, 1, 4.0)
    ens = FakeEnsemble([dom(64, 64), dom(100, 300)],
                       lambda c: 1.0 if c == best else 2.0 + c[0] + c[1] + c[2])
    r = autotune.tune(ens)
    assert not r["cached"]
    assert (r["ctas_per_sm"], r["policy"], r["boundary_weight"]) == best
    assert ens.cur == best
    assert len(r["timings"]) == len(autotune.CANDIDATES)
    assert ens.resets == len(autotune.CANDIDATES)

    # same size histogram (order does not matter): applied from the cache
    again = FakeEnsemble([dom(100, 300), dom(64, 64)],
                         lambda c: pytest.fail("a cached schedule was timed again"))
    r2 = autotune.tune(again)
    assert r2["cached"] and again.cur == best


def test_no_cache_times_every_time(tmp_path, monkeypatch):
    monkeypatch.setenv("NL2D_TUNE_CACHE", str(tmp_path))
    calls = []
    ens = FakeEnsemble([dom(32, 32)], lambda c: calls.append(c) or 1.0 + c[1])
    autotune.tune(ens, use_cache=False)
    n = len(calls)
    autotune.tune(ens, use_cache=False)
    assert len(calls) == 2 * n > 0


def test_signature_depends_on_size_bins_and_precision():
    a = [dom(64, 64), dom(100, 300)]
    assert autotune.signature(a) == autotune.signature(list(reversed(a)))
    assert autotune.signature(a) != autotune.signature(a, "mixed")
    assert autotune.signature(a) != autotune.signature([dom(64, 64), dom(600, 300)])
    # sizes bin by powers of two per axis
    assert autotune.signature([dom(64, 64)]) == autotune.signature([dom(70, 100)])
