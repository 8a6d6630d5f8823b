"""CPU tests of the ensemble autotuner's host logic with a stand-in
ensemble: it times every candidate (schedules at the default tile shape,
then every shape under the best schedule; the march's strip heights for the
mixed and FP64-equivalent forms), applies the fastest, leaves the ensemble at rest after each
trial, caches the choice per domain-size signature and reuses it without
timing again."""
import pytest

from psyclonebench_gb300 import autotune


class FakeEnsemble:
    """The calls tune() makes on an Ensemble: schedule, run, reset."""

    def __init__(self, domains, cost):
        self.domains = domains
        self.cost = cost          # ms per step of (cps, policy, weight, tile, march_rows)
        self.cur = None
        self.resets = 0

    def schedule(self, cps, pol, bw, tile=(32, 16), march_rows=32):
        self.cur = (cps, pol, bw, tuple(tile), march_rows)

    def run(self, every, steps):
        return self.cost(self.cur) * steps, None

    def reset(self):
        self.resets += 1


def dom(nx, ny):
    return {"dims": (nx + 2, ny + 2, 1, nx, 1, ny)}


def test_tune_picks_the_fastest_and_reuses_the_cache(tmp_path, monkeypatch):
    monkeypatch.setenv("NL2D_TUNE_CACHE", str(tmp_path))
    best = (2, 1, 4.0, (32, 16), 32)
    ens = FakeEnsemble([dom(64, 64), dom(100, 300)],
                       lambda c: 1.0 if c == best else 2.0 + c[0] + c[1] + c[2])
    r = autotune.tune(ens)
    assert not r["cached"]
    assert (r["ctas_per_sm"], r["policy"], r["boundary_weight"]) == best[:3]
    assert ens.cur == best
    n = len(r["timings"])
    assert n == len(autotune.SCHEDULES) + 2 * (len(autotune.SHAPES) - 1)
    assert ens.resets == n

    # same size histogram (order does not matter): applied from the cache
    again = FakeEnsemble([dom(100, 300), dom(64, 64)],
                         lambda c: pytest.fail("a cached schedule was timed again"))
    r2 = autotune.tune(again)
    assert r2["cached"] and again.cur == best


def test_a_non_default_tile_shape_can_win(tmp_path, monkeypatch):
    """The second stage times every shape under the best schedule and keeps
    a shape other than the default when it is faster."""
    monkeypatch.setenv("NL2D_TUNE_CACHE", str(tmp_path))

    def cost(c):
        base = 1.0 + 0.1 * c[1]  # policy 0 is the best schedule at any shape
        return base * (0.7 if c[3] == (16, 16) else 1.0)
    ens = FakeEnsemble([dom(20, 20)] * 8, cost)
    r = autotune.tune(ens)
    assert tuple(r["tile"]) == (16, 16) and r["policy"] == 0
    assert ens.cur[3] == (16, 16)
    shapes = {tuple(t["tile"]) for t in r["timings"]}
    assert shapes == set(autotune.SHAPES)


def test_mixed_form_searches_the_march_strip(tmp_path, monkeypatch):
    monkeypatch.setenv("NL2D_TUNE_CACHE", str(tmp_path))
    base = {"ctas_per_sm": 1, "policy": 2, "boundary_weight": 0.0, "tile": [64, 8]}
    ens = FakeEnsemble([dom(64, 64)], lambda c: {8: 3.0, 16: 1.0, 32: 2.0, 64: 2.5}[c[4]])
    r = autotune.tune(ens, precision="mixed", base=base)
    assert r["march_rows"] == 16 and len(r["timings"]) == len(autotune.MARCH_ROWS)
    assert ens.cur == (1, 2, 0.0, (64, 8), 16)  # the FP64 knobs are kept


def test_df_form_searches_the_march_strip_and_caches_apart(tmp_path, monkeypatch):
    """The FP64-equivalent form searches the strip height like the mixed
    form, keeps the FP64 knobs, and is cached under its own signature."""
    monkeypatch.setenv("NL2D_TUNE_CACHE", str(tmp_path))
    base = {"ctas_per_sm": 2, "policy": 2, "boundary_weight": 0.0, "tile": [32, 16]}
    ens = FakeEnsemble([dom(64, 64)], lambda c: {8: 3.0, 16: 2.0, 32: 1.5, 64: 1.0}[c[4]])
    r = autotune.tune(ens, precision="df", base=base)
    assert r["march_rows"] == 64 and not r["cached"]
    assert ens.cur == (2, 2, 0.0, (32, 16), 64)
    assert autotune.signature(ens.domains, "df") != autotune.signature(ens.domains, "mixed")
    m = autotune.tune(ens, precision="mixed", base=base)
    assert not m["cached"]  # a df entry does not answer for the mixed form
    assert autotune.tune(ens, precision="df", base=base)["cached"]


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
