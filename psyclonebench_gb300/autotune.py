"""Autotuner for the ensemble's schedule and tile shapes.

The search space is what the ensemble exposes (nl2d_ens_schedule,
nl2d_ens_tile):

* FP64 form: persistent CTAs per SM (1 or 2), tile assignment (contiguous
  cost-balanced chunks, longest processing time first, or one tile per CTA
  left to the hardware block scheduler), the cost weight given to the edge
  cells of boundary tiles (which take the general per-cell path), and the
  tile shape (32 x 16, 32 x 8, 16 x 16, 64 x 8, 32 x 32).  The reference's
  tiled OpenMP layer (psykal_omp/time_step_mod.f90:587-1182) takes its tile
  size as a run parameter; here it is searched.  The search has two stages:
  every schedule at the default shape, then every shape under the best
  schedule and under one-tile-per-CTA.
* Mixed and FP64-equivalent ("df") forms: the column march's strip height
  (8, 16, 32 or 64 rows), under the FP64 knobs already applied.

Each candidate is timed on a few steps of the actual ensemble (after one
untimed step), the domains are put back at rest, and the fastest candidate
is kept.  Results are cached on disk per (domain size histogram, precision),
so a repeated ensemble of the same shape skips the search.  Results do not
depend on any knob: the FP64 form is bit-identical under every one.
"""
import hashlib
import json
import os

# (CTAs per SM, policy, boundary weight); policy 2 (one tile per CTA)
# ignores the CTAs per SM and the edge weight
SCHEDULES = ([(cps, pol, bw) for cps in (1, 2) for pol in (0, 1) for bw in (0.0, 4.0, 16.0)] +
             [(2, 2, 0.0)])
SHAPES = ((32, 16), (32, 8), (16, 16), (64, 8), (32, 32))
DEFAULT_SHAPE = SHAPES[0]
MARCH_ROWS = (8, 16, 32, 64)
DEFAULT_MARCH_ROWS = 32


def cache_path():
    base = os.environ.get("NL2D_TUNE_CACHE") or os.path.join(
        os.environ.get("XDG_CACHE_HOME", os.path.expanduser("~/.cache")), "psyclonebench_gb300")
    return os.path.join(base, "ensemble_schedule.json")


def signature(domains, precision="fp64"):
    """Histogram of interior sizes (log2 bins per axis) plus precision."""
    hist = {}
    for d in domains:
        w, h, xs, xe, ys, ye = d["dims"]
        key = "%d:%d" % ((xe - xs + 1).bit_length(), (ye - ys + 1).bit_length())
        hist[key] = hist.get(key, 0) + 1
    blob = json.dumps([precision, sorted(hist.items())])
    return hashlib.sha1(blob.encode()).hexdigest()[:16]


def _load():
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except Exception:
        return {}


def _store(db):
    p = cache_path()
    try:
        os.makedirs(os.path.dirname(p), exist_ok=True)
        with open(p, "w") as f:
            json.dump(db, f, indent=1)
    except OSError:
        pass


def _apply(ens, c):
    ens.schedule(c["ctas_per_sm"], c["policy"], c["boundary_weight"], tuple(c["tile"]),
                 c["march_rows"])


def _time(ens, c, steps):
    _apply(ens, c)
    ens.run(1, 1)  # untimed: builds the schedule and graph
    ms, _ = ens.run(2, steps)
    ens.reset()
    return ms / steps


def _fp64_candidates(best_schedule=None):
    if best_schedule is None:
        return [{"ctas_per_sm": cps, "policy": pol, "boundary_weight": bw,
                 "tile": list(DEFAULT_SHAPE), "march_rows": DEFAULT_MARCH_ROWS}
                for cps, pol, bw in SCHEDULES]
    out = []
    for shape in SHAPES[1:]:
        for sched in sorted({best_schedule, (2, 2, 0.0)}):
            cps, pol, bw = sched
            out.append({"ctas_per_sm": cps, "policy": pol, "boundary_weight": bw,
                        "tile": list(shape), "march_rows": DEFAULT_MARCH_ROWS})
    return out


def tune(ens, steps=4, precision="fp64", use_cache=True, base=None):
    """Picks and applies the fastest knobs for `ens` in its current form
    (precision "fp64", "mixed" or "df"); returns a dict with the choice and
    the timings.  For "mixed" and "df", `base` holds the FP64 knobs to keep
    (default: the defaults).  Leaves the ensemble at rest."""
    sig = signature(ens.domains, precision)
    db = _load() if use_cache else {}
    if sig in db:
        c = db[sig]
        _apply(ens, c)
        return dict(c, cached=True)
    timings = []
    if precision in ("mixed", "df"):
        b = dict(base or {"ctas_per_sm": 2, "policy": 0, "boundary_weight": 4.0,
                          "tile": list(DEFAULT_SHAPE)})
        for mr in MARCH_ROWS:
            c = {"ctas_per_sm": b["ctas_per_sm"], "policy": b["policy"],
                 "boundary_weight": b["boundary_weight"], "tile": list(b["tile"]),
                 "march_rows": mr}
            timings.append((_time(ens, c, steps), c))
    else:
        for c in _fp64_candidates():
            timings.append((_time(ens, c, steps), c))
        first = min(timings, key=lambda t: t[0])[1]
        sched = (first["ctas_per_sm"], first["policy"], first["boundary_weight"])
        for c in _fp64_candidates(sched):
            timings.append((_time(ens, c, steps), c))
    ms, best = min(timings, key=lambda t: t[0])
    choice = dict(best, ms_per_step=ms,
                  timings=[dict(c, ms_per_step=t) for t, c in timings])
    _apply(ens, best)
    db[sig] = choice
    if use_cache:
        _store(db)
    return dict(choice, cached=False)
