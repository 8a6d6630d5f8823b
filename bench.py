"""Benchmark: NEMOLite2D FP64 time step at 4096 x 4096 interior cells.

`python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]`

A "step" is one NEMOLite2D time step over the whole 4096^2 domain
(namelist jpiglo = jpjglo = 4098, jphgr_msh = 1, dx = dy = 1000 m,
depth 100 m, rdt = 20 s, cbfr = 1.5e-4, visc = 0.1, tide 0.2 m / 12.42 h,
rest start).  The domain does not shard: with N > 1 every rank runs an
independent replica and `value` counts all ranks' cell-steps ("replicas
only").

ours:
  value  Mcell-steps/s over K fused FP64 steps with the state resident in
         HBM: one CUDA-graph launch timed with CUDA events on the library's
         stream.  Every field is larger than L2 (4098 x 4104 FP64 = 135 MB >
         129 MB), and the per-step working set is ~1.3 GB, so no flush is
         needed.
  e2e    the same K steps through the reference-facing C-ABI from HOST
         buffers (initialised by writing them, as the reference's driver
         does, and pinned with nl2d_host_register during set-up):
         c_invoke_time_step per step (the first call uploads all 25
         arrays), then c_read_from_device of sshn_t, un and vn; host wall
         clock around all of it.  `e2e.pageable`: the same from pageable
         arrays.
  roofline  HBM: 76 algorithmic bytes per interior cell-step (read sshn_t,
         un, vn, ht, hu, hv as FP64 + tmask as int32; write sshn_t, un, vn)
         divided by the fused kernel's event time, against the measured HBM
         copy bandwidth.  `fp64` adds the FP64-pipe view of the same kernel.
  cpu_baseline  the CPU reference timed on this host's cores (the
         reference's OpenMP PSy layer where it was compiled here, else the
         oracle's OpenMP port) on a bounded sample of the same domain.
reference:
  the reference's CPU implementation on all host threads, K steps of the
  same domain.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

ALG_BYTES_PER_CELL = 76  # 6 x 8 B read + 4 B mask + 3 x 8 B write
NPTS = 4096


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, default=NPTS, help="interior cells per side")
    ap.add_argument("--state", default="rest", choices=["rest", "active"],
                    help="rest: the reference's start (default); active: every cell in "
                         "motion on a Fourier bathymetry (rdt 5 s)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-forms", action="store_true",
                    help="skip the mixed-precision, ensemble and emulator measurements")
    ap.add_argument("--no-emulator", action="store_true", help="skip the emulator (config 4)")
    ap.add_argument("--forms", default="cfg0,mixed,active,df,sweep,ensemble,tra_adv,emulator",
                    help="comma-separated forms to measure after the headline number")
    ap.add_argument("--form-steps", type=int, default=1000,
                    help="timed steps of the mixed-precision form and its FP64 twin")
    ap.add_argument("--emu-iters", type=int, default=8000, help="emulator training iterations")
    ap.add_argument("--emu-domains", type=int, default=200, help="emulator training domains")
    ap.add_argument("--emu-horizon", type=int, default=5000,
                    help="solver steps of the emulator's trajectories and roll-out")
    ap.add_argument("--case", default=None,
                    choices=["fused", "fused_active", "mixed", "df", "tra_adv", "emu", "rates",
                             "ensemble", "ensemble_mixed", "ensemble_df"],
                    help="run one small case of one kernel family and print its device time "
                         "(for profiler captures; prints no bench line)")
    ap.add_argument("--batch", type=int, default=24, help="--case emu: images of 256^2")
    ap.add_argument("--domains", type=int, default=512,
                    help="--case ensemble*: the first N domains of the 512-domain draw")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def make_problem(n, written=False):
    """The reference's initial state for an n x n interior through the
    library's own set-up (psyclonebench_gb300.model.reference_problem)."""
    from psyclonebench_gb300.model import reference_problem
    return reference_problem(n, written=written)


def make_problem_oracle(n):
    """The same initial state through the oracle's set-up, for the CPU legs:
    they load no library of the product."""
    from oracle import cpu as O
    from psyclonebench_gb300.model import Model
    jp = n + 2
    return O.setup_model(Model(jp, jp, width=((jp + 1 + 7) // 8) * 8))


def bench_config(n, width, rdt, active=False, world=1):
    """The config object both arms print (same keys and values)."""
    return {"workload": "nemolite2d_fp64_%dx%d%s" % (n, n, "_active" if active else ""),
            "interior": [n, n], "jphgr_msh": 1, "rdt": rdt, "width": width,
            "l2": "inputs larger than L2 (135 MB per field)" if n >= 4096 else
                  "working set per step above L2 only from 4096^2",
            "parallelism": "replicas" if world > 1 else "single"}


def make_active(m, seed=3):
    """Puts every cell of m in motion: the seeded Fourier bathymetry
    (50-500 m, rdt 5 s) and a random start, sea-surface height within
    +-0.1 m and velocities within +-0.05 m/s everywhere.  From rest the tide
    enters through the open south row only, so within a few hundred steps
    most cells still hold zeros; here (almost) no operand is zero."""
    from psyclonebench_gb300.workloads import fourier_depth
    ht, hu, hv = fourier_depth(m.width, m.height, seed)
    m.f["ht"][:], m.f["hu"][:], m.f["hv"][:] = ht, hu, hv
    rng = np.random.default_rng(seed)
    for k, a in (("sshn_t", 0.1), ("un", 0.05), ("vn", 0.05)):
        m.f[k][:] = rng.uniform(-a, a, size=m.f[k].shape)
    m.rdt = BATHY_RDT
    return m


def peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi samples (every 200 ms) while the timed region runs."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.rows = []
        self.gpu = gpu_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for k, nm in enumerate(names):
                if len(r) > 4 + k and r[4 + k].lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def load_profile_figures():
    """DRAM bytes and FP64 thread-instructions per cell of the fused kernel,
    per start state ("rest", "active"), from the committed ncu summary."""
    p = os.path.join(REPO, "profiles", "fused_fp64_step.json")
    try:
        with open(p) as f:
            return json.load(f)
    except Exception:
        return {}


def time_cpu(m, nsteps, fn, target_s=None, istep0=1):
    """Times CPU steps of one step function; if target_s is given, runs
    until ~target_s seconds (at least one step).  Returns (steps, seconds)."""
    from oracle import cpu as O
    done, t0 = 0, time.perf_counter()
    while True:
        O.call_step(fn, m.step_args(istep0 + done))
        done += 1
        el = time.perf_counter() - t0
        if target_s is None and done >= nsteps:
            break
        if target_s is not None and (el >= target_s or done >= nsteps):
            break
    return done, time.perf_counter() - t0


def time_cpu_layers(n, nsteps, warmup, target_s):
    """The reference's two OpenMP PSy layers (time_step_omp.cpp, worksharing;
    time_step_ompopt.cpp, partially fused) on the n x n domain from rest,
    each after `warmup` untimed steps: the reference's own builds where
    oracle/_ref holds them, else the oracle's ports.  Returns the faster
    one's (Mcell-steps/s, steps, seconds, kind, description) and every
    layer's rate."""
    from oracle import cpu as O
    best, rates = None, {}
    for fn, kind, desc in O.cpu_step_fns():
        m = make_problem_oracle(n)
        time_cpu(m, max(warmup, 1), fn)
        steps, secs = time_cpu(m, nsteps, fn, target_s=target_s, istep0=1 + max(warmup, 1))
        val = n * n * steps / secs / 1e6
        rates[desc] = val
        if best is None or val > best[0]:
            best = (val, steps, secs, kind, desc)
        del m
    return best, rates


SEQ_SAMPLE = 32  # domains timed one at a time for the ensemble comparison
BATHY_RDT = 5.0  # s, for the 50-500 m bathymetry configurations
MIXED_BYTES_PER_CELL = 48  # read ssh pair 8 + un 4 + vn 4 + ht/hu/hv 12 + mask 4; write 16


def measure_form(lib, n, precision, steps, warmup, seed=2):
    """Config 2: the 4096^2 domain on a seeded Fourier bathymetry, advanced
    warmup + steps steps in one precision; returns (ms per timed step,
    final fields)."""
    import psyclonebench_gb300 as P
    from psyclonebench_gb300.model import register
    from psyclonebench_gb300.workloads import fourier_depth
    m = make_problem(n)
    ht, hu, hv = fourier_depth(m.width, m.height, seed)
    m.f["ht"][:], m.f["hu"][:], m.f["hv"][:] = ht, hu, hv
    # 500 m deep water carries gravity waves at sqrt(g h) = 70 m/s: the
    # explicit step needs rdt well below dx / 70 m/s = 14 s.
    m.rdt = BATHY_RDT
    register(lib, m)
    lib.nl2d_set_precision(precision)
    ms = ctypes.c_double(0.0)
    P.check(lib.nl2d_timed_run(1, warmup, ctypes.byref(ms)), "form warm-up")
    P.check(lib.nl2d_timed_run(1 + warmup, steps, ctypes.byref(ms)), "form run")
    out = {}
    for k in ("sshn_t", "un", "vn"):
        a = m.f[k]
        lib.c_read_from_device(a.ctypes.data, a.ctypes.data, 1, 1, m.width, m.height, True)
        x0, x1, y0, y1 = m.regions()["t" if k == "sshn_t" else ("u" if k == "un" else "v")]
        out[k] = a[y0:y1 + 1, x0:x1 + 1].copy()
    P.check(None, "form read")
    lib.nl2d_set_precision(0)
    lib.nl2d_finalize()
    return ms.value / steps, out


def run_forms(lib, n, steps=1000, warmup=3):
    fp64_ms, ref = measure_form(lib, n, 0, steps, warmup)
    mix_ms, mix = measure_form(lib, n, 1, steps, warmup)
    cells = n * n
    hbm, _ = peaks()
    err = {}
    for k, name in (("sshn_t", "ssh"), ("un", "u"), ("vn", "v")):
        d = mix[k] - ref[k]
        err[name] = {"rms": float(np.sqrt(np.mean(d * d))), "max": float(np.abs(d).max()),
                     "field_max": float(np.abs(ref[k]).max())}
    ach = MIXED_BYTES_PER_CELL * cells / (mix_ms * 1e-3) / 1e9
    return {"mixed": {
        "workload": "nemolite2d_mixed_%dx%d_fourier_bathymetry_seed2_rdt5_%d_steps" % (
            n, n, steps + warmup),
        "value": cells / (mix_ms * 1e-3) / 1e6, "unit": "Mcell-steps/s",
        "fp64_value_same_inputs": cells / (fp64_ms * 1e-3) / 1e6,
        "speedup_vs_fp64": fp64_ms / mix_ms,
        "roofline": {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s",
                     "frac": ach / hbm, "alg_bytes_per_cell": MIXED_BYTES_PER_CELL},
        "error_vs_fp64": err, "dtype": "f32 + compensated-f32 ssh"}}


def run_active(lib, n, rest_value, steps=200, warmup=5):
    """The FP64 step with every cell in motion (make_active): the same
    kernel and timing as the headline number, on a state where the exact
    division's zero-dividend shortcut (almost) never applies."""
    import psyclonebench_gb300 as P
    from psyclonebench_gb300.model import dptr, register
    m = make_active(make_problem(n))
    register(lib, m)
    ms = ctypes.c_double(0.0)
    P.check(lib.nl2d_timed_run(1, warmup, ctypes.byref(ms)), "active warm-up")
    P.check(lib.nl2d_timed_run(1 + warmup, steps, ctypes.byref(ms)), "active run")
    sums = np.zeros(3)
    P.check(lib.nl2d_checksums(dptr(sums)), "active checksums")
    lib.nl2d_finalize()
    value = n * n * steps / (ms.value * 1e-3) / 1e6
    return {"workload": "nemolite2d_fp64_%dx%d_active_fourier_bathymetry_seed3_rdt5" % (n, n),
            "value": value, "unit": "Mcell-steps/s", "ms_per_step": ms.value / steps,
            "steps": steps, "warmup": warmup, "ratio_to_rest_start": value / rest_value,
            "checksums": {"ssh": sums[0], "u": sums[1], "v": sums[2]}, "dtype": "f64"}


def run_df_form(lib, n, steps=200, warmup=5):
    """The FP64-equivalent form (double-float interior, exact FP64 elsewhere)
    at the headline workload (n x n from rest) and with every cell in motion
    (make_active): device-resident rate, and each field's relative L2
    difference to the bitwise FP64 path after the same warmup + steps
    steps (the FP64-equivalent contract: 1e-10 per field)."""
    import psyclonebench_gb300 as P
    from psyclonebench_gb300.model import read_fields, register
    cells = n * n
    hbm, _ = peaks()
    out = {}
    for state in ("rest", "active"):
        res = {}
        for precision in (0, 2):
            m = make_problem(n)
            if state == "active":
                make_active(m)
            register(lib, m)
            lib.nl2d_set_precision(precision)
            ms = ctypes.c_double(0.0)
            P.check(lib.nl2d_timed_run(1, warmup, ctypes.byref(ms)), "df warm-up")
            P.check(lib.nl2d_timed_run(1 + warmup, steps, ctypes.byref(ms)), "df run")
            lib.nl2d_set_precision(0)
            read_fields(lib, m, ("sshn_t", "un", "vn"))
            lib.nl2d_finalize()
            res[precision] = (ms.value / steps, {k: m.f[k].copy() for k in ("sshn_t", "un", "vn")})
            del m
        ms64, f64 = res[0]
        msdf, fdf = res[2]
        rel = {}
        for k in ("sshn_t", "un", "vn"):
            a, b = fdf[k], f64[k]
            den = float(np.sqrt(np.sum(b * b)))
            rel[k] = float(np.sqrt(np.sum((a - b) ** 2))) / den if den > 0 else 0.0
        ach = ALG_BYTES_PER_CELL * cells / (msdf * 1e-3) / 1e9
        out[state] = {
            "value": cells / (msdf * 1e-3) / 1e6, "unit": "Mcell-steps/s",
            "ms_per_step": msdf, "fp64_value_same_inputs": cells / (ms64 * 1e-3) / 1e6,
            "speedup_vs_fp64": ms64 / msdf, "steps": steps + warmup,
            "rel_l2_vs_fp64": rel,
            "roofline": {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s",
                         "frac": ach / hbm, "alg_bytes_per_cell": ALG_BYTES_PER_CELL,
                         # what the march moves per cell it writes: the FP64
                         # state in and out plus five double-float statics
                         # and a flag byte (89.0 B measured by ncu at 2048^2)
                         "march_bytes_per_cell": 89}}
    return {"workload": "nemolite2d_fp64_equivalent_%dx%d" % (n, n),
            "dtype": "double-float (FP32 pairs) interior, FP64 boundary cells and storage",
            "bar": "relative L2 <= 1e-10 per field against the FP64 path", **out}


def run_cfg0(lib, nsteps=2000, every=100):
    """Config 0, the parity namelist (128^2 interior, rest start, 2000
    steps): on the GPU as one captured graph of fused steps (CUDA events,
    nl2d_timed_run), then again through nl2d_run_steps with the ssh / u / v
    checksums every 100 steps in the graph; on one host core through the
    serial step (the reference's own serial build where oracle/_ref holds
    it, else the oracle's restatement) from the same start, its checksums at
    the same steps beside the GPU's."""
    import psyclonebench_gb300 as P
    from psyclonebench_gb300.model import dptr, register
    from oracle import cpu as O
    n = 128
    out = {"workload": "nemolite2d_cfg0_128x128_%d_steps" % nsteps, "unit": "Mcell-steps/s"}
    m = make_problem(n)
    register(lib, m)
    ms = ctypes.c_double(0.0)
    P.check(lib.nl2d_timed_run(1, nsteps, ctypes.byref(ms)), "cfg0 warm-up")
    lib.nl2d_finalize()
    m = make_problem(n)
    register(lib, m)
    P.check(lib.nl2d_timed_run(1, nsteps, ctypes.byref(ms)), "cfg0 run")
    out["gpu"] = {"value": n * n * nsteps / (ms.value * 1e-3) / 1e6, "ms": ms.value}
    lib.nl2d_finalize()
    m = make_problem(n)
    register(lib, m)
    sums = np.zeros(3 * (nsteps // every))
    P.check(lib.nl2d_run_steps(1, nsteps, every, dptr(sums)), "cfg0 checksums")
    lib.nl2d_finalize()
    ref = O.load_ref("serial")
    fn, kind = ((ref.c_invoke_time_step, "reference") if ref is not None else
                (O.load_oracle().oracle_invoke_time_step, "port"))
    o = O.load_oracle()
    c = make_problem_oracle(n)
    cpu_sums, t0 = [], time.perf_counter()
    for k in range(nsteps):
        O.call_step(fn, c.step_args(1 + k))
        if (k + 1) % every == 0:
            r = c.regions()
            cpu_sums.append([o.oracle_field_checksum(dptr(c.f[f]), c.width, *r[kk])
                             for f, kk in (("sshn_t", "t"), ("un", "u"), ("vn", "v"))])
    secs = time.perf_counter() - t0
    out["cpu_serial"] = {"value": n * n * nsteps / secs / 1e6, "seconds": secs, "cores": 1,
                         "kind": kind,
                         "sample": "the full %d steps, checksums every %d included" %
                                   (nsteps, every)}
    got = sums.reshape(-1, 3)
    want = np.array(cpu_sums)
    out["checksums_max_rel_diff"] = float(np.max(np.abs(got - want) /
                                                 np.maximum(np.abs(want), 1e-300)))
    out["speedup_gpu_vs_cpu_serial"] = out["gpu"]["value"] / out["cpu_serial"]["value"]
    return out


def run_sweep(lib, sizes=(256, 512, 1024, 2048, 4096, 8192)):
    """Config 1's sweep of interior sizes (the reference's
    scripts/problemsize.sh:15-22 edits the namelist's jpiglo / jpjglo): the
    FP64 step and the mixed form at each size, device-resident, from the
    reference's rest start, with about the same number of cell-steps per
    size."""
    import psyclonebench_gb300 as P
    from psyclonebench_gb300.model import register
    out = []
    for n in sizes:
        m = make_problem(n)
        register(lib, m)
        steps = max(20, min(400, int(2e9 / (n * n))))
        ms = ctypes.c_double(0.0)
        P.check(lib.nl2d_timed_run(1, 5, ctypes.byref(ms)), "sweep warm-up")
        P.check(lib.nl2d_timed_run(6, steps, ctypes.byref(ms)), "sweep fp64")
        fp64 = n * n * steps / (ms.value * 1e-3) / 1e6
        lib.nl2d_set_precision(1)
        P.check(lib.nl2d_timed_run(6 + steps, 5, ctypes.byref(ms)), "sweep mixed warm-up")
        P.check(lib.nl2d_timed_run(11 + steps, steps, ctypes.byref(ms)), "sweep mixed")
        mixed = n * n * steps / (ms.value * 1e-3) / 1e6
        lib.nl2d_set_precision(0)
        lib.nl2d_finalize()
        del m
        out.append({"interior": n, "steps": steps, "fp64": fp64, "mixed": mixed})
    return {"unit": "Mcell-steps/s", "sizes": out}


def run_ensemble(lib, steps=20, ndom=512, seed=7, rank=0, world=1):
    """Config 3: 512 seeded domains (log-uniform 64..1024 per axis, Fourier
    bathymetry 50-500 m, tide 0.05-0.5 m / 10-14 h, random open side), one
    persistent launch per step; with N ranks each takes a cell-balanced
    shard of whole domains (weak scaling, no collective)."""
    from psyclonebench_gb300 import autotune
    from psyclonebench_gb300.ensemble import Ensemble, build_domain, shard_domains
    from psyclonebench_gb300.workloads import ensemble_domains
    specs = ensemble_domains(ndom, seed)
    mine = shard_domains(specs, world)[rank] if world > 1 else list(range(ndom))
    doms = [build_domain(specs[k]) for k in mine]
    ens = Ensemble(doms, lib=lib)
    tune = autotune.tune(ens, steps=3)
    ens.run(1, 1)
    ms, _ = ens.run(2, steps)
    cells, ntiles, nctas = ens.info()
    ens.set_precision(1)
    tune_mixed = autotune.tune(ens, steps=3, precision="mixed", base=tune)
    ens.run(1, 1)
    ms_mix, _ = ens.run(2, steps)
    # the FP64-equivalent form (FP64 state, double-float interior)
    ens.set_precision(2)
    tune_df = autotune.tune(ens, steps=3, precision="df", base=tune)
    ens.run(1, 1)
    ms_df, _ = ens.run(2, steps)
    ens.close()
    # The same domains one at a time through the single-domain FP64 path (a
    # sample of SEQ_SAMPLE domains, each timed as one graph launch of
    # `steps` fused steps): what running the ensemble without the
    # persistent kernel costs.
    seq_ms, seq_cells = 0.0, 0
    import psyclonebench_gb300 as P
    from psyclonebench_gb300 import workloads as W
    from psyclonebench_gb300.model import Model, register
    sample = doms[:SEQ_SAMPLE]
    for d in sample:
        w, h, xs, xe, ys, ye = d["dims"]
        m = Model.from_extents(w, h, xs, xe, ys, ye).uniform_metrics()
        m.grid["tmask"][:] = np.ascontiguousarray(d["tmask"], np.int32)
        m.f["ht"][:], m.f["hu"][:], m.f["hv"][:] = d["ht"], d["hu"], d["hv"]
        m.rdt, m.cbfr, m.visc = W.ENSEMBLE_RDT, W.ENSEMBLE_CBFR, W.ENSEMBLE_VISC
        register(lib, m)
        t = ctypes.c_double(0.0)
        P.check(lib.nl2d_timed_run(1, 2, ctypes.byref(t)), "seq warm-up")
        P.check(lib.nl2d_timed_run(3, steps, ctypes.byref(t)), "seq run")
        seq_ms += t.value
        seq_cells += (xe - xs + 1) * (ye - ys + 1)
    lib.nl2d_finalize()
    ens_s = Ensemble(sample, lib=lib)
    ens_s.schedule(tune["ctas_per_sm"], tune["policy"], tune["boundary_weight"],
                   tuple(tune["tile"]), tune["march_rows"])
    ens_s.run(1, 1)
    ms_s, _ = ens_s.run(2, steps)
    ens_s.close()
    return {"workload": "nemolite2d_ensemble_%d_domains_seed%d_rdt5" % (ndom, seed),
            "domains_this_rank": len(mine), "cells_this_rank": cells, "tiles": ntiles,
            "persistent_ctas": nctas, "steps": steps,
            "fp64": {"ms_per_step": ms / steps, "value": cells / (ms / steps * 1e-3) / 1e6},
            "mixed": {"ms_per_step": ms_mix / steps,
                      "value": cells / (ms_mix / steps * 1e-3) / 1e6},
            "fp64_equivalent": {"ms_per_step": ms_df / steps,
                                "value": cells / (ms_df / steps * 1e-3) / 1e6,
                                "march_rows": tune_df["march_rows"],
                                "march_timings_ms": [
                                    (t["march_rows"], round(t["ms_per_step"], 4))
                                    for t in tune_df.get("timings", [])]},
            "unit": "Mcell-steps/s",
            "one_domain_at_a_time_fp64": {
                "sample_domains": len(sample), "sample_cells": seq_cells,
                "value": seq_cells / (seq_ms / steps * 1e-3) / 1e6,
                "persistent_value_same_sample": seq_cells / (ms_s / steps * 1e-3) / 1e6,
                "speedup_persistent_vs_sequential": seq_ms / ms_s},
            "schedule": {k: tune[k] for k in ("ctas_per_sm", "policy", "boundary_weight",
                                              "tile", "cached")},
            "schedule_timings_ms": [(t["ctas_per_sm"], t["policy"], t["boundary_weight"],
                                     t["tile"], round(t["ms_per_step"], 4))
                                    for t in tune.get("timings", [])],
            "mixed_march_rows": tune_mixed["march_rows"],
            "mixed_march_timings_ms": [(t["march_rows"], round(t["ms_per_step"], 4))
                                       for t in tune_mixed.get("timings", [])]}


def run_emulator(lib, count=200, horizon=5000, iters=8000, seed=11):
    """Config 4: the learned emulator.  Mixed-precision ensemble
    trajectories of `count` domains of 256^2 cells over `horizon` steps from
    rest, kept only where the solver itself stays finite; 100 (state, state + 10 steps)
    pairs per domain spread over the horizon (20000 for 200 domains); the
    6-layer 48-channel network trains on 90 % of the domains (tcgen05
    forward and backward).  Reported: the one-step ssh error against
    persistence on the held-out domains and on a fresh test set (FP64
    trajectories), the inference throughput in solver-equivalent cell-steps
    against the FP64 and the mixed-precision solvers on domains of the same
    size, and a hybrid roll-out of 16 test domains
    over the whole horizon judged by the FP64 solver every 50 emulator
    steps (window redone by the solver above 1 mm ssh RMS)."""
    import torch
    from psyclonebench_gb300 import emulator as E
    nsnap = horizon // E.K_STEPS + 1
    t0 = time.perf_counter()
    ds = E.Dataset(count=count, nsnap=nsnap, seed=seed, n=256, lib=lib, pairs_per_domain=100)
    gen_s = time.perf_counter() - t0
    nhold = max(2, count // 10)
    hold = list(range(count - nhold, count))
    net = E.ConvNet(16, 256, 256, lib=lib)
    t0 = time.perf_counter()
    hist = E.train(ds, net, iters=iters, holdout=nhold, pushforward=0.5, max_unroll=2,
                   noise_frac=E.TRAIN_NOISE)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    probe_snaps = sorted(set([1, 5] + [int(v) for v in np.linspace(10, nsnap - 2, 8)]))
    err_net, err_pers = E.evaluate(ds, net, hold, probe_snaps)
    # inference: one emulator step (k = 10 solver steps) of 16 domains
    P_ = 16 * 256 * 256
    x = torch.zeros(P_, E.CPAD_IN, dtype=torch.bfloat16, device="cuda")
    ds.batch([(hold[q % nhold], 5) for q in range(16)], x, None)
    for _ in range(3):
        net.forward(x)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record()
    reps = 50
    for _ in range(reps):
        net.forward(x)
    ev1.record()
    torch.cuda.synchronize()
    fwd_ms = ev0.elapsed_time(ev1) / reps
    flops = 2 * 9 * sum(ci * co for ci, co, _ in E.LAYERS) * P_
    emu_value = P_ * E.K_STEPS / (fwd_ms * 1e-3) / 1e6
    # a fresh test set (another seed, normalised as the training data), all
    # its domains finite over the horizon
    test = E.Dataset(count=16, nsnap=nsnap, seed=seed + 1000, n=256, lib=lib, scales_from=ds,
                     solver="fp64")
    t_net, t_pers = E.evaluate(test, net, list(range(16)), probe_snaps)
    # the network on its own over the whole horizon (no judge), then the
    # judged hybrid
    free = E.rollout(test, net, range(16), start_snap=0, emu_steps=nsnap - 1, judge_every=50,
                     threshold=1e-3, judge_share=0.0, track_truth=True)
    roll = E.rollout(test, net, range(16), start_snap=0, emu_steps=nsnap - 1, judge_every=50,
                     threshold=1e-3, judge_share=0.5)
    return {
        "workload": "nemolite2d_emulator_%d_domains_256x256_%d_pairs_k10_horizon%d" % (
            count, count * len(ds.pair_starts), horizon),
        "candidates_generated": ds.candidates, "dropped_unstable_in_solver": len(ds.dropped),
        "data_generation_s": gen_s,
        "train": {"iterations": iters, "batch": 16, "seconds": train_s,
                  "ms_per_step": train_s / iters * 1e3,
                  "loss_first": hist[0], "loss_last100": sum(hist[-100:]) / 100},
        "held_out_one_step_ssh_rms_m": {"domains": nhold, "snapshots": probe_snaps,
                                        "network": err_net, "persistence": err_pers,
                                        "gain": err_pers / err_net},
        "test_set_one_step_ssh_rms_m": {"domains": 16, "network": t_net,
                                        "persistence": t_pers, "gain": t_pers / t_net},
        "inference": {"forward_ms_16x256x256": fwd_ms,
                      "tflops": flops / (fwd_ms * 1e-3) / 1e12,
                      "value": emu_value, "unit": "solver-equivalent Mcell-steps/s",
                      "fp64_solver_same_size_domains": test.solver_mcells,
                      "speedup_vs_fp64_solver": emu_value / test.solver_mcells,
                      "mixed_solver_same_size_domains": ds.solver_mcells,
                      "speedup_vs_mixed_solver": emu_value / ds.solver_mcells},
        "free_running": {k: free[k] for k in ("final_ssh_rms_error_m",
                                                 "final_ssh_rms_error_worst_domain_m",
                                                 "final_ssh_rms_m", "final_nonfinite",
                                                 "emulator_ms", "solver_only_ms",
                                                 "window_errors_m", "window_mean_offsets_m")},
        "train_input_noise": E.TRAIN_NOISE,
        "rollout": roll,
    }


def run_tra_adv(lib, jpi=512, jpj=512, jpk=75, iters=500, cpu_iters=10):
    """The tracer-advection benchmark (benchmarks/nemo/tracer_advection) at
    the largest size of the reference's problem-size sweep
    (scripts/problemsize.sh: JPI = JPJ = 512, JPK = 75, IT = 500), from the
    benchmark's own initial values.  value: Mpoint-iterations/s of `iters`
    iterations on the device-resident state (CUDA events); e2e: the same
    iterations through tra_adv_compute from host arrays, with the upload of
    the first call and the final read-back; roofline: 72 algorithmic bytes
    per point-iteration (read mydomain, pun, pvn, pwn, umask, vmask, tmask
    and the precomputed zind; write mydomain); cpu_baseline: the oracle's
    OpenMP port on all host cores for `cpu_iters` iterations."""
    from psyclonebench_gb300.workloads import tra_adv_fields
    f = tra_adv_fields(jpi, jpj, jpk)
    D = ctypes.POINTER(ctypes.c_double)

    def p(a):
        return a.ctypes.data_as(D)

    args = [p(f[n]) for n in ("ztfreez", "pun", "pvn", "pwn", "umask", "vmask", "tmask",
                              "rnfmsk", "rnfmsk_z", "upsmsk", "mydomain", "tsn")] + \
        [jpi, jpj, jpk]
    points = jpi * jpj * jpk
    # e2e: host arrays in, result out
    t0 = time.perf_counter()
    for _ in range(iters):
        lib.tra_adv_compute(*args)
    out = np.empty_like(f["mydomain"])
    rc = lib.tra_adv_read(p(out))
    e2e_s = time.perf_counter() - t0
    buf = ctypes.create_string_buffer(256)
    if rc != 0 or lib.tra_adv_last_error(buf, 256) != 0:
        raise RuntimeError("tra_adv failed: %s" % buf.value.decode())
    csum = ctypes.c_double(0.0)
    lib.tra_adv_checksum(ctypes.byref(csum))
    # value: resident state, after warm-up
    ms = ctypes.c_double(0.0)
    lib.tra_adv_run(3, ctypes.byref(ms))
    lib.tra_adv_run(iters, ctypes.byref(ms))
    lib.tra_adv_finalize()
    value = points * iters / (ms.value * 1e-3) / 1e6
    hbm, peak_kind = peaks()
    ach = 72.0 * points * iters / (ms.value * 1e-3) / 1e9
    in_bytes = sum(f[n].nbytes for n in f)
    # CPU: the oracle's OpenMP port on a bounded sample of the same workload
    from oracle import cpu as O
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count()))
    lib_o = O.load_oracle()
    g = {n: v.copy() for n, v in f.items()}
    w = O.tra_zero_work(g["mydomain"].shape)
    t0 = time.perf_counter()
    O.tra_oracle_run(lib_o, g, w, cpu_iters, omp=True)
    cpu_s = time.perf_counter() - t0
    return {
        "workload": "tra_adv_%dx%dx%d_%d_iterations" % (jpi, jpj, jpk, iters),
        "metric": "Mpoint-iterations/s", "value": value, "ms_per_iteration": ms.value / iters,
        "checksum_after_first_run": csum.value,
        "e2e": {"value": points * iters / e2e_s / 1e6, "unit": "Mpoint-iterations/s",
                "h2d_bytes_per_step": in_bytes / iters,
                "d2h_bytes_per_step": out.nbytes / iters, "seconds": e2e_s},
        "roofline": {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s",
                     "frac": ach / hbm, "peak_kind": peak_kind,
                     "alg_bytes_per_point": 72,
                     "kernels": ["k_tra_horizontal_tiled", "k_tra_vertical"]},
        "cpu_baseline": {"value": points * cpu_iters / cpu_s / 1e6,
                         "unit": "Mpoint-iterations/s",
                         "cores": int(os.environ["OMP_NUM_THREADS"]), "kind": "port",
                         "sample": "%d iterations of the same domain (oracle OpenMP port)" %
                                   cpu_iters},
        "dtype": "f64",
        # bitwise against the oracle's restatement of tra_adv.F90, which no
        # reference build checks here (no Fortran compiler)
        "parity": "unpinned",
    }


def run_reference(args, rank, world):
    """The reference arm: the reference's CPU implementation of the step on
    all host cores, K steps of the same domain after W warm-up steps, built
    with the oracle's set-up (no library of the product is loaded).  Both
    OpenMP PSy layers run; the faster one is the line's value."""
    if rank != 0:
        return
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count()))
    n = args.size
    best, rates = time_cpu_layers(n, args.steps, args.warmup, target_s=90.0)
    val, steps, secs, kind, desc = best
    width = ((n + 3 + 7) // 8) * 8
    line = {
        "metric": "Mcell-steps/s", "value": val, "unit": "Mcell-steps/s",
        "impl": "reference", "n_gpus": args.gpus, "steps": steps, "warmup": args.warmup,
        "ms_per_step": secs / steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (reference initial state: rest, constant depth)",
        "config": bench_config(n, width, 20.0, world=world),
        "cpu_baseline": {"value": val, "unit": "Mcell-steps/s", "cores": cores,
                         "kind": kind, "sample": "%d steps of the %dx%d domain (%s)" % (
                             steps, n, n, desc),
                         "layers": rates},
        "e2e": {"value": val, "unit": "Mcell-steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def page_aligned_copy(a, page=4096):
    """A copy of array a in a buffer of its own that starts on a page and
    ends on one."""
    nb = -(-a.nbytes // page) * page
    raw = np.empty(nb + page, np.uint8)
    off = (-raw.ctypes.data) % page
    out = raw[off:off + a.nbytes].view(a.dtype).reshape(a.shape)
    out[...] = a
    return out


def run_e2e(lib, n, steps, active, world, pinned=True):
    """The K steps through the reference-facing C-ABI from HOST buffers,
    initialised by writing them as the reference's driver does: the first
    c_invoke_time_step uploads all 25 arrays, every call takes one step, then
    c_read_from_device brings sshn_t, un and vn back; host wall clock around
    all of it.  pinned: the arrays are page-locked first with
    nl2d_host_register (set-up, outside the timed region), so the copies run
    from pinned memory; otherwise they are pageable numpy arrays."""
    import psyclonebench_gb300 as P
    import torch
    m = make_problem(n, written=True)
    if active:
        make_active(m)
    held = []
    try:
        if pinned:
            # page-aligned copies whose pages no other array shares (pinning
            # works on whole pages)
            for d in (m.f, m.grid):
                for k in d:
                    d[k] = page_aligned_copy(d[k])
            for a in list(m.f.values()) + list(m.grid.values()):
                P.check(lib.nl2d_host_register(a.ctypes.data, a.nbytes), "host register")
                held.append(a)
        spec0 = (ctypes.c_int * 2)()
        P.check(lib.nl2d_speculation_counts(spec0), "speculation counts")
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        lib.c_invoke_time_step(*m.step_args(1))
        first_path = lib.nl2d_last_path()
        t1 = time.perf_counter()
        for k in range(1, steps):
            lib.c_invoke_time_step(*m.step_args(1 + k))
        lib.nl2d_sync()
        t2 = time.perf_counter()
        for k in ("sshn_t", "un", "vn"):
            a = m.f[k]
            lib.c_read_from_device(a.ctypes.data, a.ctypes.data, 1, 1, m.width, m.height, True)
        P.check(None, "e2e")
        secs = time.perf_counter() - t0
        # the bytes the library copied (the 25 arrays at registration, the
        # three fields read back)
        moved = (ctypes.c_longlong * 2)()
        P.check(lib.nl2d_transfer_bytes(moved), "transfer bytes")
        spec1 = (ctypes.c_int * 2)()
        P.check(lib.nl2d_speculation_counts(spec1), "speculation counts")
        lib.nl2d_finalize()
    finally:
        for a in held:
            lib.nl2d_host_unregister(a.ctypes.data)
    return {"value": n * n * steps * world / secs / 1e6, "unit": "Mcell-steps/s",
            "h2d_bytes_per_step": moved[0] / steps,
            "d2h_bytes_per_step": moved[1] / steps,
            "host_memory": "pinned (nl2d_host_register at set-up)" if pinned else "pageable",
            "first_step_path": {1: "reference-structured", 2: "fused"}.get(first_path),
            "seconds": secs, "first_call_s": t1 - t0, "read_back_s": secs - (t2 - t0),
            # pinned arrays: the first steps run while the other arrays and
            # the registration checks follow; how those checks ended
            "speculation": {"kept": spec1[0] - spec0[0], "redone": spec1[1] - spec0[1]}}


def run_ours(args, rank, world, local):
    import psyclonebench_gb300 as P
    import torch
    import torch.distributed as dist
    from psyclonebench_gb300.model import dptr, register

    if world > 1:
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    lib = P.load_library()
    n = args.size
    cells = n * n

    # ---- value: resident state, one graph launch of K fused steps ----
    active = args.state == "active"
    m = make_problem(n)
    if active:
        make_active(m)
    register(lib, m)
    ms = ctypes.c_double(0.0)
    P.check(lib.nl2d_timed_run(1, 1 + args.warmup, ctypes.byref(ms)), "warm-up")
    istep = 2 + args.warmup
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        P.check(lib.nl2d_timed_run(istep, args.steps, ctypes.byref(ms)), "timed run")
    torch.cuda.synchronize()
    kernel_ms = ms.value
    if world > 1:
        t = torch.tensor([kernel_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        kernel_ms = float(t.item())
    sums = np.zeros(3)
    P.check(lib.nl2d_checksums(dptr(sums)), "checksums")
    value = cells * args.steps * world / (kernel_ms * 1e-3) / 1e6
    ms_step = kernel_ms / args.steps
    lib.nl2d_finalize()

    # ---- e2e: host buffers through c_invoke_time_step ----
    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(lib, n, args.steps, active, world, pinned=True)
        e2e["pageable"] = {k: v for k, v in
                           run_e2e(lib, n, args.steps, active, world, pinned=False).items()
                           if k in ("value", "seconds", "first_call_s", "read_back_s")}

    hbm, peak_kind = peaks()
    prof = load_profile_figures()
    fig = prof.get("states", {}).get(args.state, {})
    achieved = ALG_BYTES_PER_CELL * cells / (ms_step * 1e-3) / 1e9
    traffic = fig.get("dram_bytes_per_cell")
    roof = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
            "frac": achieved / hbm, "peak_kind": peak_kind,
            "traffic": traffic * cells if traffic else None,
            "traffic_bytes_per_cell": traffic,
            "traffic_capture": fig.get("traffic_capture"),
            "kernel": "k_fused_step", "alg_bytes_per_cell": ALG_BYTES_PER_CELL}
    if fig.get("fp64_ops_per_cell"):
        # FP64 thread-instructions per cell from the ncu capture of the same
        # start state (the count depends on it: zero dividends skip the
        # division's FP64 work)
        gops = fig["fp64_ops_per_cell"] * cells / (ms_step * 1e-3) / 1e9
        # the FP64 pipe's rate measured on this GPU now (best of FMA,
        # multiply and add streams)
        rates = (ctypes.c_double * 4)()
        P.check(lib.nl2d_measure_pipe_rates(rates), "pipe rates")
        peak = max(rates[0], rates[1], rates[2])
        roof["fp64"] = {
            "achieved_gops": gops, "ops_per_cell": fig["fp64_ops_per_cell"],
            "peak_gops": peak, "peak_kind": "measured in this run (nl2d_measure_pipe_rates)",
            "frac": gops / peak if peak else None,
            "pipe_rates_gops": {"dfma": rates[0], "dmul": rates[1], "dadd": rates[2],
                                "ffma": rates[3]},
            "profile": fig.get("source"),
        }

    forms = None
    want = set(args.forms.split(","))
    if "emulator" in want and args.no_emulator:
        want.discard("emulator")
    if rank == 0 and not args.no_forms:
        forms = {}
        if "cfg0" in want:
            forms["cfg0"] = run_cfg0(lib)
        if "mixed" in want:
            forms.update(run_forms(lib, n, steps=args.form_steps))
        if "active" in want:
            forms["fp64_active"] = run_active(lib, n, value)
        if "df" in want:
            forms["fp64_equivalent"] = run_df_form(lib, n)
        if "sweep" in want:
            forms["size_sweep"] = run_sweep(lib)
        if "ensemble" in want:
            ens = run_ensemble(lib)
            for form in ("fp64", "mixed", "fp64_equivalent"):
                ens[form]["speedup_vs_single_4096_domain_fp64"] = ens[form]["value"] / value
            # every ensemble domain is in motion: the like-for-like single-
            # domain rate is the one with every cell active
            act = (forms.get("fp64_active") or {}).get("value")
            if act:
                for form in ("fp64", "mixed", "fp64_equivalent"):
                    ens[form]["speedup_vs_single_4096_domain_fp64_active"] = (
                        ens[form]["value"] / act)
            forms["ensemble"] = ens
        if "tra_adv" in want:
            forms["tra_adv"] = run_tra_adv(lib)
        if "emulator" in want:
            forms["emulator"] = run_emulator(lib, count=args.emu_domains,
                                             horizon=args.emu_horizon, iters=args.emu_iters)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count()))
        best, rates = time_cpu_layers(n, 10 ** 6, 2, target_s=10.0)
        val, steps, secs, kind, desc = best
        cpu = {"value": val, "unit": "Mcell-steps/s",
               "cores": int(os.environ["OMP_NUM_THREADS"]), "kind": kind,
               "sample": "%d steps of the %dx%d domain from rest (%s, the faster of the "
                         "reference's two OpenMP layers), ~10 s each" % (steps, n, n, desc),
               "layers": rates}

    if rank == 0:
        line = {
            "metric": "Mcell-steps/s", "value": value, "unit": "Mcell-steps/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64",
            "data": ("synthetic (every cell in motion: Fourier bathymetry, random start)"
                     if active else "synthetic (reference initial state: rest, constant depth)"),
            "config": bench_config(n, m.width, m.rdt, active, world),
            "roofline": roof, "cpu_baseline": cpu, "e2e": e2e,
            "gpu_launches": args.steps,
            "clocks": clk.summary(),
            "checksums": {"ssh": sums[0], "u": sums[1], "v": sums[2]},
            "forms": forms,
        }
        print(json.dumps(line))
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


def run_case(args):
    """One small case for a profiler: --size interior (levels 75 for the
    tracer; --batch images for the emulator), --warmup untimed then --steps
    timed steps or iterations, device time from the library's CUDA events."""
    import psyclonebench_gb300 as P
    from psyclonebench_gb300.model import register
    lib = P.load_library()
    n, out = args.size, {"case": args.case, "size": args.size, "steps": args.steps}
    ms = ctypes.c_double(0.0)
    if args.case in ("fused", "fused_active", "mixed", "df"):
        m = make_problem(n)
        if args.case == "fused_active":
            make_active(m)
        if args.case == "mixed":
            from psyclonebench_gb300.workloads import fourier_depth
            m.f["ht"][:], m.f["hu"][:], m.f["hv"][:] = fourier_depth(m.width, m.height, 2)
            m.rdt = BATHY_RDT
        register(lib, m)
        lib.nl2d_set_precision({"mixed": 1, "df": 2}.get(args.case, 0))
        P.check(lib.nl2d_timed_run(1, 1 + args.warmup, ctypes.byref(ms)), "case warm-up")
        P.check(lib.nl2d_timed_run(2 + args.warmup, args.steps, ctypes.byref(ms)), "case run")
        lib.nl2d_set_precision(0)
        lib.nl2d_finalize()
    elif args.case == "tra_adv":
        from psyclonebench_gb300.workloads import tra_adv_fields
        f = tra_adv_fields(n, n, 75)
        D = ctypes.POINTER(ctypes.c_double)
        targs = [f[k].ctypes.data_as(D) for k in ("ztfreez", "pun", "pvn", "pwn", "umask",
                                                  "vmask", "tmask", "rnfmsk", "rnfmsk_z",
                                                  "upsmsk", "mydomain", "tsn")]
        for _ in range(max(1, args.warmup)):
            lib.tra_adv_compute(*targs, n, n, 75)
        rc = lib.tra_adv_run(args.steps, ctypes.byref(ms))
        buf = ctypes.create_string_buffer(256)
        if rc or lib.tra_adv_last_error(buf, 256):
            raise RuntimeError("tra_adv: %s" % buf.value.decode())
        lib.tra_adv_finalize()
    elif args.case in ("ensemble", "ensemble_mixed", "ensemble_df"):
        # the first --domains domains of run_ensemble's 512-domain draw on
        # the default schedule, in the case's form
        from psyclonebench_gb300.ensemble import Ensemble, build_domain
        from psyclonebench_gb300.workloads import ensemble_domains
        specs = ensemble_domains(512, 7)[:max(1, min(512, args.domains))]
        ens = Ensemble([build_domain(sp) for sp in specs], lib=lib)
        ens.set_precision({"ensemble_mixed": 1, "ensemble_df": 2}.get(args.case, 0))
        ens.run(1, 1 + args.warmup)
        ms.value, _ = ens.run(2 + args.warmup, args.steps)
        out["cells"] = ens.info()[0]
        ens.close()
    elif args.case == "rates":
        rates = (ctypes.c_double * 4)()
        P.check(lib.nl2d_measure_pipe_rates(rates), "pipe rates")
        out["gops"] = {"dfma": rates[0], "dmul": rates[1], "dadd": rates[2], "ffma": rates[3]}
    elif args.case == "emu":
        import torch
        from psyclonebench_gb300 import emulator as E
        net = E.ConvNet(args.batch, 256, 256, seed=0, lib=lib)
        npx = args.batch * 256 * 256
        g = torch.Generator(device="cuda").manual_seed(0)
        x = torch.randn(npx, E.CPAD_IN, device="cuda", generator=g).to(torch.bfloat16)
        target = torch.randn(npx, 3, device="cuda", generator=g)
        for _ in range(max(1, args.warmup)):
            net.forward(x)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            net.forward(x)
        e1.record()
        torch.cuda.synchronize()
        ms.value = e0.elapsed_time(e1)
        net.train_step(x, target)
        torch.cuda.synchronize()
        if int(net.err.item()) != 0:
            raise RuntimeError("emulator: a tensor-core wait ran out")
        out["batch"] = args.batch
    out["ms_per_step"] = ms.value / max(1, args.steps)
    print(json.dumps(out))


def main():
    args = parse()
    rank, world, local = dist_env()
    # The CPU legs (the reference arm, the CPU baselines) run OpenMP on every
    # host core, one thread per core, threads kept close (OpenMP reads these
    # when the CPU library is first loaded, always after this point).
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count()))
    os.environ.setdefault("OMP_PROC_BIND", "close")
    os.environ.setdefault("OMP_PLACES", "cores")
    if args.case:
        run_case(args)
    elif args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world, local)


if __name__ == "__main__":
    main()
