"""Host-level sharding of an ensemble over ranks (the multi-GPU plan: no
device collective; each rank owns whole domains).  Run as two gloo ranks on
CPU, each advancing its shard with the oracle; the gathered per-domain
checksums must equal a one-process run."""
import os

import numpy as np
import pytest

import nl2d_testlib as T

SPECS = [{"nx": n, "ny": m, "depth_seed": s, "tide_amp": a, "tide_period_h": p,
          "open_side": o}
         for n, m, s, a, p, o in [(14, 11, 1, 0.2, 12.42, "S"), (9, 17, 2, 0.3, 11.0, "E"),
                                  (20, 8, 3, 0.1, 13.5, "N"), (12, 12, 4, 0.45, 10.2, "W"),
                                  (8, 9, 5, 0.25, 12.0, "S")]]
NSTEPS = 30


def test_shards_cover_every_domain_once():
    from psyclonebench_gb300.ensemble import shard_domains
    from psyclonebench_gb300.workloads import ensemble_domains
    specs = ensemble_domains(200, 3)
    for world in (1, 2, 3, 8):
        parts = shard_domains(specs, world)
        flat = sorted(k for p in parts for k in p)
        assert flat == list(range(len(specs)))
        loads = [sum(specs[k]["nx"] * specs[k]["ny"] for k in p) for p in parts]
        assert max(loads) - min(loads) <= max(s["nx"] * s["ny"] for s in specs)


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from psyclonebench_gb300.ensemble import build_domain, shard_domains
    mine = shard_domains(SPECS, world)[rank]
    res = {}
    for k in mine:
        _, sums = T.ensemble_oracle_run(build_domain(SPECS[k]), NSTEPS, every=NSTEPS)
        res[k] = [sums[-1]["sshn_t"], sums[-1]["un"], sums[-1]["vn"]]
    from psyclonebench_gb300.ensemble import gather_results
    merged = gather_results(res, timeout_s=60.0)
    if rank == 0:
        out.put(merged)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_gloo_matches_single_process():
    import multiprocessing as mp
    import socket
    from psyclonebench_gb300.ensemble import build_domain
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    merged = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert sorted(merged) == list(range(len(SPECS)))
    for k, spec in enumerate(SPECS):
        _, sums = T.ensemble_oracle_run(build_domain(spec), NSTEPS, every=NSTEPS)
        want = [sums[-1]["sshn_t"], sums[-1]["un"], sums[-1]["vn"]]
        assert merged[k] == want


def _rank_dies(rank, world, port, out):
    """Rank 1 fails before the gather (an exception on the host, as a crashed
    solver process would); rank 0 reports what gather_results raises."""
    import datetime

    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world,
                            timeout=datetime.timedelta(seconds=30))
    from psyclonebench_gb300 import Nl2dError
    from psyclonebench_gb300.ensemble import gather_results
    if rank == 1:
        raise SystemExit(3)
    try:
        gather_results({0: [1.0, 2.0, 3.0]}, timeout_s=5.0)
        out.put("no error")
    except Nl2dError as e:
        out.put("Nl2dError: %s" % e)


def test_a_dead_rank_is_reported_not_waited_for():
    """A rank that exits before the gather: the surviving rank gets an
    Nl2dError naming it within the barrier's timeout (host-side failure
    detection; no GPU involved)."""
    import multiprocessing as mp
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_dies, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    msg = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
    assert procs[1].exitcode == 3
    assert msg.startswith("Nl2dError") and "1" in msg, msg
