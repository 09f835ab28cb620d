"""bench.py's host logic on CPU.  The multi-rank plumbing: two gloo ranks
over 127.0.0.1 -- process-group setup from the launcher's environment, the
barrier, the max over ranks of the timed region, the reference arm doing its
work on rank 0 only, and replica seeds that never repeat across ranks.  The
CPU baseline's sample over every source, and the compact summary of the legs
at the end of the benchmark line."""
import os
import socket
import sys
from pathlib import Path

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, q) -> None:
    os.environ.update(WORLD_SIZE=str(world), RANK=str(rank), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import bench
    import torch.distributed as dist
    w, r, local = bench.dist_setup()
    assert (w, r, local) == (world, rank, rank) and dist.get_backend() == "gloo"
    bench.barrier(w)
    m = bench.max_over_ranks(1.5 + rank, w)

    class Args:
        gpus, steps, warmup = world, 1, 0

    ran = None
    if rank != 0:
        ran = bench.run_reference(Args, w, r)  # returns at once off rank 0
    bench.barrier(w)
    dist.destroy_process_group()
    q.put((rank, m, ran))


def test_two_gloo_ranks():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(world))
    assert [m for _, m, _ in res] == [2.5, 2.5]
    assert res[1][2] is None


def test_replica_seeds_are_distinct():
    sys.path.insert(0, str(ROOT))
    import bench
    seeds = {bench.step_seed(r, i) for r in range(8) for i in range(-10, 20_000)}
    assert len(seeds) == 8 * 20_010


def test_cpu_sample_spreads_over_every_source():
    """The CPU baseline times the first photons of every source in
    proportion to its photons (not the first N photon ids, which all belong
    to the first cascade), within the global photon-id ranges of each source."""
    sys.path.insert(0, str(ROOT))
    import bench

    class Src:
        def __init__(self, n):
            self.photons = n

    class Setup:
        sources = [Src(10_000_000), Src(2_000_000_000), Src(0), Src(500_000_000)]

    n = 1_000_000
    ranges = bench.sample_ranges(Setup, n)
    counts = [s.photons for s in Setup.sources]
    starts = [sum(counts[:i]) for i in range(len(counts))]
    total = sum(counts)
    assert len(ranges) == 3  # the empty source takes no range
    for (b, e), i in zip(ranges, (0, 1, 3)):
        assert b == starts[i] and e - b == round(n * counts[i] / total)
    assert abs(sum(e - b for b, e in ranges) - n) <= len(ranges)


def test_legs_summary_keeps_every_leg_in_a_short_tail():
    """The headline numbers of the legs come last on the benchmark line in a
    compact block: a 1500-character tail of the line holds all of them."""
    import json
    sys.path.insert(0, str(ROOT))
    import bench
    msd = lambda x: {"mean": x, "sd": x / 10}  # noqa: E731
    out = {
        "serving": {"saturated": {"events_per_s": 560.0}, "realtime": {"latency_p50_ms": 0.9, "latency_p99_ms": 33.0}},
        "flow": {"table": {"rows": 19_513_125},
                 "training": {"samples_per_s": 7.9e7, "roofline": {"achieved": 85.0, "frac": 0.05}},
                 "inference": {"tuples_per_s": 3.3e10, "e2e": {"tuples_per_s": 5.5e9}}},
        "hybrid": {"saturated": {"events_per_s": 7000.0}, "realtime": {"latency_p50_ms": 2.0, "latency_p99_ms": 3.2},
                   "plain_mc": {"events_per_s": 0.36}, "speedup_vs_plain_mc": 19000.0,
                   "error_vs_mc": {"rel_err_median": msd(0.017), "rel_err_p90": msd(0.064), "ks_median": msd(0.011),
                                   "ks_max": msd(0.022), "ks_max_spread_events": msd(0.021), "seeds": 3,
                                   "events": 12},
                   "ks_check": {"raw_at_most_threshold": 4, "checks": 4}},
    }
    s = bench.legs_summary(out)
    assert set(s) == {"serving", "flow", "hybrid"}
    tail = json.dumps({"legs": s})
    assert len(tail) < 1500, len(tail)
    assert s["hybrid"]["ks_checks_raw_le_0.02"] == [4, 4]
    assert s["flow"]["train_frac_of_bf16_sustained"] == 0.05
