"""The multi-rank plumbing of bench.py on CPU: two gloo ranks over
127.0.0.1 -- process-group setup from the launcher's environment, the
barrier, the max over ranks of the timed region, the reference arm doing its
work on rank 0 only, and replica seeds that never repeat across ranks."""
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
