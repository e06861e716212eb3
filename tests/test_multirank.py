"""The multi-rank host logic of bench.py on two gloo ranks on the CPU (the GPU job runs one process
per GPU): round-robin sharding of a batch's transforms (every transform on exactly one rank, no
collective on the data path) and the max-over-ranks reduction of the step time that the whole-job
throughput is computed from."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, out):
    import sys
    from pathlib import Path

    root = str(Path(__file__).resolve().parents[1])
    if root not in sys.path:
        sys.path.insert(0, root)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench

        specs = bench.batch_specs("mixed_512")
        mine = bench.shard(len(specs), rank, world)
        gathered = [None] * world
        dist.all_gather_object(gathered, mine)
        local_ms = 10.0 + 5.0 * rank  # rank 1 is the slower one
        job_ms = bench.max_over_ranks(local_ms, world)
        out.put((rank, gathered, job_ms, len(specs)))
    finally:
        dist.destroy_process_group()


def test_sharding_and_max_over_ranks_on_two_gloo_ranks():
    world = 2
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    results = [out.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, gathered, job_ms, count in results:
        owned = sorted(i for part in gathered for i in part)
        assert owned == list(range(count))  # each transform exactly once
        assert abs(len(gathered[0]) - len(gathered[1])) <= 1
        assert job_ms == 15.0  # the slowest rank's time on every rank
    # whole-job throughput as bench.py reports it: all transforms over the slowest rank's time
    steps = 4
    assert 512 * steps / (15.0 / 1e3) == pytest.approx(136533.33, rel=1e-6)
