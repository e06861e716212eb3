"""The multi-rank host logic of bench.py on the CPU (the GPU job runs one process per GPU):
sharding of a batch's transforms by algorithmic bytes (every transform on exactly one rank, the
ranks' byte totals within 10%, no collective on the data path), the max-over-ranks reduction of the
step time that the whole-job throughput is computed from (two gloo ranks), and the launch path:
`bench.py --gpus 2` without a launcher starts two ranks itself."""
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
        costs = [bench.transform_cost(*s) for s in specs]
        mine = bench.shard(costs, rank, world)
        gathered = [None] * world
        dist.all_gather_object(gathered, mine)
        local_ms = 10.0 + 5.0 * rank  # rank 1 is the slower one
        job_ms = bench.max_over_ranks(local_ms, world)
        out.put((rank, gathered, job_ms, len(specs), costs))
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
    for rank, gathered, job_ms, count, costs in results:
        owned = sorted(i for part in gathered for i in part)
        assert owned == list(range(count))  # each transform exactly once
        loads = [sum(costs[i] for i in part) for part in gathered]
        assert max(loads) <= 1.10 * min(loads), loads  # balanced by algorithmic bytes
        assert job_ms == 15.0  # the slowest rank's time on every rank
    # whole-job throughput as bench.py reports it: all transforms over the slowest rank's time
    steps = 4
    assert 512 * steps / (15.0 / 1e3) == pytest.approx(136533.33, rel=1e-6)


def test_lpt_sharding_balances_bytes_for_every_world_size():
    import sys
    from pathlib import Path

    sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
    import bench

    for name in ("mixed_512", "c2c_128_uneven256"):
        costs = [bench.transform_cost(*s) for s in bench.batch_specs(name)]
        for world in (2, 4, 8):
            parts = [bench.shard(costs, r, world) for r in range(world)]
            assert sorted(i for p in parts for i in p) == list(range(len(costs)))
            loads = [sum(costs[i] for i in p) for p in parts]
            assert max(loads) <= 1.10 * min(loads), (name, world, loads)


def test_gpus_flag_starts_the_ranks_itself():
    import json
    import subprocess
    import sys
    from pathlib import Path

    root = Path(__file__).resolve().parents[1]
    env = {k: v for k, v in os.environ.items() if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK")}
    res = subprocess.run([sys.executable, str(root / "bench.py"), "--gpus", "2", "--launch-check"],
                         capture_output=True, text=True, timeout=300, cwd=root, env=env)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [json.loads(line) for line in res.stdout.splitlines() if line.startswith("{")]
    assert sorted(d["rank"] for d in lines) == [0, 1]
    assert all(d["world_size"] == 2 and d["gpus"] == 2 for d in lines)
    # a launcher whose world size disagrees with --gpus is refused
    bad = subprocess.run([sys.executable, str(root / "bench.py"), "--gpus", "4", "--launch-check"],
                         capture_output=True, text=True, timeout=120, cwd=root,
                         env={**env, "WORLD_SIZE": "2", "RANK": "0"})
    assert bad.returncode == 2
