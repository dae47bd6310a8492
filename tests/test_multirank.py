"""The multi-rank host logic of bench.py on CPU, with gloo ranks.

One graph does not shard (it runs as replicas). The mixed-graph stream shards
by graph, with no collective on the data path. Each rank computes its share
with shard_graphs, and only the final metrics are reduced (sum of rates and
work, maximum of times). These tests run that split and those reductions as
two gloo processes.
"""
from __future__ import annotations

import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))


def test_shards_cover_every_graph_once_and_balance():
    import bench
    specs = bench.mix_sizes(64, 1e3, 5e5, 1000003)
    for world in (1, 2, 3, 8):
        parts = [bench.shard_graphs(specs, r, world) for r in range(world)]
        flat = sorted(i for part in parts for i in part)
        assert flat == list(range(len(specs)))
        loads = [sum(specs[i][0] * specs[i][1] for i in part) for part in parts]
        biggest = max(s[0] * s[1] for s in specs)
        assert max(loads) - min(loads) <= biggest  # greedy split: within one graph of even


def _rank_main(rank, world, port, out):
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    td = bench.dist_init(world)
    try:
        specs = bench.mix_sizes(16, 1e3, 5e5, 1000003)
        mine = bench.shard_graphs(specs, rank, world)
        work = float(sum(specs[i][0] for i in mine))      # stands in for affected edges
        seconds = 1.0 + rank                               # stands in for a rank's timed span
        total = bench.dist_sum(td, work)
        slowest = bench.dist_max(td, seconds)
        count = bench.dist_sum(td, float(len(mine)))
        bench.dist_barrier(td)
        out.put((rank, total, slowest, count))
    finally:
        td.destroy_process_group()


def test_two_gloo_ranks_reduce_shard_metrics():
    torch = pytest.importorskip("torch")
    import socket
    import bench
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = torch.multiprocessing.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    specs = bench.mix_sizes(16, 1e3, 5e5, 1000003)
    want_total = float(sum(s[0] for s in specs))
    for _, total, slowest, count in got:
        assert total == want_total
        assert slowest == 2.0
        assert count == 16.0


def test_bench_gpus_flag_launches_that_many_ranks():
    """`bench.py --gpus 2` (no WORLD_SIZE in the environment) starts two ranks
    itself; the shard-check arm does no GPU work, so the launcher, the shard
    split and the metric reductions run here on CPU with gloo."""
    pytest.importorskip("torch")
    import json
    import subprocess
    import bench
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK")}
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "shard-check", "--gpus", "2"],
                         capture_output=True, text=True, timeout=300, env=env)
    assert out.returncode == 0, out.stderr
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1  # rank 0 alone prints
    got = json.loads(lines[0])
    specs = bench.mix_sizes(512, 1e3, 5e5, 1000003)
    assert got["n_gpus"] == 2 and got["graphs"] == 512
    assert got["total_load"] == sum(s[0] * s[1] for s in specs)
    assert sorted(set(got["owners"])) == [1, 2]  # every graph owned by exactly one of the two ranks
    for r in (0, 1):
        mine = bench.shard_graphs(specs, r, 2)
        assert all(got["owners"][i] == r + 1 for i in mine)
    assert got["max_load"] == max(sum(specs[i][0] * specs[i][1] for i in bench.shard_graphs(specs, r, 2))
                                  for r in (0, 1))
