"""CPU, world size 2 over gloo: the multi-GPU form of the bench — independent
systems sharded round-robin over ranks with no data-path collective, a
barrier, and max/sum reductions of the per-rank timings and atom counts."""
from __future__ import annotations

import os
import socket

import pytest


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank: int, world: int, port: int, q):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    specs = bench.workload_sizes("batch256", 256, 20261203)
    mine = [i for i in range(len(specs)) if i % world == rank]
    atoms = sum(10 * c * r for c, r, _ in (specs[i] for i in mine))
    bench.barrier(world)
    t_max = bench.max_over_ranks(float(rank + 1), world)
    total = bench.sum_over_ranks(float(atoms), world)
    q.put((rank, mine, atoms, t_max, total))
    dist.destroy_process_group()


def test_sharding_and_reductions_world2():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, m0, a0, t0, s0), (r1, m1, a1, t1, s1) = res
    assert set(m0).isdisjoint(m1) and sorted(m0 + m1) == list(range(256))
    assert t0 == t1 == 2.0  # max over ranks
    assert s0 == s1 == float(a0 + a1)  # whole-job atom count


@pytest.mark.parametrize("n,k", [(256, 8), (5, 8), (9, 3)])
def test_stratified_sample(n, k):
    import bench

    s = bench.stratified(n, k)
    assert s[0] == 0 and s[-1] == n - 1 and len(s) == min(n, k)


def test_spawn_path_starts_one_rank_per_device(tmp_path):
    """bench.py --gpus 2 without a launcher re-executes itself through
    torch.distributed.run: two ranks, each selecting the library device of its
    LOCAL_RANK, sharding the systems and reducing over gloo."""
    import json

    import bench
    from conftest import ROOT

    rc = bench.spawn_ranks(2, [str(ROOT / "tests" / "dist_rank.py"), str(tmp_path), "2"])
    assert rc == 0
    recs = sorted((json.loads((tmp_path / f"rank{r}.json").read_text()) for r in range(2)), key=lambda d: d["rank"])
    assert [d["world"] for d in recs] == [2, 2]
    assert [d["device"] for d in recs] == [d["local"] for d in recs] == [0, 1]
    m0, m1 = recs[0]["mine"], recs[1]["mine"]
    assert set(m0).isdisjoint(m1) and sorted(m0 + m1) == list(range(256))
    assert recs[0]["t_max"] == recs[1]["t_max"] == 2.0
    assert recs[0]["total"] == recs[1]["total"] == float(recs[0]["atoms"] + recs[1]["atoms"])


def test_world_size_must_match_the_requested_gpus(monkeypatch):
    import bench

    monkeypatch.setenv("WORLD_SIZE", "1")
    with pytest.raises(SystemExit):
        bench.dist_setup(2)
