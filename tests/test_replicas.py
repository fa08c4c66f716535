"""Host logic of the multi-GPU layout (replicas / independent scenes), run as gloo ranks on CPU."""
import os
import socket

import pytest

from akuaengine_gb300 import replicas


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    env = replicas.dist_env()
    dist.init_process_group("gloo", rank=env.rank, world_size=env.world)
    try:
        elapsed = 1.0 + 0.5 * rank  # rank 1 is the slow one
        dist.barrier()
        t = replicas.max_over_ranks(elapsed)
        rate = replicas.aggregate_rate(100, t, env.world)
        shards = replicas.shard_scenes([5000, 64000, 2000, 31000, 17000], env.world)
        q.put((rank, t, rate, shards, replicas.replica_seed(7, rank)))
    finally:
        dist.destroy_process_group()


def test_two_ranks_gloo():
    import torch.multiprocessing as mp

    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(world))
    for rank, t, rate, shards, seed in res:
        assert t == 1.5                      # max over ranks, on every rank
        assert rate == pytest.approx(200 / 1.5)
        assert shards == [[1], [0, 2, 3, 4]]  # identical split on every rank
    assert res[0][4] != res[1][4]            # each replica has its own seed


def test_shard_scenes_balances_and_covers():
    counts = [2000 + 997 * (s * 7919 % 61) for s in range(256)]
    for world in (1, 2, 4, 8):
        shards = replicas.shard_scenes(counts, world)
        flat = sorted(s for sh in shards for s in sh)
        assert flat == list(range(256))
        loads = [sum(counts[s] for s in sh) for sh in shards]
        assert max(loads) - min(loads) <= max(counts)


def test_dist_env_defaults_and_errors(monkeypatch):
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    assert replicas.dist_env() == replicas.DistEnv(1, 0, 0)
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "2")
    with pytest.raises(ValueError):
        replicas.dist_env()
    with pytest.raises(ValueError):
        replicas.aggregate_rate(1, 0.0, 1)
