"""Replica sharding across ranks (replicas.py), on CPU with two gloo ranks:
every image goes to exactly one rank, the split balances the pixel load,
all ranks agree on it without communicating, and the reported time is the
max over ranks."""
import os
import socket

import pytest

import conftest  # noqa: F401  (spawned ranks import this module: registers the package)
from zenav1_svt_gb300 import replicas, synth


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, weights, times, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = replicas.shard(weights, rank, world)
    t = replicas.max_over_ranks(times[rank])
    # gather every rank's shard to check disjointness on each rank
    got = [None] * world
    dist.all_gather_object(got, mine)
    dist.destroy_process_group()
    out.put((rank, mine, t, got))


def test_two_gloo_ranks_shard_and_max():
    import torch.multiprocessing as mp
    specs = synth.batch_specs(64, max_dim=1024)
    weights = [w * h for w, h, _, _ in specs]
    times = [0.25, 0.40]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, weights, times, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=60) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    shards = [m for _, m, _, _ in res]
    assert sorted(shards[0] + shards[1]) == list(range(len(weights)))
    assert not set(shards[0]) & set(shards[1])
    for _, _, t, got in res:
        assert t == max(times)
        assert got == shards  # both ranks computed the same assignment
    loads = [sum(weights[i] for i in s) for s in shards]
    assert max(loads) - min(loads) <= max(weights)  # LPT balance bound
    assert replicas.job_rate(10.0, 2, 0.5) == 40.0


def test_shard_single_rank_and_errors():
    assert replicas.shard([3, 1, 2], 0, 1) == [0, 1, 2]
    with pytest.raises(ValueError):
        replicas.shard([1], 2, 2)
    assert replicas.max_over_ranks(1.5) == 1.5
