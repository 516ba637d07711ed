"""Instance sharding across ranks: host logic and a world-size-2 gloo check on CPU."""

import os

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from evoxels_gb300.partition import partition_instances


def test_partition_covers_every_instance_once_and_balances():
    rng = np.random.default_rng(4)
    shapes = [(int(a),) * 3 for a in rng.choice([32, 48, 64, 96, 128], 64)]
    for ws in (1, 2, 4, 8):
        parts = partition_instances(shapes, ws)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(64))
        loads = [sum(np.prod(shapes[i]) for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(np.prod(s) for s in shapes)


def test_partition_rejects_bad_world_size():
    with pytest.raises(ValueError):
        partition_instances([(4, 4, 4)], 0)


def _worker(rank, world, port, shapes, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = partition_instances(shapes, world)[rank]
    # every rank derives the same split on its own; gather only to check it
    t = torch.zeros(len(shapes), dtype=torch.int64)
    t[mine] = rank + 1
    dist.all_reduce(t)
    gathered = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(gathered, torch.tensor([sum(int(np.prod(shapes[i])) for i in mine)]))
    if rank == 0:
        out.put((t.tolist(), [int(g) for g in gathered]))
    dist.destroy_process_group()


def test_two_ranks_agree_on_a_disjoint_cover():
    shapes = [(32, 32, 32), (128, 128, 128), (64, 64, 64), (48, 48, 48), (96, 96, 96), (32, 32, 32), (64, 64, 64)]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + (os.getpid() % 1000)
    procs = [ctx.Process(target=_worker, args=(r, 2, port, shapes, q)) for r in range(2)]
    for p in procs:
        p.start()
    owners, loads = q.get(timeout=120)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert sorted(set(owners)) == [1, 2] and all(o in (1, 2) for o in owners)
    assert sum(loads) == sum(int(np.prod(s)) for s in shapes)


def _shard_worker(rank, world, port, out):
    """One rank of a sharded batch: its share of the instances, each advanced by the oracle (the
    CPU stand-in for the batched GPU step); the results are gathered only to check them."""
    import oracle
    from evoxels_gb300.partition import shard
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    shapes, M, eps, fields = _batch()
    idx, sub, m, e, f = shard(shapes, rank, world, M, eps, fields)
    mine = {i: oracle.ch_imex_run(torch.tensor(fi).unsqueeze(0), 2, 0.1, float(ei), float(mi)).numpy()
            for i, fi, mi, ei in zip(idx, f, m, e)}
    assert [tuple(s) for s in sub] == [tuple(shapes[i]) for i in idx]
    got = [None] * world
    dist.all_gather_object(got, mine)
    if rank == 0:
        out.put(got)
    dist.destroy_process_group()


def _batch():
    rng = np.random.default_rng(5)
    shapes = [(int(a), int(a), 4) for a in rng.choice([4, 6, 8], 7)]
    M = rng.uniform(0.5, 2.0, 7)
    eps = rng.uniform(0.5, 3.0, 7) / 2
    fields = [0.5 + 0.1 * np.random.default_rng([5, i]).random(s) for i, s in enumerate(shapes)]
    return shapes, M, eps, fields


def test_sharded_batch_two_ranks_equals_one_rank():
    import oracle
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29600 + (os.getpid() % 1000)
    procs = [ctx.Process(target=_shard_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = q.get(timeout=180)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    shapes, M, eps, fields = _batch()
    merged = {}
    for part in got:
        assert not set(part) & set(merged)          # disjoint shares
        merged.update(part)
    assert sorted(merged) == list(range(len(shapes)))
    for i, f in enumerate(fields):
        ref = oracle.ch_imex_run(torch.tensor(f).unsqueeze(0), 2, 0.1, float(eps[i]), float(M[i])).numpy()
        np.testing.assert_array_equal(merged[i], ref)


def test_shard_validates_its_arguments():
    from evoxels_gb300.partition import shard
    with pytest.raises(ValueError):
        shard([(4, 4, 4)], 1, 1)
    with pytest.raises(ValueError):
        shard([(4, 4, 4), (4, 4, 4)], 0, 2, [1.0])
