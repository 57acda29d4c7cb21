"""Multi-process (gloo, world size 2, CPU) tests of the replica bookkeeping used by bench.py:
droplet sharding and the max / sum over ranks."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.join(os.path.dirname(here), "bacterial-droplet_gb300"))
    import torch.distributed as dist
    from ttsh import replicas as R
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sizes = [256, 128, 128, 96, 192, 160, 128, 64]
    mine = R.balanced_shard(sizes, rank, world)
    load = sum(sizes[i] ** 3 for i in mine)
    mx = R.max_over_ranks(float(rank + 1) * 10.0)
    total = R.sum_over_ranks(float(load))
    dist.barrier()
    q.put((rank, mine, mx, total))
    dist.destroy_process_group()


def test_gloo_two_ranks_shard_and_reduce():
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
    sizes = [256, 128, 128, 96, 192, 160, 128, 64]
    owned = sorted(res[0][1] + res[1][1])
    assert owned == list(range(len(sizes)))            # every droplet exactly once
    assert all(r[2] == 20.0 for r in res)               # max over ranks
    assert all(r[3] == sum(n ** 3 for n in sizes) for r in res)
    loads = [sum(sizes[i] ** 3 for i in r[1]) for r in res]
    assert max(loads) <= 1.3 * min(loads)               # greedy balance


def test_shard_round_robin():
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.join(os.path.dirname(here), "bacterial-droplet_gb300"))
    from ttsh import replicas as R
    items = list(range(10))
    parts = [R.shard(items, r, 3) for r in range(3)]
    assert sorted(sum(parts, [])) == items
    with pytest.raises(ValueError):
        R.shard(items, 3, 3)
