"""The N > 1 path: sharding by slice and max-over-ranks timing, on two gloo
ranks (CPU, no GPU)."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from bimsim_gb300 import dist


def test_shard_covers_all_items_once():
    items = list(range(517))
    for world in (1, 2, 3, 4, 8):
        parts = [dist.shard(items, r, world) for r in range(world)]
        assert sum(parts, []) == items
        assert max(map(len, parts)) - min(map(len, parts)) <= 1


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import torch.distributed as tdist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank))
    tdist.init_process_group("gloo", rank=rank, world_size=world)
    lams = [2.5 + 10.0 * i / 511 for i in range(512)]
    mine = dist.shard(lams, rank, world)
    t = dist.max_over_ranks(1.0 + rank)
    tdist.barrier()
    q.put((rank, len(mine), mine[0], t))
    tdist.destroy_process_group()


@pytest.mark.timeout(120)
def test_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=100) for _ in procs)
    for p in procs:
        p.join(timeout=30)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [256, 256]
    assert out[1][2] > out[0][2]
    assert all(o[3] == 2.0 for o in out)
