"""Two gloo ranks on CPU: member sharding covers an ensemble exactly once, and the
job time is the slowest rank's."""
import os
import socket

import pytest

from conformal_cubed_sphere_gb300.parallel import shard_members


def test_shard_members_partition():
    for n in (1, 7, 64):
        for w in (1, 2, 3, 8):
            got = sorted(m for r in range(w) for m in shard_members(n, r, w))
            assert got == list(range(n))
    with pytest.raises(ValueError):
        shard_members(4, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from conformal_cubed_sphere_gb300.parallel import shard_members, slowest_rank_seconds
    mine = shard_members(64, rank, world)
    dist.barrier()
    t = slowest_rank_seconds(1.0 + rank)
    q.put((rank, mine, t))
    dist.destroy_process_group()


def test_two_gloo_ranks():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[0][1] == list(range(0, 64, 2)) and res[1][1] == list(range(1, 64, 2))
    assert res[0][2] == res[1][2] == 2.0
