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


def _member_digests(members, N=8, steps=2):
    """Member k of the seeded ensemble advanced `steps` RK4 steps by the CPU
    restatement of the reference step, as SHA-256 digests of its prognostic fields."""
    import hashlib

    import numpy as np

    from conformal_cubed_sphere_gb300 import model as M
    from oracle import oracle as O
    out = {}
    for k in members:
        mesh = M.Mesh(N, 3)
        st = M.ensemble_member_state(mesh, k, seed=1)
        dt = M.cfl_dt(mesh, st, 0.5)
        orc = O.Oracle.from_mesh(mesh)
        orc.set_state(st.arrays)
        orc.run(dt, steps)
        s = orc.get_state()
        out[k] = hashlib.sha256(np.concatenate([s["phiG"], s["u"], s["v"]]).tobytes()).hexdigest()
        orc.close()
    return out


def _ensemble_worker(rank, world, port, n_members, q):
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from conformal_cubed_sphere_gb300.parallel import shard_members
    mine = _member_digests(shard_members(n_members, rank, world))
    # a check outside the data path: every rank's members, gathered for the test
    got = [None] * world
    dist.all_gather_object(got, mine)
    q.put((rank, got))
    dist.destroy_process_group()


def test_sharded_ensemble_members_advance_as_in_one_process():
    """Two gloo ranks each advance their own members of a 5-member ensemble (C8,
    two RK4 steps of the CPU restatement); with no exchange between the ranks, the
    union of their members equals one process advancing all five, bit for bit:
    a member's state depends on its index only, not on the rank that owns it."""
    import multiprocessing as mp
    n = 5
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_ensemble_worker, args=(r, 2, port, n, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=300) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    serial = _member_digests(range(n))
    for rank, got in res:
        merged = {}
        for part in got:
            assert not set(part) & set(merged)  # every member on exactly one rank
            merged.update(part)
        assert merged == serial, rank
    assert sorted(res[0][1][0]) == [0, 2, 4] and sorted(res[0][1][1]) == [1, 3]
