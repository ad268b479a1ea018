"""Replica sharding across ranks (world_size 2, gloo, CPU): ranges tile the
item list, and the gathered per-rank results equal the single-process ones."""

import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from klampt_gb300.shard import shard_range


def test_shard_ranges_tile():
    for n in (0, 1, 7, 16384, 16385):
        for world in (1, 2, 3, 8):
            ranges = [shard_range(n, r, world) for r in range(world)]
            assert ranges[0][0] == 0 and ranges[-1][1] == n
            assert all(ranges[i][1] == ranges[i + 1][0] for i in range(world - 1))
            sizes = [e - b for b, e in ranges]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard_range(10, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    import torch.distributed as dist
    from klampt_gb300 import scenes as sc
    from klampt_gb300.shard import run_sharded
    from oracle.oracle_py import Oracle

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    robot, env, q = sc.scene_cfg0()
    o = Oracle(robot, env)
    qa, qb, ns = sc.random_edges(robot, 37, np.random.default_rng(2))
    res = run_sharded(37, lambda b, e: o.check_edges(qa[b:e], qb[b:e], ns[b:e])[0])
    if rank == 0:
        full, _ = o.check_edges(qa, qb, ns)
        out.put(bool(np.array_equal(res, full)))
    dist.barrier()
    dist.destroy_process_group()


def test_sharded_edges_gloo_world2():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    ok = q.get(timeout=300)
    for p in procs:
        p.join(timeout=120)
    assert ok
    assert all(p.exitcode == 0 for p in procs)
