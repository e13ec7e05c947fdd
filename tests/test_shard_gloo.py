"""Sharding a batch of independent grids across ranks (CPU, gloo, world
size 2): the partition covers every grid once, balances cost, and the
per-grid results of the sharded run equal the single-process run -- the
step has no data-path exchange, only the final statistics are gathered."""

import os
import socket

import numpy as np
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from panopaea_gb300.batch import partition_by_cost


def test_partition_properties():
    from panopaea_gb300 import workloads as W

    dims, _, _ = W.batch_grids(count=64, seed=5)
    for n in (1, 2, 3, 8):
        parts = partition_by_cost(dims, n)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(dims)))
        loads = [sum(dims[i][0] * dims[i][1] for i in p) for p in parts]
        biggest = max(h * w for h, w in dims)
        assert max(loads) - min(loads) <= biggest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _per_grid(dims, idx):
    """The per-grid work of one rank, on the CPU oracle: one reference step
    of each assigned grid (walls, buoyancy, PCG to 1e-6)."""
    from oracle import pyoracle as O

    out = {}
    for i in idx:
        h, w = dims[i]
        r = np.random.default_rng(1000 + i)
        vel = O.walls(r.standard_normal(O.num_faces((h, w))), (h, w))
        rho = r.random((h, w))
        p = np.zeros((h, w))
        prm = O.step_params(dt=0.5, buoyancy=1.0, walls_after_advect=True, rel_stop=True, rel_tol=1e-6,
                            max_iter=100000)
        O.step(vel, rho, p, (h, w), prm)
        out[i] = float(np.abs(vel).sum() + np.abs(rho).sum())
    return out


def _worker(rank, world, port, dims, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    parts = partition_by_cost(dims, world)
    mine = _per_grid(dims, parts[rank])
    gathered = [None] * world
    dist.all_gather_object(gathered, mine)  # statistics only, after the step
    if rank == 0:
        merged = {}
        for d in gathered:
            merged.update(d)
        q.put(merged)
    dist.destroy_process_group()


def test_sharded_equals_single_process():
    dims = [(12, 16), (20, 9), (8, 8), (16, 24), (10, 30), (14, 14)]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    mp.spawn(_worker, args=(2, port, dims, q), nprocs=2, join=True)
    merged = q.get(timeout=60)
    single = _per_grid(dims, range(len(dims)))
    assert sorted(merged) == list(range(len(dims)))
    for i in range(len(dims)):
        assert merged[i] == single[i]
