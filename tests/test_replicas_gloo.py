"""Replica sharding over pulses, on CPU with a world_size-2 gloo group.

Each rank takes its share of a 64-pulse-like batch (uneven grids), advances
its pulses with the FP64 oracle for two z-steps on a tiny grid (standing in
for the GPU work the same code drives on a GB300), gathers the per-pulse
results, and checks that every pulse was computed exactly once and equals a
single-process run."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from rapport_gb300.replicas import pulse_cost, shard_pulses

GRIDS = [(512, 1024), (768, 2048), (1024, 4096), (512, 4096), (1024, 1024), (768, 1024), (512, 2048)]


def test_shards_cover_every_pulse_once_and_balance():
    costs = [pulse_cost(a, b) for a, b in GRIDS]
    for world in (1, 2, 3, 4, 8):
        parts = [shard_pulses(costs, world, r) for r in range(world)]
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(GRIDS)))
        loads = [sum(costs[i] for i in p) for p in parts]
        assert max(loads) <= sum(costs) / world + max(costs)   # LPT bound
    with pytest.raises(ValueError):
        shard_pulses(costs, 2, 2)


def _tiny_result(i):
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.join(os.path.dirname(here), "oracle"))
    import nlse_oracle as O
    g = O.OracleGrid(O.workload_config(16, 32, 1e-4, 1e-5, 3e-13))
    u0 = O.lens_gaussian(g, 1e-5, 100e-15, 1.0 + 0.5 * i, 1e-2, i)
    u, rho, _ = g.propagate(u0, 2, 5e-6)
    return float(np.sum(np.abs(u) ** 2)), float(rho.max())


def _worker(rank, world, port, out):
    import torch.distributed as dist
    from rapport_gb300.replicas import gather_by_pulse, max_over_ranks
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    costs = [pulse_cost(a, b) for a, b in GRIDS]
    mine = shard_pulses(costs, world, rank)
    local = {i: _tiny_result(i) for i in mine}
    res = gather_by_pulse(local, len(GRIDS))
    t = max_over_ranks(1.0 + rank)
    if rank == 0:
        out.put((res, t))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_gloo_replicas_equal_single_process():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res, t = q.get(timeout=300)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert t == 2.0
    ref = [_tiny_result(i) for i in range(len(GRIDS))]
    assert res == ref
