"""Replicas over pulses: the only multi-GPU form of this propagator.

Within one pulse nothing shards without an all-to-all every half step (the
QDHT couples all radii, the FFT and the carrier march all times), so N GPUs
advance N disjoint sets of independent pulses -- one process per GPU, no
collective on the data path.  This module holds the host logic: a balanced
assignment of pulses to ranks (cost ~ Nr^2 Nt, the tensor-core product) and
the gathers used after the run (per-pulse results, max-over-ranks timing).
"""


def pulse_cost(Nr, Nt):
    """Relative cost of one z-step of a pulse (the 8 Nr^2 Nt product dominates)."""
    return float(Nr) * Nr * Nt


def shard_pulses(costs, world, rank):
    """Indices of the pulses rank `rank` of `world` advances: greedy longest-
    processing-time assignment (largest pulse to the least-loaded rank), ties
    broken by rank then index, so every rank computes the same partition."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"bad rank {rank} of {world}")
    load = [0.0] * world
    owner = [0] * len(costs)
    for i in sorted(range(len(costs)), key=lambda k: (-costs[k], k)):
        r = min(range(world), key=lambda q: (load[q], q))
        owner[i] = r
        load[r] += costs[i]
    return [i for i in range(len(costs)) if owner[i] == rank]


def gather_by_pulse(local, n_pulses, group=None):
    """all_gather of {pulse index: result} dicts from every rank -> list indexed by pulse."""
    import torch.distributed as dist
    world = dist.get_world_size(group)
    parts = [None] * world
    dist.all_gather_object(parts, local, group=group)
    out = [None] * n_pulses
    for part in parts:
        for i, v in part.items():
            if out[i] is not None:
                raise RuntimeError(f"pulse {i} reported by two ranks")
            out[i] = v
    missing = [i for i, v in enumerate(out) if v is None]
    if missing:
        raise RuntimeError(f"pulses {missing} reported by no rank")
    return out


def max_over_ranks(seconds, group=None):
    """The slowest rank's time (whole-job wall time of a replica run)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(seconds)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())
