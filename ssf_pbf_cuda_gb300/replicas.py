"""Multi-GPU = replicas: scenes are independent, so each GPU runs its own
batched engine on its own scenes with no data-path collective.  One scene's
step would need a halo exchange to span GPUs; that is not done.

Weak scaling: every rank gets a full batched workload of its own seeded
scenes (same size distribution), so the job's work grows with the number of
ranks.  The only collectives are the host-side timing reductions of the
benchmark (barrier, max over ranks, sum of particles).
"""
from __future__ import annotations

import math

from . import scenes


def rank_scenes(n_scenes: int, rank: int, world: int) -> list:
    """The batched workload of one rank (rank 0 gets the canonical seeds)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    if rank == 0:
        return scenes.config4(n_scenes)
    rng = scenes.rng_for(4 + 7919 * rank)
    out = []
    for s in range(n_scenes):
        n = int(round(math.exp(rng.uniform(math.log(4096), math.log(65536)))))
        out.append(scenes._random_scene(rng, 1000 + s + 100000 * rank, n))
    return out


def assign_scenes(sizes: list, world: int) -> list:
    """Longest-processing-time assignment of a fixed scene list to ranks
    (for strong-scaling use): returns rank -> list of scene indices."""
    loads = [0] * world
    out = [[] for _ in range(world)]
    for i in sorted(range(len(sizes)), key=lambda k: -sizes[k]):
        r = min(range(world), key=lambda q: loads[q])
        out[r].append(i)
        loads[r] += sizes[i]
    return [sorted(o) for o in out]


def job_throughput(particles_per_rank: list, steps: int, ms_per_rank: list) -> float:
    """Whole-job particle-steps/s: all ranks' particles over the slowest rank's time."""
    return float(sum(particles_per_rank)) * steps / (max(ms_per_rank) / 1e3)
