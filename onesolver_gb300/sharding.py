"""Several processes (one per GPU): exhaustive search sharded by fixed top
bits with a host-side merge of the shard results, and replicas of the
annealing-family solvers merged by their best state.

The 2^n states split by their top k bits into 2^k contiguous shards
(`fixed_high_bits = k`, `prefix = p` enumerates the states
[p * 2^(n-k), (p + 1) * 2^(n-k))). Ranks take the shards round-robin, so
there is no exchange on the data path; the only collective is one gather of
each rank's (energy, minimisers) record after the kernels finish. The merged
answer is the one `exhaustive::solve` gives on the whole space
(include/exhaustive/exhaustive.hpp:130-133, 158-166): the lowest energy, and
among its minimisers the smallest state integer.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Callable, Optional, Sequence

import numpy as np


def shard_bits(n: int, world: int, shards_per_rank: int = 4) -> int:
    """Fixed top bits so that every rank gets about `shards_per_rank` shards
    (never more bits than n - 1: each shard keeps at least two states)."""
    if world < 1:
        raise ValueError("world must be >= 1")
    if world == 1:
        return 0
    k = math.ceil(math.log2(world * shards_per_rank))
    return max(0, min(k, n - 1))


def shard_prefixes(world: int, rank: int, k: int) -> list[int]:
    """Prefixes (values of the top k bits) enumerated by `rank`."""
    if not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside [0, {world})")
    return list(range(rank, 1 << k, world))


@dataclass
class ShardRecord:
    energy: float              # +inf for a rank with no shard
    states: np.ndarray         # uint64 minimisers of that energy, ascending
    count: int                 # total minimisers (may exceed len(states))
    states_enumerated: int


def merge_records(records: Sequence[ShardRecord], max_minimisers: Optional[int] = None) -> ShardRecord:
    """Lowest energy over the records; the union of the minimisers at that
    energy, ascending (the smallest is the reference's answer)."""
    recs = [r for r in records if r.states_enumerated > 0]
    if not recs:
        raise ValueError("no shard was enumerated")
    e = min(r.energy for r in recs)
    best = [r for r in recs if r.energy == e]
    states = np.unique(np.concatenate([np.asarray(r.states, dtype=np.uint64) for r in best]))
    count = sum(r.count for r in best)
    if max_minimisers is not None:
        states = states[:max_minimisers]
    return ShardRecord(e, states, count, sum(r.states_enumerated for r in recs))


def gpu_shard_solver(f: np.ndarray, *, ctx=None, max_minimisers: int = 4096) -> Callable[[int, int], ShardRecord]:
    """Shard solver running the library's kernels (one ExhaustivePlan call
    per shard)."""
    from . import exhaustive

    def solve(k: int, prefix: int) -> ShardRecord:
        r = exhaustive(f, ctx=ctx, fixed_high_bits=k, prefix=prefix, max_minimisers=max_minimisers)
        return ShardRecord(r.energy, np.asarray(r.states, dtype=np.uint64), int(r.count), int(r.states_enumerated))

    return solve


def _gather_on_rank0(obj, world: int, rank: int, group) -> Optional[list]:
    """torch.distributed.gather_object of `obj` to rank 0 over `group` (None =
    the default process group, which must be initialised); the list of every
    rank's object on rank 0, None elsewhere."""
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized():
        raise ValueError("world > 1 needs an initialised torch.distributed process group")
    gathered = [None] * world if rank == 0 else None
    dist.gather_object(obj, gathered, dst=0, group=group)
    return gathered


def exhaustive_sharded(f: np.ndarray, solve_shard: Callable[[int, int], ShardRecord], *, world: int = 1,
                       rank: int = 0, group=None, shards_per_rank: int = 4,
                       max_minimisers: Optional[int] = None) -> Optional[ShardRecord]:
    """Enumerate this rank's shards with `solve_shard(k, prefix)` (e.g.
    `gpu_shard_solver(f)`), then gather the records on rank 0 and merge them.
    Returns the merged record on rank 0 and None elsewhere. With world > 1
    the records travel over `group` (a torch.distributed ProcessGroup; None =
    the default group); with world == 1 no process group is needed."""
    n = f.shape[0]
    k = shard_bits(n, world, shards_per_rank)
    mine = [solve_shard(k, p) for p in shard_prefixes(world, rank, k)]
    local = merge_records(mine) if mine else ShardRecord(math.inf, np.zeros(0, np.uint64), 0, 0)
    if world == 1:
        return merge_records([local], max_minimisers)
    payload = (local.energy, local.states.tolist(), local.count, local.states_enumerated)
    gathered = _gather_on_rank0(payload, world, rank, group)
    if rank != 0:
        return None
    return merge_records([ShardRecord(e, np.asarray(s, dtype=np.uint64), c, m) for e, s, c, m in gathered],
                         max_minimisers)


# ---------------------------------------------------------------------------
# Replicas: annealing, parallel tempering, population annealing
# ---------------------------------------------------------------------------
#
# Trajectories, chains and populations are independent, so N ranks run N
# replicas of a solve with distinct Philox keys and rank 0 keeps the best
# state: one gather of (energy, state) per rank after the kernels finish, and
# the first minimum in rank order, the way sa::anneal takes the first
# minimum over its trajectories (include/simulated_annealing/annealing.hpp:
# 134-139) when rank r holds the r-th block of them.

_GOLDEN64 = 0x9E3779B97F4A7C15


def replica_seed(seed: int, rank: int) -> int:
    """Philox key of `rank`'s replica: distinct per rank, equal to `seed` on
    rank 0 (so a one-rank run is the plain call)."""
    return (seed + rank * _GOLDEN64) % (1 << 64)


@dataclass
class ReplicaBest:
    energy: float
    state: np.ndarray   # uint8[n]
    rank: int           # rank whose replica found it


def best_over_ranks(energy: float, state: np.ndarray, *, world: int = 1, rank: int = 0,
                    group=None) -> Optional[ReplicaBest]:
    """Gather every rank's best (energy, state) on rank 0 over `group` (a
    torch.distributed ProcessGroup; None = the default group) and return the
    first minimum in rank order there (None on the other ranks)."""
    state = np.asarray(state, dtype=np.uint8)
    if world == 1:
        return ReplicaBest(float(energy), state, 0)
    gathered = _gather_on_rank0((float(energy), state.tobytes()), world, rank, group)
    if rank != 0:
        return None
    best = 0
    for r in range(1, world):
        if gathered[r][0] < gathered[best][0]:
            best = r
    e, s = gathered[best]
    return ReplicaBest(e, np.frombuffer(s, dtype=np.uint8).copy(), best)


def solve_replicas(solve: Callable[[int], tuple], seed: int, *, world: int = 1, rank: int = 0,
                   group=None) -> Optional[ReplicaBest]:
    """Run `solve(seed)` -> (energy, state) with this rank's replica seed
    (e.g. `lambda s: (r := temper_sparse(csr, beta, seed=s)).energy, r.state`)
    and merge on rank 0."""
    e, state = solve(replica_seed(seed, rank))
    return best_over_ranks(e, state, world=world, rank=rank, group=group)
