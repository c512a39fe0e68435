"""Multi-process paths on the CPU (torch.distributed, gloo, world size 2).

Exhaustive search shards the state space by its top bits over the ranks and
merges one record per rank on rank 0; the bench's N > 1 timing takes the
maximum over ranks. The shard solver here is the oracle (exhaustive::solve
restated), so the host logic is checked without a GPU; on a GPU machine the
same function runs `gpu_shard_solver`.
"""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

import oracle  # noqa: E402
from onesolver_gb300 import sharding  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _int_qubo(n, seed):
    rng = np.random.default_rng(seed)
    u = np.triu(rng.integers(-3, 4, size=(n, n)).astype(np.float64))
    return u + np.triu(u, 1).T


def oracle_shard_solver(f):
    n = f.shape[0]

    def solve(k, prefix):
        lo = prefix << (n - k)
        hi = (prefix + 1) << (n - k)
        e, count, states = oracle.exhaustive_all(f, lo, hi)
        return sharding.ShardRecord(e, np.asarray(states, dtype=np.uint64), int(count), hi - lo)

    return solve


def _worker(rank, world, port, n, seed, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        f = _int_qubo(n, seed)
        # An explicit ProcessGroup object (not the torch.distributed module).
        group = dist.new_group(list(range(world)))
        rec = sharding.exhaustive_sharded(f, oracle_shard_solver(f), world=world, rank=rank, group=group)
        # bench.py's max-over-ranks timing reduction
        import bench
        t = bench.max_over_ranks(dist, float(rank + 1) * 1.5)
        if rank == 0:
            np.savez(os.path.join(out_dir, "merged.npz"), energy=rec.energy, states=rec.states, count=rec.count,
                     enumerated=rec.states_enumerated, tmax=t)
        else:
            assert rec is None
            np.savez(os.path.join(out_dir, f"rank{rank}.npz"), tmax=t)
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("n,seed", [(12, 0), (14, 5)])
def test_sharded_exhaustive_matches_whole_space(tmp_path, n, seed):
    oracle.build()
    world = 2
    mp.start_processes(_worker, args=(world, _free_port(), n, seed, str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    got = np.load(tmp_path / "merged.npz")
    f = _int_qubo(n, seed)
    e, count, states = oracle.exhaustive_all(f, 0, 1 << n)
    assert float(got["energy"]) == e
    assert int(got["count"]) == count
    assert np.array_equal(got["states"], np.asarray(states, dtype=np.uint64))
    assert int(got["enumerated"]) == 1 << n
    # the timing reduction is the maximum over ranks on every rank
    assert float(got["tmax"]) == 3.0
    assert float(np.load(tmp_path / "rank1.npz")["tmax"]) == 3.0


def test_shard_assignment_covers_every_prefix_once():
    for world in (1, 2, 3, 4, 8):
        for n in (3, 10, 36):
            k = sharding.shard_bits(n, world)
            seen = sorted(p for r in range(world) for p in sharding.shard_prefixes(world, r, k))
            assert seen == list(range(1 << k))
            if world > 1 and n - 1 >= 3:
                assert (1 << k) >= world


def test_merge_keeps_lowest_energy_and_union_of_minimisers():
    R = sharding.ShardRecord
    recs = [R(-5.0, np.array([7, 3], np.uint64), 2, 8), R(-5.0, np.array([12], np.uint64), 1, 8),
            R(-4.0, np.array([1], np.uint64), 1, 8), R(float("inf"), np.zeros(0, np.uint64), 0, 0)]
    m = sharding.merge_records(recs)
    assert m.energy == -5.0 and m.count == 3 and m.states_enumerated == 24
    assert m.states.tolist() == [3, 7, 12]
    with pytest.raises(ValueError):
        sharding.merge_records([R(float("inf"), np.zeros(0, np.uint64), 0, 0)])
    with pytest.raises(ValueError):
        sharding.shard_prefixes(2, 2, 3)


@pytest.mark.gpu
def test_gpu_shards_of_two_ranks_merge_to_the_whole_space():
    """Both ranks' shard lists run on this GPU in turn (no process group):
    the merged record equals the single-call result and the oracle."""
    import onesolver_gb300 as osg
    f = _int_qubo(22, 3)
    solve = sharding.gpu_shard_solver(f)
    world = 2
    k = sharding.shard_bits(22, world)
    per_rank = [sharding.merge_records([solve(k, p) for p in sharding.shard_prefixes(world, r, k)])
                for r in range(world)]
    merged = sharding.merge_records(per_rank)
    whole = osg.exhaustive(f)
    assert merged.energy == whole.energy
    assert merged.count == whole.count
    assert merged.states.tolist() == np.asarray(whole.states, dtype=np.uint64).tolist()
    assert merged.states_enumerated == 1 << 22
    e, count, states = oracle.exhaustive_all(f, 0, 1 << 22)
    assert merged.energy == e and merged.count == count


def _replica_worker(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        f = _int_qubo(16, 3)

        def solve(seed):
            # the oracle's free-running anneal stands in for the GPU solver
            states, energies, _ = oracle.anneal_free(f, oracle.schedule_geometric(0.2, 3.0, 40), 8, 1,
                                                     seed=seed % (1 << 31), acceptance=1, site_order=1)
            k = int(np.argmin(energies))
            return float(energies[k]), np.asarray(states[k], dtype=np.uint8)

        e, s = solve(sharding.replica_seed(77, rank))
        best = sharding.solve_replicas(solve, 77, world=world, rank=rank)
        np.savez(os.path.join(out_dir, f"rep{rank}.npz"), e=e, s=s,
                 best_e=np.nan if best is None else best.energy,
                 best_s=np.zeros(0, np.uint8) if best is None else best.state,
                 best_rank=-1 if best is None else best.rank)
    finally:
        dist.destroy_process_group()


def test_replicas_merge_to_the_first_minimum_over_ranks(tmp_path):
    world = 2
    mp.spawn(_replica_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    r = [np.load(tmp_path / f"rep{k}.npz") for k in range(world)]
    energies = [float(x["e"]) for x in r]
    first = int(np.argmin(energies))
    assert int(r[0]["best_rank"]) == first
    assert float(r[0]["best_e"]) == min(energies)
    assert np.array_equal(r[0]["best_s"], r[first]["s"])
    assert oracle.energy(_int_qubo(16, 3), r[0]["best_s"]) == min(energies)
    assert int(r[1]["best_rank"]) == -1


def test_replica_seeds():
    assert sharding.replica_seed(5, 0) == 5
    seeds = {sharding.replica_seed(5, r) for r in range(64)}
    assert len(seeds) == 64 and all(0 <= s < (1 << 64) for s in seeds)
