#!/usr/bin/env python3
"""Benchmark of the GB300 oneSolver hot paths; prints one JSON line.

Workloads (--workload):
  exhaustive36  Exhaustive search on a dense QUBO with n = 36 and integer
                coefficients drawn uniformly from [-8, 8] (seed 0): 2^36
                states, int32 Gray-code enumeration, ground energy and all
                degenerate minimisers. Metric: enumerated states/s. (default)
  sa-chimera    Sparse SA on a 16x16 Chimera of K4,4 cells (2048 spins),
                J in {-1,+1}, h = 0, converted to QUBO; 1024 trajectories x
                10,000 sweeps, linear beta 0.1 -> 3.0, FP32 fields with an
                FP64 resync every 256 sweeps. Metric: spin-flip attempts/s.
  sa-sk         Dense SA on a Sherrington-Kirkpatrick QUBO, n = 1024,
                J_ij ~ N(0, 1/n); 512 trajectories x 1,000 sweeps, geometric
                beta 0.1 -> 5.0. Metric: spin-flip attempts/s.
  sa-batch      Batched dense SA: 512 instances, n ~ U[64, 1024], entries
                N(0, 1/n); 256 trajectories x 2,000 sweeps each, geometric
                beta 0.1 -> 5.0, one persistent launch per 250-sweep chunk,
                CUDA-graph replay, autotuned trajectories per CTA.
  sa-learned    Learned warm start on SK n = 1024 (J_ij ~ N(0, 1/n)): the
                network the library ships (onesolver_gb300/data/
                warmstart_sk1024.npz, trained on 4,096 seeded instances by
                onesolver_gb300/train_warmstart.py with the library's own
                kernels), on --learned-eval of its 256 held-out seeds: the
                time-to-target (within 0.5% of the seed's 10^5-sweep plain-SA
                best) of the gated warm start vs plain random-init SA, 512
                trajectories each. Metric: seconds (median).
  pt-droplet    Parallel tempering on the reference's Chimera droplet 512/001
                (committed fixture): 128 chains x 32 temperatures, 20,000
                exchange rounds of 5 sweeps. Metric: spin-flip attempts/s;
                the best energies are reported against the tensor-network
                ground state and the reference's best published SA energy.
  pa-droplet    Population annealing on the same fixture: 16,384 replicas,
                1,000 steps of linear beta 0.05 -> 3.0 with 5 sweeps each.
                Metric: spin-flip attempts/s; best energies and the final
                free-energy estimate are reported.
  sa-n64        Dense SA, n = 64, N(0,1) entries (seed 0), 100 trajectories x
                100 random-site steps, geometric beta 0.1 -> 1.0 with the
                reference's acceptance rule. Metric: spin-flip attempts/s.

A "step" is one whole pass of the workload (every state, or every sweep of
every trajectory). `value` is timed on the device with CUDA events around the
library's kernels (inputs resident in HBM, L2 flushed between steps); `e2e`
times the reference-facing call with host buffers (upload, kernels, download).
--impl reference times the reference algorithm (the oracle's CPU restatement)
on the host cores instead.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

L2_FLUSH_BYTES = 256 << 20     # > 129 MB L2


# ---------------------------------------------------------------------------
# Workload generators (seeded synthetic instances with the configs' shapes)
# ---------------------------------------------------------------------------

def int_qubo(n: int, seed: int, lo: int = -8, hi: int = 8) -> np.ndarray:
    rng = np.random.default_rng(seed)
    u = np.triu(rng.integers(lo, hi + 1, size=(n, n)).astype(np.float64))
    return u + np.triu(u, 1).T


def normal_qubo(n: int, seed: int, scale: float = 1.0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    u = np.triu(rng.normal(0.0, scale, size=(n, n)))
    return u + np.triu(u, 1).T


def sk_qubo(n: int, seed: int) -> np.ndarray:
    """SK Ising J_ij ~ N(0, 1/n), h = 0 -> QUBO (x = (s+1)/2, offset dropped)."""
    rng = np.random.default_rng(seed)
    J = np.triu(rng.normal(0.0, 1.0 / math.sqrt(n), size=(n, n)), 1)
    Js = J + J.T
    f = 4.0 * Js
    np.fill_diagonal(f, -2.0 * Js.sum(axis=1))
    return f


def chimera_csr(L: int, seed: int):
    """L x L Chimera (K4,4 cells), J in {-1,+1}, h = 0 -> QUBO in CSR form."""
    import onesolver_gb300 as osg
    rng = np.random.default_rng(seed)
    n = 8 * L * L
    rows, cols = [], []

    def idx(r, c, side, k):
        return (r * L + c) * 8 + side * 4 + k

    for r in range(L):
        for c in range(L):
            for a in range(4):
                for b in range(4):
                    rows.append(idx(r, c, 0, a)); cols.append(idx(r, c, 1, b))
            if r + 1 < L:
                for k in range(4):
                    rows.append(idx(r, c, 0, k)); cols.append(idx(r + 1, c, 0, k))
            if c + 1 < L:
                for k in range(4):
                    rows.append(idx(r, c, 1, k)); cols.append(idx(r, c + 1, 1, k))
    J = rng.choice([-1.0, 1.0], size=len(rows))
    rows = np.array(rows); cols = np.array(cols)
    diag = np.zeros(n)
    np.add.at(diag, rows, -2.0 * J)
    np.add.at(diag, cols, -2.0 * J)
    r2 = np.concatenate([rows, cols]); c2 = np.concatenate([cols, rows]); v2 = np.concatenate([4 * J, 4 * J])
    order = np.lexsort((c2, r2))
    r2, c2, v2 = r2[order], c2[order], v2[order]
    rp = np.zeros(n + 1, dtype=np.int32)
    np.add.at(rp, r2 + 1, 1)
    rp = np.cumsum(rp).astype(np.int32)
    return osg.Csr(n, rp, c2.astype(np.int32), v2.astype(np.float64), diag)


# ---------------------------------------------------------------------------
# Clocks during the timed region
# ---------------------------------------------------------------------------

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict | None:
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# Distributed plumbing (one rank per GPU; replicas of independent instances)
# ---------------------------------------------------------------------------

def dist_setup(n_gpus: int):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
        pg = dist
    return world, rank, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, value: float) -> float:
    if pg is None:
        return value
    import torch
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def load_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return json.loads(p.read_text())
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "fallback": True}


# ---------------------------------------------------------------------------
# Our implementation
# ---------------------------------------------------------------------------

def timed_steps(ctx_stream_setter, flush, run_one, kernel_ms, steps: int, warmup: int, pg):
    """W untimed warm-up steps, then K timed steps with an L2 flush before
    each; returns (per-step device ms list, per-step kernel ms list)."""
    import torch
    for _ in range(warmup):
        run_one()
    torch.cuda.synchronize()
    barrier(pg)
    torch.cuda.synchronize()
    step_ms, kern_ms = [], []
    for _ in range(steps):
        flush()
        s = torch.cuda.Event(enable_timing=True)
        e = torch.cuda.Event(enable_timing=True)
        s.record()
        run_one()
        e.record()
        e.synchronize()
        step_ms.append(s.elapsed_time(e))
        kern_ms.append(kernel_ms())
    torch.cuda.synchronize()
    barrier(pg)
    return step_ms, kern_ms


def bench_exhaustive(args, ctx, pg, rank, world):
    import torch
    import onesolver_gb300 as osg
    n = 36
    f = int_qubo(n, rank)  # seed 0 on rank 0; independent instances on replicas
    plan = osg.ExhaustivePlan(f, ctx=ctx, max_minimisers=1 << 16, variant=args.exh_variant)
    flush_buf = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    launches = []

    def run_one():
        plan.execute()
        launches.append(plan.launches)

    sampler = ClockSampler(torch.cuda.current_device())
    for _ in range(args.warmup):
        run_one()
    torch.cuda.synchronize()
    sampler.start()
    launches.clear()
    step_ms, kern_ms = timed_steps(None, lambda: flush_buf.zero_(), run_one, plan.kernel_ms, args.steps, 0, pg)
    clocks = sampler.stop()
    res = plan.result()
    states = float(1 << n)
    t_step = max_over_ranks(pg, sum(step_ms) / len(step_ms))
    value = world * states / (t_step * 1e-3)

    # End to end: the reference-facing call with host buffers (upload, kernels, download).
    torch.cuda.synchronize()
    e2e_t = []
    for i in range(max(3, args.steps // 5)):
        t0 = time.perf_counter()
        r = osg.exhaustive(f, ctx=ctx, max_minimisers=1 << 16)
        e2e_t.append(time.perf_counter() - t0)
    assert r.energy == res.energy and r.count == res.count
    e2e_step = max_over_ranks(pg, statistics.mean(e2e_t))
    h2d = n * n * 4 + 512 * 4
    d2h = 56 + 8 * min(r.count, 1 << 16)

    k_ms = statistics.mean(kern_ms)
    # Matched ceiling: this plan's variant's own inner block walk (the
    # kernel's instruction sequence without per-item bookkeeping), measured in
    # this run; MEASURED_PEAKS.json has no integer figure.
    variant = plan.variant
    peak = osg.probe_exhaustive_pair(variant, ctx)
    achieved = states / (k_ms * 1e-3)
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    out = {
        "metric": "exhaustive enumerated states/s (n=36, int32 Gray code, all degenerate minimisers)",
        "value": value, "unit": "states/s", "ms_per_step": t_step,
        "dtype": "int32",
        "config": {"workload": "exhaustive search, dense QUBO n=36, integer Q_ij ~ U{-8..8} (seed 0), "
                               "2^36 states, ground energy + all degenerate minimisers",
                   "n": n, "states_per_step": int(states), "l2": "flushed (256 MB write) before every timed step",
                   "parallelism": f"replicas x{world}" if world > 1 else "1 GPU"},
        "result": {"energy": res.energy, "state": res.state, "minimisers": res.count},
        "roofline": {"bound": "int-issue", "achieved": achieved, "peak": peak, "unit": "states/s",
                     "frac": achieved / peak, "traffic": TRAFFIC.get("exhaustive36"),
                     "variant": variant, "ops_per_unit": 2, "kernel_ms": k_ms,
                     "states_per_sm_clock": achieved / (sms * load_peaks().get("sm_max_mhz", 2070.0) * 1e6),
                     "peak_source": ("os_probe_exhaustive_pair(%d): this variant's own inner block walk (the "
                                     "kernel's instruction sequence, couplings changing per block, no per-item "
                                     "bookkeeping), measured in this run (MEASURED_PEAKS.json has no integer "
                                     "figure)" % variant)},
        "e2e": {"value": world * states / e2e_step, "unit": "states/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": e2e_step * 1e3},
        "gpu_launches": int(sum(launches)),
        "clocks": clocks,
    }
    plan.close()
    return out


def bench_sa(args, ctx, pg, rank, world, workload):
    import torch
    import onesolver_gb300 as osg
    if workload == "sa-chimera":
        q = chimera_csr(16, rank)
        n, T = q.n, 1024
        beta = osg.linear_schedule(0.1, 2.9, 10000)  # reference linear form: ends at 0.1 + 2.9 = 3.0
        plan = osg.AnnealPlan(q, beta, num_tries=T, resync_every=256, acceptance=osg.ACCEPT_PHYSICAL, ctx=ctx)
        desc = ("sparse SA, 16x16 Chimera (K4,4 cells), 2048 spins, J in {-1,+1}, h=0 -> QUBO; 1024 "
                "trajectories x 10,000 sweeps, linear beta 0.1->3.0, FP32 fields, FP64 resync every 256 sweeps")
        attempts = T * 10000 * n
        h2d = (q.row_ptr.nbytes + q.col.nbytes + q.val.nbytes + q.diag.nbytes + beta.nbytes)
        upload = lambda: osg.anneal_sparse(q, beta, num_tries=T, resync_every=256, acceptance=osg.ACCEPT_PHYSICAL,
                                           ctx=ctx)
        avg_deg = float(q.row_ptr[-1]) / n  # neighbours updated per accepted flip
    elif workload == "sa-sk":
        n, T = 1024, 512
        f = sk_qubo(n, rank)
        beta = osg.geometric_schedule(0.1, 5.0, 1000)
        plan = osg.AnnealPlan(f, beta, num_tries=T, resync_every=250, acceptance=osg.ACCEPT_PHYSICAL,
                              site_order=osg.SITES_SEQUENTIAL, ctx=ctx)
        desc = ("dense SA, SK n=1024 J~N(0,1/n) -> QUBO; 512 trajectories x 1,000 sweeps, geometric beta "
                f"0.1->5.0, FP32 fields, FP64 resync every 250 sweeps, autotuned {plan.warps} trajectories per CTA")
        attempts = T * 1000 * n
        h2d = f.nbytes + beta.nbytes
        upload = lambda: osg.anneal(f, beta, num_tries=T, resync_every=250, acceptance=osg.ACCEPT_PHYSICAL,
                                    site_order=osg.SITES_SEQUENTIAL, ctx=ctx)
    elif workload == "sa-batch":
        rng = np.random.default_rng(rank)
        sizes = rng.integers(64, 1025, size=512)
        fs = [normal_qubo(int(m), 1000 * rank + k, scale=1.0 / math.sqrt(m)) for k, m in enumerate(sizes)]
        T = 256
        beta = osg.geometric_schedule(0.1, 5.0, 2000)
        plan = osg.BatchedAnnealPlan(fs, beta, num_tries=T, resync_every=250, ctx=ctx)
        n = int(sizes.max())
        desc = ("batched dense SA, 512 instances n~U[64,1024] (seeded), entries N(0,1/n); 256 trajectories x "
                f"2,000 sweeps each, geometric beta 0.1->5.0, one persistent launch per 250-sweep chunk, CUDA graph, "
                f"autotuned {plan.warps} trajectories per CTA")
        attempts = int(sizes.sum()) * T * 2000
        h2d = sum(f.nbytes for f in fs) + beta.nbytes
        upload = lambda: osg.anneal_batched(fs, beta, num_tries=T, resync_every=250, ctx=ctx)
    else:  # sa-n64
        n, T = 64, 100
        f = normal_qubo(n, rank)
        beta = osg.geometric_schedule(0.1, 1.0, 100)
        plan = osg.AnnealPlan(f, beta, num_tries=T, acceptance=osg.ACCEPT_REFERENCE, site_order=osg.SITES_RANDOM,
                              ctx=ctx)
        desc = ("dense SA, n=64, N(0,1) entries (seed 0); 100 trajectories x 100 random-site steps, geometric "
                "beta 0.1->1.0, reference acceptance (the reference CLI's default run)")
        attempts = T * 100
        h2d = f.nbytes + beta.nbytes
        upload = lambda: osg.anneal(f, beta, num_tries=T, ctx=ctx)
    flush_buf = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    launches = []

    def run_one():
        plan.execute()
        launches.append(plan.launches)

    for _ in range(args.warmup):
        run_one()
    torch.cuda.synchronize()
    sampler = ClockSampler(torch.cuda.current_device())
    sampler.start()
    launches.clear()
    steps = args.steps
    step_ms, kern_ms = timed_steps(None, lambda: flush_buf.zero_(), run_one, plan.kernel_ms, steps, 0, pg)
    clocks = sampler.stop()
    res = plan.result()
    if isinstance(res, list):  # batched: aggregate over instances
        acc_total = sum(r.accepted for r in res)
        att_total = sum(r.attempts for r in res)
        # Shared-memory bytes: every accepted flip reads its coupling row.
        smem_bytes = float(sum(4.0 * int(m) * r.accepted for m, r in zip(sizes, res)))

        class _Agg:
            accepted, attempts = acc_total, att_total
            energy = float(np.mean([r.energy for r in res]))
            max_field_drift = max(r.max_field_drift for r in res)
        res = _Agg()
    elif workload == "sa-chimera":
        # Per attempt: the site's field (4 B) and spin (1 B); per accepted
        # flip: the spin write and a read-modify-write of each neighbour's field.
        smem_bytes = 5.0 * res.attempts + res.accepted * (1.0 + 8.0 * avg_deg)
    else:
        smem_bytes = 4.0 * n * res.accepted
    t_step = max_over_ranks(pg, statistics.mean(step_ms))
    value = world * attempts / (t_step * 1e-3)
    e2e_t = []
    for _ in range(max(1 if workload == "sa-batch" else 2, steps // 5)):
        t0 = time.perf_counter()
        r = upload()
        e2e_t.append(time.perf_counter() - t0)
    e2e_step = max_over_ranks(pg, statistics.mean(e2e_t))
    k_ms = statistics.mean(kern_ms)
    peak = osg.probe_smem_row_peak(ctx)
    # The FP32-FMA view: n FMAs per attempt, as a branch-free field update
    # would do them (dense workloads), against the measured FP32 FMA rate.
    fma_peak = osg.probe_fp32_fma_peak(ctx)
    if workload == "sa-batch":
        fmas_per_step = float(T) * 2000 * float((sizes.astype(np.float64) ** 2).sum())
    elif workload == "sa-chimera":
        fmas_per_step = None
    else:
        fmas_per_step = float(attempts) * n
    acc_rate = res.accepted / max(res.attempts, 1)
    # The result counters cover the last executed step.
    achieved = smem_bytes / (k_ms * 1e-3) / 1e9
    roofline = {"bound": "smem", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "peak_source": "os_probe_smem_row_peak (128-bit shared loads + paired FP32 FMAs) measured in this "
                               "run"}
    if workload == "sa-chimera":
        # The sparse sweep is issue-bound: its roofline is issue-slot use,
        # warp instructions per attempt (ncu, SPARSE_WARP_INST_PER_ATTEMPT)
        # times attempts/s over one warp instruction per scheduler per clock.
        sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
        mhz = (clocks or {}).get("sm_mhz") or load_peaks().get("sm_max_mhz", 2070.0)
        issue = attempts / (k_ms * 1e-3) * SPARSE_WARP_INST_PER_ATTEMPT
        issue_peak = sms * 4 * mhz * 1e6
        roofline = {"bound": "issue", "achieved": issue, "peak": issue_peak, "unit": "warp-inst/s",
                    "frac": issue / issue_peak, "warp_inst_per_attempt": SPARSE_WARP_INST_PER_ATTEMPT,
                    "thread_inst_per_attempt": SPARSE_WARP_INST_PER_ATTEMPT * SPARSE_LANES_PER_INST,
                    "smem_view": {"achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak},
                    "peak_source": "SMs x 4 schedulers x median SM clock; instructions per attempt from "
                                   "profiles/sa_sparse_chimera2048.md"}
    out = {
        "metric": "SA spin-flip attempts/s",
        "value": value, "unit": "attempts/s", "ms_per_step": t_step, "dtype": "fp32",
        "config": {"workload": desc, "n": n, "trajectories": T, "attempts_per_step": attempts,
                   "l2": "flushed (256 MB write) before every timed step",
                   "parallelism": f"replicas x{world}" if world > 1 else "1 GPU"},
        "result": {"best_energy": res.energy, "acceptance_rate": acc_rate, "max_field_drift": res.max_field_drift},
        "roofline": {**roofline, "traffic": TRAFFIC.get(workload), "kernel_ms": k_ms,
                     "kernel_attempts_per_s": attempts / (k_ms * 1e-3),
                     "bytes_per_step": smem_bytes,
                     "fp32_fma_view": None if fmas_per_step is None else {
                         "achieved_gflops": 2 * fmas_per_step / (k_ms * 1e-3) / 1e9, "peak_gflops": fma_peak,
                         "frac": 2 * fmas_per_step / (k_ms * 1e-3) / 1e9 / fma_peak,
                         "note": "n FP32 FMAs per attempt over os_probe_fp32_fma_peak"}},
        "e2e": {"value": world * attempts / e2e_step, "unit": "attempts/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(n * T + 8 * T + 8 * 3), "ms_per_step": e2e_step * 1e3},
        "gpu_launches": int(sum(launches)),
        "clocks": clocks,
    }
    plan.close()
    return out


def bench_pt(args, ctx, pg, rank, world):
    """Parallel tempering on the reference's Chimera droplet 512/001 (committed
    fixture): attempts/s and the best energy against the tensor-network ground
    state and the reference's best published SA energy."""
    import torch
    import onesolver_gb300 as osg
    g = json.loads((ROOT / "tests" / "golden" / "chimera_golden.json").read_text())["512"]
    f = osg.Model.load(ROOT / "tests" / "golden" / g["file"]).flatten()
    csr = osg.Csr.from_dense(f)
    n = csr.n
    beta = np.geomspace(0.05, 3.0, 32)
    chains, rounds, spr, resync = 128, 20000, 5, 200
    T = chains * len(beta)
    attempts = T * rounds * spr * n
    run = lambda: osg.temper_sparse(csr, beta, num_chains=chains, num_rounds=rounds, sweeps_per_round=spr,
                                    resync_every=resync, seed=1000 * rank + len(dev_ms), ctx=ctx)
    dev_ms, wall, best, acc = [], [], [], []
    for _ in range(args.warmup):
        run()
    torch.cuda.synchronize()
    barrier(pg)
    sampler = ClockSampler(torch.cuda.current_device())
    sampler.start()
    for _ in range(args.steps):
        t0 = time.perf_counter()
        r = run()
        wall.append(time.perf_counter() - t0)
        dev_ms.append(r.device_ms)
        best.append(r.energy)
        acc.append(r.accepted)
    clocks = sampler.stop()
    barrier(pg)
    t_dev = max_over_ranks(pg, statistics.mean(dev_ms))
    t_e2e = max_over_ranks(pg, statistics.mean(wall))
    launches = 3 + rounds * 2 + rounds // resync + 2
    # Shared-memory bytes of the sweeps, as for the sparse anneal: 5 per
    # attempt (field, spin) and 1 + 8 deg per accepted flip.
    avg_deg = float(csr.row_ptr[-1]) / n
    smem_bytes = 5.0 * attempts + statistics.mean(acc) * (1.0 + 8.0 * avg_deg)
    achieved = smem_bytes / (t_dev * 1e-3) / 1e9
    peak = osg.probe_smem_row_peak(ctx)
    h2d = csr.row_ptr.nbytes + csr.col.nbytes + csr.val.nbytes + csr.diag.nbytes + beta.nbytes
    return {
        "metric": "parallel-tempering spin-flip attempts/s", "value": world * attempts / (t_dev * 1e-3),
        "unit": "attempts/s", "ms_per_step": t_dev, "dtype": "fp32",
        "config": {"workload": f"parallel tempering, Chimera droplet 512/001 (reference fixture), {chains} chains x "
                               f"{len(beta)} temperatures (beta geometric 0.05->3.0), {rounds} rounds x {spr} sweeps, "
                               f"FP64 resync every {resync} rounds",
                   "n": n, "replicas": T, "attempts_per_step": attempts,
                   "timing": "device_ms: CUDA events around the rounds; e2e: the host-buffer call"},
        "result": {"best_energy_per_step": best, "tn_ground_qubo": g["tn_ground_qubo"],
                   "published_best_sa": g["published_best_sa"],
                   "steps_at_tn_ground": sum(abs(b - g["tn_ground_qubo"]) < 1e-6 for b in best),
                   "acceptance_rate": statistics.mean(acc) / attempts},
        "roofline": {"bound": "smem", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": None, "bytes_per_step": smem_bytes,
                     "kernel_ms": t_dev, "note": "device time of the rounds (sweeps, exchanges, resyncs)",
                     "peak_source": "os_probe_smem_row_peak measured in this run"},
        "e2e": {"value": world * attempts / t_e2e, "unit": "attempts/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(n + 8 * chains + 12 * T + 16 * (len(beta) - 1)), "ms_per_step": t_e2e * 1e3},
        "gpu_launches": launches * args.steps,
        "clocks": clocks,
    }


def bench_pa(args, ctx, pg, rank, world):
    """Population annealing on the reference's Chimera droplet 512/001
    (committed fixture): attempts/s, best energy, free-energy estimate."""
    import torch
    import onesolver_gb300 as osg
    g = json.loads((ROOT / "tests" / "golden" / "chimera_golden.json").read_text())["512"]
    f = osg.Model.load(ROOT / "tests" / "golden" / g["file"]).flatten()
    csr = osg.Csr.from_dense(f)
    n = csr.n
    R, K, spb, resync = 16384, 1000, 5, 100
    beta = np.linspace(0.05, 3.0, K)
    attempts = R * K * spb * n
    seeds = iter(range(10 ** 6))
    run = lambda: osg.population_anneal_sparse(csr, beta, population=R, sweeps_per_beta=spb, resync_every=resync,
                                               seed=1000 * rank + next(seeds), ctx=ctx)
    for _ in range(args.warmup):
        run()
    torch.cuda.synchronize()
    barrier(pg)
    sampler = ClockSampler(torch.cuda.current_device())
    sampler.start()
    dev_ms, wall, best, fam, lz = [], [], [], [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        r = run()
        wall.append(time.perf_counter() - t0)
        dev_ms.append(r.device_ms)
        best.append(r.energy)
        fam.append(r.families)
        lz.append(float(r.log_z[-1]))
    clocks = sampler.stop()
    barrier(pg)
    t_dev = max_over_ranks(pg, statistics.mean(dev_ms))
    t_e2e = max_over_ranks(pg, statistics.mean(wall))
    h2d = csr.row_ptr.nbytes + csr.col.nbytes + csr.val.nbytes + csr.diag.nbytes + beta.nbytes
    return {
        "metric": "population-annealing spin-flip attempts/s", "value": world * attempts / (t_dev * 1e-3),
        "unit": "attempts/s", "ms_per_step": t_dev, "dtype": "fp32",
        "config": {"workload": f"population annealing, Chimera droplet 512/001 (reference fixture), {R} replicas, "
                               f"{K} steps of linear beta 0.05->3.0 x {spb} sweeps, systematic resampling",
                   "n": n, "population": R, "attempts_per_step": attempts,
                   "timing": "device_ms: CUDA events around the steps; e2e: the host-buffer call"},
        "result": {"best_energy_per_step": best, "families_per_step": fam, "log_z_final_per_step": lz,
                   "tn_ground_qubo": g["tn_ground_qubo"], "published_best_sa": g["published_best_sa"],
                   "steps_at_tn_ground": sum(abs(b - g["tn_ground_qubo"]) < 1e-6 for b in best)},
        "e2e": {"value": world * attempts / t_e2e, "unit": "attempts/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(n + 8 * K + 8 * R + 12 * R), "ms_per_step": t_e2e * 1e3},
        "gpu_launches": (3 + 4 * K + K // resync + 2) * args.steps,  # per step: min, weights, assign, sweep
        "clocks": clocks,
    }


WARM_BETA_MIN = 2.0  # schedule of the warm-started runs and of their fair-coin control


def bench_learned(args, ctx, pg, rank, world):
    """Time-to-target of the shipped learned warm start on held-out SK seeds."""
    import onesolver_gb300 as osg
    from onesolver_gb300 import warmstart as ws
    sh = ws.load_shipped(ctx)
    meta, net = sh.meta, sh.net
    n = meta["n"]
    k_eval = min(args.learned_eval, len(sh.eval_seeds))
    rows = []
    for k in range(k_eval):
        seed, target = int(sh.eval_seeds[k]), float(sh.targets[k])
        f = ws.sk_qubo(n, seed)
        net.predict(f)                                                      # warm the kernels once
        t0 = time.perf_counter()
        prob = net.predict(f)
        t_pred = time.perf_counter() - t0
        t0 = time.perf_counter()
        gate = ws.probe_gate(f, prob, beta_min=WARM_BETA_MIN, ctx=ctx)
        t_gate = time.perf_counter() - t0
        plain = ws.time_to_target(f, target, ctx=ctx)                       # config schedule, fair coins
        cold = ws.time_to_target(f, target, beta_min=WARM_BETA_MIN, ctx=ctx)  # warm runs' schedule, fair coins
        # The warm arm predicts on the device from each try's own plan
        # (os_sa_plan_warm_start), inside its timed region; the host-path
        # prediction above (predict_s) and the gate's probe runs are reported apart.
        warm = ws.time_to_target(f, target, net=net, beta_min=WARM_BETA_MIN, ctx=ctx)
        warm_s = warm.seconds
        chosen_s = warm_s if gate.use_warm else cold.seconds
        chosen_sw = warm.sweeps if gate.use_warm else cold.sweeps
        rows.append({"seed": seed, "target": target, "use_warm": bool(gate.use_warm),
                     "probe_warm": gate.warm_energy, "probe_cold": gate.cold_energy, "gate_s": t_gate,
                     "plain_sweeps": plain.sweeps, "plain_s": plain.seconds,
                     "cold_sweeps": cold.sweeps, "cold_s": cold.seconds,
                     "warm_sweeps": warm.sweeps, "warm_run_s": warm.seconds, "predict_s": t_pred,
                     "warm_s": warm_s, "chosen_s": chosen_s, "chosen_sweeps": chosen_sw,
                     "prob_abs_dev": float(np.mean(np.abs(prob - 0.5)))})
    net.close()

    def med(key, rs=rows):
        v = [r[key] for r in rs if r[key] is not None]
        return statistics.median(v) if v else None
    succ = lambda key: sum(r[key] is not None for r in rows) / len(rows)
    # Equal success: the seeds every arm solved within the largest budget.
    both = [r for r in rows if r["plain_s"] is not None and r["chosen_s"] is not None and r["cold_s"] is not None
            and r["warm_s"] is not None]
    budgets = (50, 100, 200, 400, 1600)
    at_budget = {str(b): {a: sum(1 for r in rows if r[a + "_sweeps"] is not None and r[a + "_sweeps"] <= b)
                          / len(rows) for a in ("plain", "cold", "warm", "chosen")} for b in budgets}
    value = med("chosen_s", both)
    out = {
        "metric": "SA time-to-target (within 0.5% of a 10^5-sweep plain-SA best), learned warm start with probe "
                  "gate (device-side prediction inside each timed run, probe runs reported apart)",
        "value": value, "unit": "s", "ms_per_step": None, "dtype": "fp32 fields, bf16 network",
        "higher_is_better": False,
        "config": {"workload": f"SK n=1024 J~N(0,1/n); network trained on {meta['train_seeds'][1]} instances "
                               f"(labels: {meta['labels']}); {k_eval} held-out seeds from {meta['eval_seeds'][0]}; "
                               f"target = {meta['targets']}; 512 trajectories per time-to-target run; plain = "
                               f"beta 0.1->5.0 from fair coins; the warm start and its control (fair coins) both run "
                               f"beta {WARM_BETA_MIN}->5.0; the probe gate compares those two",
                   "network": "3 message-passing layers, hidden 64, BF16 tensor-core messages + FP32; node "
                              "features: diagonal, row sum, anchor spin, power-iteration low-spectrum vector (FP32 products, FP64 norms)"},
        "result": {"instances": len(rows), "solved_by_all_arms": len(both),
                   "plain_median_s": med("plain_s", both), "cold_schedule_random_median_s": med("cold_s", both),
                   "warm_median_s": med("warm_s", both), "predict_median_s": med("predict_s"),
                   "gate_median_s": med("gate_s"),
                   "speedup_vs_plain": (med("plain_s", both) / value) if value else None,
                   "network_gain": (med("cold_s", both) / med("warm_s", both))
                   if med("cold_s", both) and med("warm_s", both) else None,
                   "median_sweeps": {"plain": med("plain_sweeps", both), "cold": med("cold_sweeps", both),
                                     "warm": med("warm_sweeps", both)},
                   "success_within_1600_sweeps": {"plain": succ("plain_s"), "cold": succ("cold_s"),
                                                  "warm": succ("warm_s"), "chosen": succ("chosen_s")},
                   "success_at_budget": at_budget,
                   "gate_uses_warm": sum(r["use_warm"] for r in rows),
                   "train_loss_first_last": meta["loss_first_last"], "rows": rows},
        "gpu_launches": None,
    }
    return out


# DRAM bytes (read + write) per launch of the dominant kernel, from one ncu
# capture (dram__bytes_read.sum + dram__bytes_write.sum) of the n = 36
# launch (profiles/exhaustive_gray_n36.md): a constant ~64 KB (coefficients
# and parameters; the per-CTA records stay in L2) whatever the number of
# states. The SA kernels keep their working set on chip for a launch; their
# DRAM bytes per launch depend on the chunk length, not on the attempts, and
# are not reported.
TRAFFIC: dict = {"exhaustive36": 63488}

# Warp instructions per attempt of the sparse sweep kernel and the active
# lanes per instruction, from one ncu capture of the Chimera 2048 profile
# case (smsp__inst_executed.sum over 1,024 trajectories x 50 sweeps x 2,048
# sites; smsp__thread_inst_executed_per_inst_executed.ratio), summarised in
# profiles/sa_sparse_chimera2048.md.
SPARSE_WARP_INST_PER_ATTEMPT = 540055768 / (1024 * 50 * 2048)
SPARSE_LANES_PER_INST = 29.90


# ---------------------------------------------------------------------------
# CPU baselines (the reference's algorithm, restated in oracle/)
# ---------------------------------------------------------------------------

def cpu_exhaustive_rate(f: np.ndarray, budget_s: float, threads: int) -> tuple[float, int, float]:
    import oracle
    oracle.build()
    n = f.shape[0]
    t0 = time.perf_counter()
    probe = 1 << 16
    oracle.exhaustive(f, 0, probe, threads)
    rate = probe / max(time.perf_counter() - t0, 1e-6)
    sample = int(min(1 << n, max(probe, 2 ** int(math.log2(rate * budget_s)))))
    t0 = time.perf_counter()
    oracle.exhaustive(f, 0, sample, threads)
    dt = time.perf_counter() - t0
    return sample / dt, sample, dt


def cpu_sa_rate(workload: str, budget_s: float, threads: int):
    """Reference algorithm (full FP64 energy per attempt) on a bounded sample."""
    import oracle
    import onesolver_gb300 as osg
    oracle.build()
    if workload == "sa-chimera":
        f = chimera_csr(16, 0).to_dense()
        order, acc = 1, 1
        beta = osg.linear_schedule(0.1, 2.9, 10000)
    elif workload == "sa-sk":
        f = sk_qubo(1024, 0)
        order, acc = 1, 1
        beta = osg.geometric_schedule(0.1, 5.0, 1000)
    elif workload == "sa-batch":
        m = int(np.random.default_rng(0).integers(64, 1025, size=512)[0])
        f = normal_qubo(m, 0, scale=1.0 / math.sqrt(m))
        order, acc = 1, 1
        beta = osg.geometric_schedule(0.1, 5.0, 2000)
    else:
        f = normal_qubo(64, 0)
        order, acc = 0, 0
        beta = osg.geometric_schedule(0.1, 1.0, 100)
    n = f.shape[0]
    # One step of `threads` trajectories, growing until the budget is used.
    iters = 1
    while True:
        t0 = time.perf_counter()
        _, _, att = oracle.anneal_free(f, beta[:iters], threads, 1, 1, acc, order, threads)
        dt = time.perf_counter() - t0
        if dt > budget_s / 4 or iters >= len(beta):
            break
        iters = min(len(beta), iters * 4)
    return att / dt, f"{threads} trajectories x {iters} steps ({att} attempts) of the same instance", dt


def reference_arm(args, world, rank):
    """--impl reference: the reference's algorithm on the host cores."""
    if rank != 0:
        return None
    threads = os.cpu_count() or 1
    w = args.workload
    if w in ("pt-droplet", "pa-droplet"):
        return {"impl": "reference", "unavailable": "the reference has no parallel tempering or population "
                                                    "annealing (benchmarks/annealing/performance.md names them as "
                                                    "future work)"}
    vals = []
    sample_desc = ""
    for i in range(args.warmup + args.steps):
        if w == "exhaustive36":
            rate, sample, dt = cpu_exhaustive_rate(int_qubo(36, 0), min(10.0, args.ref_budget), threads)
            sample_desc = (f"states [0, {sample}) of the n=36 instance per step, reference O(n^2) FP64 loop "
                           f"(include/exhaustive/exhaustive.hpp:110-134)")
        else:
            rate, sample_desc, dt = cpu_sa_rate(w, min(10.0, args.ref_budget), threads)
        if i >= args.warmup:
            vals.append(rate)
    value = statistics.mean(vals)
    unit = "states/s" if w == "exhaustive36" else "attempts/s"
    return {"impl": "reference", "metric": METRICS[w], "value": value, "unit": unit, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": CONFIG_NAMES[w]},
            "cpu_baseline": {"value": value, "unit": unit, "cores": threads, "kind": "port", "sample": sample_desc},
            "e2e": {"value": value, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


METRICS = {
    "exhaustive36": "exhaustive enumerated states/s (n=36, int32 Gray code, all degenerate minimisers)",
    "sa-chimera": "SA spin-flip attempts/s",
    "sa-sk": "SA spin-flip attempts/s",
    "sa-batch": "SA spin-flip attempts/s",
    "sa-n64": "SA spin-flip attempts/s",
    "sa-learned": "SA time-to-target, learned warm start vs plain",
    "pt-droplet": "parallel-tempering spin-flip attempts/s",
    "pa-droplet": "population-annealing spin-flip attempts/s",
}
CONFIG_NAMES = {
    "exhaustive36": "exhaustive search, dense QUBO n=36, integer Q_ij ~ U{-8..8} (seed 0), 2^36 states",
    "sa-chimera": "sparse SA, 16x16 Chimera 2048 spins, 1024 trajectories x 10,000 sweeps",
    "sa-sk": "dense SA, SK n=1024, 512 trajectories x 1,000 sweeps",
    "sa-batch": "batched dense SA, 512 instances n~U[64,1024], 256 trajectories x 2,000 sweeps",
    "sa-n64": "dense SA, n=64, 100 trajectories x 100 steps (reference CLI defaults)",
    "sa-learned": "SK n=1024 learned warm start, time-to-target",
    "pt-droplet": "parallel tempering, Chimera droplet 512/001, 128 chains x 32 temperatures x 100,000 sweeps",
    "pa-droplet": "population annealing, Chimera droplet 512/001, 16,384 replicas x 1,000 steps x 5 sweeps",
}


PROFILE_CASES = ("exhaustive32", "exhaustive36", "sa-sk1024", "sa-batch48", "sa-batch128x256", "sa-chimera",
                 "mpnn-predict1024", "pt-droplet512", "pa-droplet512")


def profile_case(name: str, ctx, exh_variant: int = 0) -> None:
    """One small execution of a hot-path kernel, for ncu captures: inputs
    larger than L2 where the kernel streams them, a few GB on the device at
    most, a handful of launches."""
    import torch
    import onesolver_gb300 as osg
    if name in ("exhaustive32", "exhaustive36"):
        plan = osg.ExhaustivePlan(int_qubo(int(name[-2:]), 0), ctx=ctx, max_minimisers=1 << 16,
                                  variant=exh_variant)
    elif name == "sa-sk1024":
        plan = osg.AnnealPlan(sk_qubo(1024, 0), osg.geometric_schedule(0.1, 5.0, 10), num_tries=512,
                              acceptance=osg.ACCEPT_PHYSICAL, site_order=osg.SITES_SEQUENTIAL, ctx=ctx)
    elif name == "sa-batch128x256":
        # the batched configuration's per-CTA shape (256 trajectories, n ~ U[64, 1024]) on a quarter of
        # its instances and 8 sweeps: ~1 GB on the device, one short launch
        rng = np.random.default_rng(0)
        sizes = rng.integers(64, 1025, size=128)
        fs = [normal_qubo(int(m), k, scale=1.0 / math.sqrt(m)) for k, m in enumerate(sizes)]
        plan = osg.BatchedAnnealPlan(fs, osg.geometric_schedule(0.1, 5.0, 8), num_tries=256, ctx=ctx)
    elif name == "sa-batch48":
        rng = np.random.default_rng(0)
        sizes = rng.integers(64, 1025, size=48)
        fs = [normal_qubo(int(m), k, scale=1.0 / math.sqrt(m)) for k, m in enumerate(sizes)]
        plan = osg.BatchedAnnealPlan(fs, osg.geometric_schedule(0.1, 5.0, 8), num_tries=64, ctx=ctx)
    elif name == "sa-chimera":
        plan = osg.AnnealPlan(chimera_csr(16, 0), osg.linear_schedule(0.1, 2.9, 50), num_tries=1024,
                              acceptance=osg.ACCEPT_PHYSICAL, ctx=ctx)
    elif name == "pt-droplet512":
        g = json.loads((ROOT / "tests" / "golden" / "chimera_golden.json").read_text())["512"]
        csr = osg.Csr.from_dense(osg.Model.load(ROOT / "tests" / "golden" / g["file"]).flatten())
        r = osg.temper_sparse(csr, np.geomspace(0.05, 3.0, 32), num_chains=128, num_rounds=20, sweeps_per_round=5,
                              resync_every=200, ctx=ctx)
        torch.cuda.synchronize()
        print(json.dumps({"profile_case": name, "energy": r.energy, "device_ms": r.device_ms}))
        return
    elif name == "pa-droplet512":
        g = json.loads((ROOT / "tests" / "golden" / "chimera_golden.json").read_text())["512"]
        csr = osg.Csr.from_dense(osg.Model.load(ROOT / "tests" / "golden" / g["file"]).flatten())
        r = osg.population_anneal_sparse(csr, np.linspace(0.05, 3.0, 1000)[:20], population=16384,
                                         sweeps_per_beta=5, resync_every=100, ctx=ctx)
        torch.cuda.synchronize()
        print(json.dumps({"profile_case": name, "energy": r.energy, "device_ms": r.device_ms}))
        return
    elif name == "mpnn-predict1024":
        net = osg.WarmStartNet(seed=1, ctx=ctx)
        p = net.predict(sk_qubo(1024, 3))
        torch.cuda.synchronize()
        print(json.dumps({"profile_case": name, "mean_probability": float(p.mean())}))
        net.close()
        return
    else:
        raise SystemExit(f"unknown profile case {name}")
    plan.execute()
    torch.cuda.synchronize()
    r = plan.result()
    e = r[0].energy if isinstance(r, list) else r.energy
    print(json.dumps({"profile_case": name, "launches": plan.launches, "energy": e}))
    plan.close()


def _json_default(o):
    if hasattr(o, "item"):
        return o.item()
    return str(o)


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=0, help="timed steps (default per workload)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=list(METRICS), default="exhaustive36")
    ap.add_argument("--secondary", action=argparse.BooleanOptionalAction, default=True,
                    help="also measure the SA workloads and report them under 'secondary'")
    ap.add_argument("--cpu-baseline", action=argparse.BooleanOptionalAction, default=True)
    ap.add_argument("--ref-budget", type=float, default=8.0, help="seconds of CPU work per reference step")
    ap.add_argument("--exh-variant", type=int, default=0, choices=[0, 1, 2, 3],
                    help="exhaustive instruction variant (0 = the library's default)")
    ap.add_argument("--learned-eval", type=int, default=256,
                    help="held-out seeds of the shipped warm-start model to evaluate (sa-learned)")
    ap.add_argument("--profile-case", choices=PROFILE_CASES, default=None,
                    help="run one small execution of a hot-path kernel (for ncu) and exit")
    args = ap.parse_args()
    if args.profile_case:
        import torch
        import onesolver_gb300 as osg
        ctx = osg.Context(0)
        profile_case(args.profile_case, ctx, args.exh_variant)
        ctx.close()
        return
    if args.steps <= 0:
        args.steps = {"exhaustive36": 50, "sa-chimera": 10, "sa-sk": 5, "sa-batch": 3, "sa-n64": 50,
                      "sa-learned": 1, "pt-droplet": 3, "pa-droplet": 3}[args.workload]
    args.warmup = max(args.warmup, 3)

    world, rank, local, pg = dist_setup(args.gpus)
    if args.impl == "reference":
        out = reference_arm(args, world, rank)
        if out is not None:
            print(json.dumps(out, default=_json_default))
        return

    import torch
    import onesolver_gb300 as osg
    torch.cuda.set_device(local)
    ctx = osg.Context(local)
    # One explicit stream for the library's kernels, the L2 flush and the
    # timing events (the legacy default stream has handle 0, which the C ABI
    # reads as "use the context's own stream").
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)

    if args.workload == "exhaustive36":
        out = bench_exhaustive(args, ctx, pg, rank, world)
    elif args.workload == "sa-learned":
        out = bench_learned(args, ctx, pg, rank, world)
    elif args.workload == "pt-droplet":
        out = bench_pt(args, ctx, pg, rank, world)
    elif args.workload == "pa-droplet":
        out = bench_pa(args, ctx, pg, rank, world)
    else:
        out = bench_sa(args, ctx, pg, rank, world, args.workload)

    if args.secondary and args.workload == "exhaustive36":
        # The SA workloads beside the headline: Chimera (2,048 sites), SK
        # n = 1024 (the learned warm start's family) and the batched dense
        # workload (512 instances; about 14 s per step, so three warm-up
        # steps and one timed step), each with its CPU baseline (the
        # reference's algorithm on the host cores, a bounded sample of the
        # same workload).
        sec = {}
        for w, k, wu in (("sa-chimera", 3, 3), ("sa-sk", 3, 3), ("sa-batch", 1, 3)):
            a2 = argparse.Namespace(**vars(args))
            a2.steps, a2.warmup = k, wu
            r = bench_sa(a2, ctx, pg, rank, world, w)
            sec[w] = {"value": r["value"], "unit": r["unit"], "config": r["config"]["workload"],
                      "steps": k, "warmup": wu, "ms_per_step": r["ms_per_step"],
                      "kernel_attempts_per_s": r["roofline"]["kernel_attempts_per_s"],
                      "roofline": {k2: r["roofline"][k2] for k2 in ("bound", "achieved", "peak", "unit", "frac")},
                      "e2e": r["e2e"]["value"], "result": r["result"], "gpu_launches": r["gpu_launches"]}
            if rank == 0 and world == 1 and args.cpu_baseline:
                threads = os.cpu_count() or 1
                rate, desc, dt = cpu_sa_rate(w, 5.0, threads)
                sec[w]["cpu_baseline"] = {"value": rate, "unit": "attempts/s", "cores": threads, "kind": "port",
                                          "sample": desc + f" ({dt:.1f} s), full FP64 energy per attempt"}
        # The learned warm start's time-to-target on 8 of its held-out seeds.
        a2 = argparse.Namespace(**vars(args))
        a2.learned_eval = 8
        r = bench_learned(a2, ctx, pg, rank, world)
        sec["sa-learned"] = {"value": r["value"], "unit": r["unit"], "higher_is_better": False,
                             "config": r["config"]["workload"],
                             "result": {k: v for k, v in r["result"].items() if k != "rows"}}
        out["secondary"] = sec

    if rank == 0 and world == 1 and args.cpu_baseline and args.workload not in ("sa-learned", "pt-droplet", "pa-droplet"):
        threads = os.cpu_count() or 1
        if args.workload == "exhaustive36":
            rate, sample, dt = cpu_exhaustive_rate(int_qubo(36, 0), 15.0, threads)
            out["cpu_baseline"] = {"value": rate, "unit": "states/s", "cores": threads, "kind": "port",
                                   "sample": f"states [0, {sample}) of the same n=36 instance ({dt:.1f} s), "
                                             f"reference O(n^2) FP64 loop on {threads} threads"}
        else:
            rate, desc, dt = cpu_sa_rate(args.workload, 15.0, threads)
            out["cpu_baseline"] = {"value": rate, "unit": "attempts/s", "cores": threads, "kind": "port",
                                   "sample": desc + f" ({dt:.1f} s), full FP64 energy per attempt"}

    if rank == 0:
        line = {"metric": out["metric"], "value": out["value"], "unit": out["unit"], "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": out["ms_per_step"],
                "higher_is_better": out.get("higher_is_better", True), "scaling": "weak", "vs_baseline": None, "dtype": out["dtype"],
                "data": "synthetic (seeded; shapes and distributions of the configs)", "config": out["config"]}
        for k in ("roofline", "cpu_baseline", "e2e", "gpu_launches", "clocks", "result", "secondary"):
            if k in out:
                line[k] = out[k]
        print(json.dumps(line, default=_json_default))
    ctx.close()
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
