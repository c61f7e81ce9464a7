#!/usr/bin/env python
"""Headline benchmark: Monte Carlo trials/s of the batched semi-grand-canonical workload.

Workload (one GPU): binary FCC alloy, 16x16x16 conventional supercell (16384
sites, periodic), clusters c0, singlet, pairs to the 4th shell, triplets to
the 2nd shell, the nearest-neighbour tetrahedron; seeded ECIs (c0 = -3 eV,
singlet N(0, 0.05), pairs N(0, 0.02/shell), triplets N(0, 0.005), quadruplets
N(0, 0.002)); 64 independent chains on an 8 x 8 grid of T in [300, 1200] K x
mu in [-0.2, 0.2] eV (mu folded into c1_0); single-site flips; energy changes
in FP32, running energy / correlation functions in FP64 with a full FP64
recompute after every step.  One step = 100 sweeps of every chain
(64 x 100 x 16384 trials) in one persistent launch plus the recompute,
replayed from a CUDA graph; 20 steps are the full 2000-sweep budget.

``--impl reference`` times the CPU restatement of the reference's updater and
Metropolis loop on the host cores instead (the reference tree is not present
where this runs, so its compiled updater is not available; the restatement is
bit-identical to it on the pinned fixtures).

Multi-GPU (torchrun, one rank per GPU): independent replicas, no data-path
collective; the barrier and the max-over-ranks timing are the only collectives.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "MC trials/sec, batched FP32-dE vs plain GPU vs CPU ref; job p50/p99 latency"
UNIT = "trials/s"
KB = 8.6173303e-5
L_CELL = 16
N_CHAINS = 64
SWEEPS_PER_STEP = 100
SHELLS = (4, 2, 1)
SPECIES = ["Al", "Mg"]
BYTES_PER_FLIP = None  # 5 * n_cols + 1, set from the model


def workload(seed_offset: int = 0):
    from cemc_gb300.lattice import fcc_settings, seeded_ecis
    from cemc_gb300.tables import CEModel
    from cemc_gb300.batch import sgc_grid, fold_chemical_potential
    s = fcc_settings(L_CELL, *SHELLS, SPECIES)
    eci = seeded_ecis(s.cset, 0)
    m = CEModel(s, list(eci))
    rng = np.random.default_rng(seed_offset)
    occ = np.zeros((N_CHAINS, m.n_sites), dtype=np.int8)
    half = m.n_sites // 2
    for c in range(N_CHAINS):
        occ[c, rng.permutation(m.n_sites)[:half]] = 1  # 50/50 random initial configuration
    Ts, mus = sgc_grid()
    ev = fold_chemical_potential(m, m.eci_vector(eci), mus)
    return s, m, occ, ev, Ts


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def init_dist(world: int, backend: str):
    if world > 1:
        import torch.distributed as dist
        if not dist.is_initialized():
            dist.init_process_group(backend=backend)
        return dist
    return None


def max_over_ranks(value: float, dist, device=None) -> float:
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float, dist, device=None) -> float:
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        import tempfile
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            with open(self.path) as f:
                for line in f:
                    parts = [p.strip() for p in line.split(",")]
                    if len(parts) >= 9 and parts[1].replace(".", "").isdigit():
                        rows.append(parts)
        except Exception:
            pass
        finally:
            try:
                os.unlink(self.path)
            except Exception:
                pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        sm = [float(r[1]) for r in rows]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for n, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": float(rows[0][2]), "reasons": sorted(reasons),
                "samples": len(rows), "power_w_max": max(float(r[3]) for r in rows if r[3] not in ("", "[N/A]"))}


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# Figures of the headline MC kernel that only a profiler measures (one ncu capture of one
# 10-sweep launch of this kernel on this workload, --clock-control none): DRAM bytes read +
# written per launch (the one-time read of the occupations and the neighbour table after the
# L2 flush; it does not grow with the sweep count) and warp instructions issued per cycle on
# the SMs that hold a chain.  They are reported with that source, never as this run's numbers.
# Per kernel form (CEMC_KERNEL_* id): (DRAM bytes per launch, IPC per busy SM, launch captured).
NCU_FIGURES = {3: (4820224.0, 2.23, "one 10-sweep launch"),
               5: (4820992.0, 2.31, "one 2-sweep launch (traffic does not grow with sweeps)"),
               6: (4830976.0, 1.62, "one 10-sweep launch")}
NCU_SOURCE = "ncu capture of the same kernel and workload: "
KERNEL_NAMES = {1: "generic", 2: "spin", 3: "spin half-warp", 4: "table", 5: "local field", 6: "spin quarter-warp"}
KERNEL_CHOICES = {"auto": 0, "generic": 1, "spin": 2, "half": 3, "table": 4, "field": 5, "quarter": 6}


def cpu_port_rate(m, occ, ev, Ts, sample_sweeps: float, threads: int, seed: int = 7):
    """Trials/s of the CPU restatement of the reference path over a bounded sample of the workload."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    orc = O.Oracle(m)
    states = [orc.new_chain_state(occ[c], ev[c], KB * Ts[c], O.MOVE_FLIP) for c in range(len(occ))]
    n_trials = max(1, int(sample_sweeps * m.n_sites))
    t0 = time.perf_counter()
    orc.run_many(states, seed=seed, chain_ids=list(range(len(occ))), t_begin=0, n_trials=n_trials,
                 n_threads=threads)
    dt = time.perf_counter() - t0
    return len(occ) * n_trials / dt, n_trials, dt


def calibrated_cpu_sample(m, occ, ev, Ts, threads: int, target_s: float):
    rate, _, _ = cpu_port_rate(m, occ, ev, Ts, 0.02, threads)
    sweeps = max(0.02, target_s * rate / (len(occ) * m.n_sites))
    return sweeps


def correctness_sample(geo, m, occ, ev, Ts, n_trials: int = 40000, chain: int = N_CHAINS - 1, warps: int = 8,
                       kernel: int = 0):
    """FP32 energy changes vs the FP64 oracle on one chain of the workload (the hottest, highest-acceptance one),
    in the timed batch's warps and kernel form."""
    import torch
    from cemc_gb300 import engine as E
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    kT = KB * Ts[chain]
    cb = E.ChainBatch(geo, occ[chain:chain + 1], ev[chain:chain + 1], kT, E.MOVE_FLIP, seed=77)
    _, acc, de = cb.run(n_trials, precision=E.PREC_F32, warps=warps, kernel=kernel, trace=True)
    torch.cuda.synchronize()
    acc, de = acc.cpu().numpy()[0], de.cpu().numpy()[0]
    orc = O.Oracle(m)
    st = orc.new_chain_state(occ[chain], ev[chain], kT, O.MOVE_FLIP)
    tr = orc.run(st, seed=77, chain_id=0, t_begin=0, n_trials=n_trials, trace=True)
    band = 1e-5 / kT
    margin = np.abs(tr.de / kT + np.log(np.maximum(tr.u, 1e-300)))
    mism = acc != tr.acc
    first = int(np.argmax(mism)) if mism.any() else n_trials
    same = slice(0, first)
    return {"chain": chain, "T": float(Ts[chain]), "trials": n_trials, "accept_rate": float(tr.acc.mean()),
            "max_abs_dE_error_eV": float(np.max(np.abs(de[same] - tr.de[same]))) if first else 0.0,
            "decision_mismatches": int(mism.sum()), "near_threshold_trials": int((margin < band).sum()),
            "band": "|dE/kT + ln u| < 1e-5 eV / kT",
            "final_energy_rel_error": float(abs(cb.energy.item() - st.energy[0]) / abs(st.energy[0]))
            if not mism.any() else None}


def run_served(args):
    """Served stream: Poisson arrivals of mixed jobs through the continuous-batching server."""
    import torch
    from cemc_gb300.server import MCServer, poisson_stream
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    jobs = poisson_stream(args.served_jobs, rate=200.0, seed=rank,
                          sweeps_range=(1e2 * args.served_sweep_scale, 1e4 * args.served_sweep_scale))
    srv = MCServer(quantum_sweeps=1.0, capacity=64, hbm_budget_gb=120.0)
    warm_s = srv.warm(jobs)  # geometries built before the stream starts (a warm server)
    t0 = time.perf_counter()
    i = 0
    while i < len(jobs) or srv.pending or any(g.active() for g in srv.groups.values()):
        now = time.perf_counter() - t0
        while i < len(jobs) and jobs[i].arrival <= now:
            jobs[i].arrival = t0 + jobs[i].arrival
            srv.submit(jobs[i])
            i += 1
        srv.step()
    st = srv.stats()
    if rank == 0:
        print(json.dumps({"metric": METRIC, "workload": "served_stream", "value": st["trials_per_s"], "unit": UNIT,
                          "p50_latency_s": st["p50_latency_s"], "p99_latency_s": st["p99_latency_s"],
                          "p50_admission_wait_s": st["p50_admission_wait_s"],
                          "p99_admission_wait_s": st["p99_admission_wait_s"],
                          "p50_run_s": st["p50_run_s"], "p99_run_s": st["p99_run_s"], "trials": st["trials"],
                          "geometry_warmup_s": warm_s,
                          "jobs": st["jobs"], "wall_s": st["wall_s"], "hbm_used_gb": st["hbm_used_gb"],
                          "config": {"arrivals": "Poisson 200 jobs/s", "n_jobs": args.served_jobs,
                                     "supercells": "4^3-32^3 conventional, log-uniform",
                                     "sweeps": "%g-%g log-uniform" % (1e2 * args.served_sweep_scale,
                                                                     1e4 * args.served_sweep_scale),
                                     "recipes": "binary, binary to 6th shell, ternary; SGC and canonical",
                                     "T": "U[300,1200] K", "hbm_budget_gb": 120}}))
    return 0


def _timed_steps(step, stream, steps: int, warmup: int, local: int):
    """Device time of `steps` calls of step() after `warmup` untimed ones (CUDA events on `stream`)."""
    import torch
    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        a.record(stream)
        for _ in range(steps):
            step()
        b.record(stream)
        torch.cuda.synchronize()
    return a.elapsed_time(b) * 1e-3, clk.summary()


def ternary_shape(m, pair_sites: int = 16384):
    """(warps, CTAs per chain) of a ternary swap batch in the uneven workload: cells of at least
    ``pair_sites`` sites take 16 warps on a CTA pair; smaller ones one CTA with about as many trials
    per round as commit without conflicts (half of n_sites / (2 n_cols sites per swap), 4 .. 16)."""
    if m.n_sites >= pair_sites:
        return 16, 2
    return max(2, min(16, max(4, m.n_sites // (4 * m.n_cols)))), 1


def run_ternary(args):
    """Ternary canonical swaps on 256 chains of uneven supercells in one graph launch per step.

    Ternary FCC {-1, 0, 1} (basis sqrt(3/2) s, sqrt(2)(1 - 1.5 s^2)), pairs to the 5th
    shell, triplets to the 3rd, the nearest-neighbour tetrahedron; seeded ECIs; 256
    chains on conventional cells L^3, L drawn uniformly from 4..24 (256..55296 sites);
    compositions Dirichlet(2, 2, 2) per chain; T = 800 K; FP32 energy changes, FP64
    recompute every step.  Chains of one size share a geometry; every size group runs
    on its own stream inside one CUDA graph, so one graph launch steps all 256 chains.
    """
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from cemc_gb300 import engine as E
    from cemc_gb300.batch import BatchRunner, MultiBatchRunner
    from cemc_gb300.lattice import fcc_settings, seeded_ecis
    from cemc_gb300.tables import CEModel
    rng = np.random.default_rng(1000 + rank)
    sizes = rng.integers(4, 25, args.ternary_chains)
    runners = []
    for L in sorted(set(sizes.tolist())):
        n = int((sizes == L).sum())
        s = fcc_settings(int(L), 5, 3, 1, ["Al", "Mg", "Si"])
        eci = seeded_ecis(s.cset, 0)
        m = CEModel(s, list(eci))
        geo = E.Geometry(m, dev)
        occ = np.zeros((n, m.n_sites), dtype=np.int8)
        for c in range(n):
            comp = rng.dirichlet([2.0, 2.0, 2.0])
            counts = np.floor(comp * m.n_sites).astype(int)
            counts[0] += m.n_sites - counts.sum()
            occ[c] = rng.permutation(np.repeat(np.arange(3), counts))
        warps, cluster = ternary_shape(m, args.ternary_pair_sites)
        runners.append(BatchRunner(geo, occ, m.eci_vector(eci), 800.0, E.MOVE_SWAP, seed=7 + int(L),
                                   precision=E.PREC_F32, warps=args.warps or warps, cluster=args.cluster or cluster,
                                   sweeps_per_step=args.sweeps_per_step, recompute_every=1, graph=True,
                                   chain_keys=np.arange(n) + 1000 * int(L)))
    multi = MultiBatchRunner(runners)
    multi.capture()
    t, clocks = _timed_steps(multi.step, multi.stream, args.steps, args.warmup, local)
    trials = float(multi.trials_per_step * args.steps)
    for r in runners:
        r.cb.check_status()
    if rank == 0:
        print(json.dumps({"metric": METRIC, "workload": "ternary_uneven", "value": trials / t, "unit": UNIT,
                          "ms_per_step": t * 1e3 / args.steps, "steps": args.steps, "warmup": args.warmup,
                          "dtype": "f32", "clocks": clocks,
                          "config": {"workload": "ternary_swap_fcc_uneven_%dchains" % args.ternary_chains,
                                     "n_chains": int(args.ternary_chains), "sizes": "L uniform 4..24",
                                     "groups": len(runners), "sites_total": int(sum(r.n_chains * r.geo.n_sites
                                                                                    for r in runners)),
                                     "sweeps_per_step": args.sweeps_per_step,
                                     "shape": "cells of >= %d sites: 16 warps on a CTA pair; smaller: default "
                                              "width, one CTA" % args.ternary_pair_sites,
                                     "launch": "one CUDA graph per step, one stream per supercell size, "
                                               "largest cells launched first"}}))
    return 0


def run_pt(args):
    """Parallel-tempering ladder: binary FCC 32^3 (131072 sites), 48 replicas, exchange every 10 sweeps.

    Cluster set: pairs to the 6th shell, triplets to the 2nd, the nearest-neighbour
    tetrahedron; seeded ECIs; canonical swaps from a 50/50 random configuration;
    geometric ladder T in [200, 1500] K; FP32 energy changes, FP64 recompute and
    device exchange after every 10-sweep cycle.  One step = one cycle.
    """
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from cemc_gb300 import engine as E
    from cemc_gb300.lattice import fcc_settings, seeded_ecis
    from cemc_gb300.tables import CEModel
    from cemc_gb300.parallel_tempering import ParallelTempering
    s = fcc_settings(32, 6, 2, 1, SPECIES)
    eci = seeded_ecis(s.cset, 0)
    m = CEModel(s, list(eci))
    geo = E.Geometry(m, dev)
    rng = np.random.default_rng(rank)
    occ = np.zeros(m.n_sites, dtype=np.int8)
    occ[rng.permutation(m.n_sites)[: m.n_sites // 2]] = 1
    pt = ParallelTempering(geo, occ, m.eci_vector(eci), temperatures=np.geomspace(200.0, 1500.0, 48),
                           move=E.MOVE_SWAP, seed=11, precision=E.PREC_F32, warps=args.warps or 0)
    stream = torch.cuda.current_stream()
    t, clocks = _timed_steps(lambda: pt.run(sweeps_per_cycle=10.0, num_exchange_cycles=1), stream, args.steps,
                             args.warmup, local)
    trials = 48.0 * 10 * m.n_sites * args.steps
    if rank == 0:
        print(json.dumps({"metric": METRIC, "workload": "parallel_tempering", "value": trials / t, "unit": UNIT,
                          "ms_per_step": t * 1e3 / args.steps, "steps": args.steps, "warmup": args.warmup,
                          "dtype": "f32", "clocks": clocks, "exchanges_accepted": int(pt.n_accept.item()),
                          "config": {"workload": "pt_swap_fcc_binary_32x32x32_48replicas", "n_sites": m.n_sites,
                                     "n_cols": m.n_cols, "replicas": 48, "T": "geometric 200..1500 K",
                                     "sweeps_per_step": 10, "warps_per_cta": pt.warps}}))
    return 0


def run_canonical1(args):
    """One canonical swap chain in FP64: binary FCC 8x8x8 (2048 sites), 50/50 random init (seed 0),
    T = 800 K, the headline cluster set and ECI recipe; 2048 x 1000 swaps per step.

    The GPU form of the reference's plain single-chain run (CPU-runnable size).  Also times the
    CPU restatement of the reference updater and Metropolis loop on one host thread for the same
    chain (a bounded sample)."""
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from cemc_gb300 import engine as E
    from cemc_gb300.lattice import fcc_settings, seeded_ecis
    from cemc_gb300.tables import CEModel
    s = fcc_settings(8, *SHELLS, SPECIES)
    eci = seeded_ecis(s.cset, 0)
    m = CEModel(s, list(eci))
    geo = E.Geometry(m, dev)
    rng = np.random.default_rng(0)
    occ = np.zeros(m.n_sites, dtype=np.int8)
    occ[rng.permutation(m.n_sites)[: m.n_sites // 2]] = 1
    ev = m.eci_vector(eci)
    cb = E.ChainBatch(geo, occ[None], ev, KB * 800.0, E.MOVE_SWAP, seed=0)
    n = m.n_sites * 1000
    stream = cb.stream if cb.stream is not None else torch.cuda.current_stream()
    t, clocks = _timed_steps(lambda: cb.run(n, precision=E.PREC_F64, warps=args.warps or 0), stream, args.steps,
                             args.warmup, local)
    cb.check_status()
    cpu = None
    if rank == 0 and not args.no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        orc = O.Oracle(m)
        st = orc.new_chain_state(occ, ev, KB * 800.0, O.MOVE_SWAP)
        n_cpu = 200000
        t0 = time.perf_counter()
        orc.run(st, seed=0, chain_id=0, t_begin=0, n_trials=n_cpu)
        cpu = {"value": n_cpu / (time.perf_counter() - t0), "unit": UNIT, "cores": 1, "kind": "port",
               "sample": "%d swaps of the same chain on one host thread" % n_cpu}
    if rank == 0:
        print(json.dumps({"metric": METRIC, "workload": "canonical_single_chain", "value": n * args.steps / t,
                          "unit": UNIT, "ms_per_step": t * 1e3 / args.steps, "steps": args.steps,
                          "warmup": args.warmup, "dtype": "f64", "clocks": clocks, "cpu_baseline": cpu,
                          "accept_rate": float(cb.accum_host()[0, E.A_NACC] / max(cb.accum_host()[0, E.A_NSAMP], 1)),
                          "config": {"workload": "canonical_swap_fcc_binary_8x8x8_1chain", "n_sites": m.n_sites,
                                     "trials_per_step": n, "T": 800.0, "precision": "fp64",
                                     "kernel": int(cb.last_kernel), "warps_per_cta": args.warps or "auto"}}))
    return 0


def run_recompute(args):
    """Full correlation-function recompute (cemc_recompute) alone, on the ladder geometry.

    Binary FCC 32x32x32 conventional (131072 sites), pairs to the 6th shell,
    triplets to the 2nd, the nearest-neighbour tetrahedron; 48 chains with
    random 50/50 occupations.  Algorithmic bytes per chain: N * (1 + 4 * n_cols)
    (each site's occupation and its neighbour-table row), plus 8 * n_eci written.
    """
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from cemc_gb300 import engine as E
    from cemc_gb300.lattice import fcc_settings, seeded_ecis
    from cemc_gb300.tables import CEModel
    n_chains = args.recompute_chains
    s = fcc_settings(args.recompute_cell, 6, 2, 1, SPECIES)
    eci = seeded_ecis(s.cset, 0)
    m = CEModel(s, list(eci))
    geo = E.Geometry(m, dev)
    rng = np.random.default_rng(rank)
    occ = rng.integers(0, 2, (n_chains, m.n_sites)).astype(np.int8)
    ev = np.tile(m.eci_vector(eci), (n_chains, 1))
    cb = E.ChainBatch(geo, occ, ev, KB * 800.0, E.MOVE_FLIP, seed=1)
    stream = cb.stream if cb.stream is not None else torch.cuda.current_stream()
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            cb.recompute()
    torch.cuda.synchronize()
    times = []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(1)
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                cb.recompute()
                b.record(stream)
            stream.synchronize()
            times.append(a.elapsed_time(b) * 1e-3)
    t = statistics.median(times)
    alg_bytes = n_chains * (m.n_sites * (1 + 4 * m.n_cols) + 8 * m.n_eci)
    peak, peak_kind = measured_peak()
    achieved = alg_bytes / t / 1e9
    if rank == 0:
        print(json.dumps({"metric": "full correlation-function recompute, algorithmic GB/s", "workload": "recompute",
                          "value": achieved, "unit": "GB/s", "ms_per_call": t * 1e3,
                          "sites_per_s": n_chains * m.n_sites / t, "steps": args.steps, "warmup": args.warmup,
                          "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                                       "frac": achieved / peak, "peak_kind": peak_kind,
                                       "alg_bytes_per_call": alg_bytes},
                          "clocks": clk.summary(),
                          "config": {"workload": "recompute_fcc_binary_%dx%dx%d_%dchains" % ((args.recompute_cell,) * 3
                                                                                             + (n_chains,)),
                                     "n_sites": m.n_sites, "n_cols": m.n_cols, "n_eci": m.n_eci,
                                     "n_chains": n_chains, "l2": "flushed before every call (256 MB write)"}}))
    return 0


def run_reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return 0  # the CPU arm runs on rank 0 only
    s, m, occ, ev, Ts = workload(0)
    threads = os.cpu_count() or 1
    sweeps = calibrated_cpu_sample(m, occ, ev, Ts, threads, target_s=max(1.0, 150.0 / max(1, args.steps + args.warmup)))
    for _ in range(args.warmup):
        cpu_port_rate(m, occ, ev, Ts, sweeps, threads)
    total_trials, total_t = 0, 0.0
    for k in range(args.steps):
        r, n, dt = cpu_port_rate(m, occ, ev, Ts, sweeps, threads, seed=100 + k)
        total_trials += N_CHAINS * n
        total_t += dt
    value = total_trials / total_t
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * total_t / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "sgc_flip_fcc_binary_16x16x16_64chains", "n_sites": m.n_sites,
                   "n_chains": N_CHAINS, "sample_sweeps_per_step": sweeps, "l2": "cpu run"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": "%d chains x %.3f sweeps per step of the same workload on %d host threads "
                                   "(C restatement of the reference CEUpdater + Metropolis loop)"
                                   % (N_CHAINS, sweeps, threads)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def run_gpu(args):
    import torch
    rank, world, local = dist_env()
    dist = init_dist(world, "nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from cemc_gb300 import engine as E
    from cemc_gb300.batch import BatchRunner
    from cemc_gb300.calculator import model_and_geometry

    s, m, occ, ev, Ts = workload(rank)
    geo = E.Geometry(m, dev)
    bytes_per_flip = 5 * m.n_cols + 1
    keys = np.arange(N_CHAINS) + rank * N_CHAINS
    runner = BatchRunner(geo, occ, ev, Ts, E.MOVE_FLIP, seed=2026, precision=E.PREC_F32, warps=args.warps,
                         cluster=args.cluster, kernel=KERNEL_CHOICES[args.kernel],
                         sweeps_per_step=args.sweeps_per_step, recompute_every=1, graph=True, chain_keys=keys)
    stream = runner.stream
    runner.capture()
    trials_per_step = N_CHAINS * runner.trials_per_step

    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)  # > 129 MB L2

    def flush_l2():
        with torch.cuda.stream(stream):
            flush.fill_(1)

    for _ in range(args.warmup):
        runner.step()
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    ev_s = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ev_e = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            flush_l2()
            ev_s[k].record(stream)
            runner.step()
            ev_e[k].record(stream)
        torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    dev_ms = sum(a.elapsed_time(b) for a, b in zip(ev_s, ev_e))
    t_max = max_over_ranks(dev_ms * 1e-3, dist, dev)
    total_trials = sum_over_ranks(float(trials_per_step * args.steps), dist, dev)
    value = total_trials / t_max
    clocks = clk.summary()
    thermo = runner.thermodynamics()
    if args.profile:
        if rank == 0:
            print(json.dumps({"profile_case": True, "value": value, "unit": UNIT, "ms_per_step": t_max * 1e3 / args.steps,
                              "warps_per_cta": runner.warps, "ctas_per_chain": runner.cluster,
                              "sweeps_per_step": args.sweeps_per_step}))
        if dist is not None:
            dist.barrier()
            dist.destroy_process_group()
        return 0

    # -- roofline of the dominant kernel: the MC launch alone, timed on its stream --------
    cb = runner.cb
    kms = []
    for _ in range(3):
        flush_l2()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            a.record(stream)
            cb.run(runner.trials_per_step, precision=E.PREC_F32, warps=runner.warps, cluster=runner.cluster,
                   kernel=runner.kernel)
            b.record(stream)
        stream.synchronize()
        kms.append(a.elapsed_time(b))
    k_ms = statistics.median(kms)
    alg_bytes = bytes_per_flip * trials_per_step
    achieved = alg_bytes / (k_ms * 1e-3) / 1e9
    peak, peak_kind = measured_peak()
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    busy_sms = min(sms, N_CHAINS * max(1, runner.cluster))
    ncu_traffic, ncu_ipc, ncu_launch = NCU_FIGURES.get(int(cb.last_kernel), (None, None, None))

    # -- end to end through the public batched API, host buffers each step ---------------
    occ_h = torch.from_numpy(occ).pin_memory()
    eci_h = torch.from_numpy(np.ascontiguousarray(ev)).pin_memory()
    kT_h = torch.from_numpy(KB * Ts).pin_memory()
    n_out = N_CHAINS * (E.ACCUM_DOUBLES + m.n_eci + 1)
    out_h = torch.empty(n_out, dtype=torch.float64).pin_memory()
    occ_out_h = torch.empty_like(occ_h).pin_memory()
    e2e_steps = max(1, min(args.steps, 5))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        runner.load_state(occ_h, eci_h, kT_h)
        runner.step()
        with torch.cuda.stream(stream):
            packed = torch.cat([cb.accum.reshape(-1), cb.cf.reshape(-1), cb.energy.reshape(-1)])
            out_h.copy_(packed, non_blocking=True)
            occ_out_h.copy_(cb.occ, non_blocking=True)
        stream.synchronize()
    e2e_t = max_over_ranks(time.perf_counter() - t0, dist, dev)
    e2e_value = sum_over_ranks(float(trials_per_step * e2e_steps), dist, dev) / e2e_t
    h2d = occ_h.numel() + eci_h.numel() * 8 + kT_h.numel() * 8
    d2h = n_out * 8 + occ_out_h.numel()

    # -- plain GPU form: one chain per launch, FP64, one sweep per launch, no graph ------
    plain = None
    if rank == 0:
        pb = E.ChainBatch(geo, occ[:1], ev[:1], KB * Ts[:1], E.MOVE_FLIP, seed=5)
        pb.run(m.n_sites, precision=E.PREC_F64, warps=runner.warps, cluster=1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        n_launch = 4
        for _ in range(n_launch):
            pb.run(m.n_sites, precision=E.PREC_F64, warps=runner.warps, cluster=1)
        torch.cuda.synchronize()
        plain = n_launch * m.n_sites / (time.perf_counter() - t0)

    corr = (correctness_sample(geo, m, occ, ev, Ts, warps=runner.warps, kernel=runner.kernel)
            if rank == 0 and not args.no_correctness else None)

    # -- CPU baseline on a bounded sample (rank 0) --------------------------------------
    cpu = None
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        sweeps = calibrated_cpu_sample(m, occ, ev, Ts, threads, target_s=args.cpu_seconds)
        rate, n, dt = cpu_port_rate(m, occ, ev, Ts, sweeps, threads)
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": "%d chains x %.3f sweeps (%.1f s) of the same workload on %d host threads "
                         "(C restatement of the reference CEUpdater + Metropolis loop)"
                         % (N_CHAINS, sweeps, dt, threads)}

    if rank == 0:
        n_launches = 3 * args.steps  # per step: the MC kernel and the two recompute kernels
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_max * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "sgc_flip_fcc_binary_16x16x16_64chains", "n_sites": m.n_sites,
                       "n_chains": N_CHAINS, "sweeps_per_step": args.sweeps_per_step, "recompute": "fp64 every step",
                       "warps_per_cta": runner.warps, "ctas_per_chain": runner.cluster,
                       "kernel": KERNEL_NAMES.get(int(cb.last_kernel), str(cb.last_kernel)), "cuda_graph": True,
                       "l2": "flushed between timed steps (256 MB write)", "parallelism": "replicas"},
            "gpu_launches": n_launches,
            "clocks": clocks,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": ncu_traffic,
                         "traffic_source": NCU_SOURCE + ncu_launch if ncu_launch else None,
                         "peak_kind": peak_kind,
                         "kernel": "field_kernel<float>" if cb.last_kernel == E.KERNEL_FIELD
                         else "mc_kernel<float, flip, %s>" % KERNEL_NAMES.get(int(cb.last_kernel), ""),
                         "kernel_ms": k_ms,
                         "alg_bytes_per_trial": bytes_per_flip,
                         "note": "HBM does not bind: after the first sweep the kernel works from shared memory "
                                 "and L2; the issue bound below is the one that binds"},
            "issue_bound": {"sms_holding_a_chain": busy_sms, "sms": sms, "sm_fraction": busy_sms / sms,
                            "ipc_per_busy_sm": ncu_ipc, "ipc_source": NCU_SOURCE + ncu_launch if ncu_launch else None,
                            "frac_of_gpu_issue": ncu_ipc * busy_sms / (4.0 * sms) if ncu_ipc else None},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "plain_gpu": {"value": plain, "unit": UNIT,
                          "form": "one chain per launch, FP64 energy change, one sweep per launch, no graph"},
            "cpu_baseline": cpu,
            "correctness": corr,
            "thermo_sample": {"chain0": thermo[0], "chain63": thermo[-1]},
        }
        print(json.dumps(line))
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def main(argv=None):
    p = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--warps", type=int, default=0, help="evaluating warps per CTA (0 = autotuned with --cluster)")
    p.add_argument("--cluster", type=int, default=0, help="CTAs per chain, 1 or 2 (0 = chosen by the library)")
    p.add_argument("--kernel", default="auto", choices=sorted(KERNEL_CHOICES),
                   help="kernel form of the headline batch with --warps given (auto: the library's choice; "
                        "with --warps 0 the autotuner chooses)")
    p.add_argument("--cpu-seconds", type=float, default=15.0)
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--sweeps-per-step", type=float, default=SWEEPS_PER_STEP)
    p.add_argument("--no-correctness", action="store_true")
    p.add_argument("--workload", default="sgc64", choices=["sgc64", "served", "recompute", "ternary", "pt", "canonical1"],
                   help="sgc64: the headline 64-chain batch; served: the Poisson job stream; "
                        "recompute: the full correlation-function recompute alone; ternary: 256 ternary "
                        "chains of uneven size in one graph launch; pt: the 48-replica tempering ladder; "
                        "canonical1: one FP64 canonical chain of 2048 sites")
    p.add_argument("--ternary-chains", type=int, default=256)
    p.add_argument("--ternary-pair-sites", type=int, default=16384,
                   help="ternary cells of at least this many sites run on CTA pairs")
    p.add_argument("--recompute-cell", type=int, default=32)
    p.add_argument("--recompute-chains", type=int, default=48)
    p.add_argument("--served-jobs", type=int, default=300)
    p.add_argument("--served-sweep-scale", type=float, default=0.1,
                   help="scale of the served jobs' sweep budgets (1 = 10^2-10^4 sweeps)")
    p.add_argument("--profile", action="store_true",
                   help="profiling case: the timed steps only (no end-to-end, plain-GPU or CPU legs)")
    args = p.parse_args(argv)
    if args.warmup < 3:
        p.error("at least 3 warm-up steps")
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "served":
        return run_served(args)
    if args.workload == "recompute":
        return run_recompute(args)
    if args.workload == "ternary":
        return run_ternary(args)
    if args.workload == "pt":
        return run_pt(args)
    if args.workload == "canonical1":
        return run_canonical1(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
