"""Continuous-batching Monte Carlo job server on one GPU.

The reference is a single-process library with no server; this module is the
serving layer the batched kernels make possible.  Jobs (a supercell and
cluster set -- one of the built-in recipes or the job's own settings object --,
ECIs, ensemble, a temperature / chemical-potential schedule, sweep budgets)
arrive at any time.  Jobs that share a geometry (supercell size and cluster set)
share a device-resident slot batch; each batch advances all of its occupied
slots by one quantum in ONE launch of the fused kernel on its own CUDA
stream, so batches of different geometries overlap on the device.  A job is
admitted as soon as a slot of its batch is free and its state fits the HBM
budget; it leaves when its budget is spent, and its slot is reused by the
next launch of its batch.

The loop is event driven: each batch keeps at most one launch in flight and
is relaunched as soon as a CUDA event says its previous launch finished, so a
batch of small supercells never waits for one of large supercells.  A batch's
quantum (trials per slot per launch) is max(quantum_sweeps * N,
quantum_trials): small supercells run many sweeps per launch (most of their
jobs finish in one), large ones a few.  It depends on the geometry only, so a
job's launches split its trials the same way alone or in any mix.

A job's trials depend only on (seed, job key, trial index) and on its own
state, and every quantum ends with the same FP64 recompute, so a job's result
is the same whether it runs alone or in a mix (tested).

Device memory is budgeted: every geometry's tables (their exact size from the
library), every batch's slots (occupations, site lists, correlation
functions, ECIs, running sums), its recompute scratch and its conflict tables
count against ``hbm_budget_gb``.  A job whose batch or geometry does not fit
waits; batches without jobs are released (least recently used first, with
their geometry when no other batch uses it) when a waiting job needs the room.
"""
from __future__ import annotations

import hashlib
import itertools
import math
import threading
import time
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Tuple

import numpy as np
import torch

from . import _lib
from . import engine as E
from .batch import KB_EV
from .lattice import fcc_settings, seeded_ecis
from .tables import CEModel

# Cluster recipes of the benchmark configurations: (pair shells, triplet shells, quad shells, species)
RECIPES: Dict[str, Tuple[int, int, int, Tuple[str, ...]]] = {
    "binary": (4, 2, 1, ("Al", "Mg")),
    "binary6": (6, 2, 1, ("Al", "Mg")),
    "ternary": (5, 3, 1, ("Al", "Mg", "Si")),
}


@dataclass
class Job:
    """One Monte Carlo job.

    ``occ`` (species ids) defaults to a random configuration at ``composition``
    (fractions per species, default equal); ``eci`` defaults to the seeded
    recipe ECIs; ``mu`` is folded into ``c1_0`` for semi-grand-canonical jobs.

    ``settings``: the job's own settings object (anything ``tables.CEModel``
    accepts: the CLEASE-style attributes the reference's CE updater reads),
    used instead of the built-in recipe; ``eci`` is then required and names
    the cluster set.  ``schedule``: a list of (sweeps, T, mu) segments run one
    after the other (annealing, chemical-potential scans); it replaces
    ``sweeps``, ``T`` and ``mu``, and the result carries the averages of each
    segment under ``"segments"``.
    """

    L: int
    recipe: str = "binary"
    ensemble: str = "sgc"  # "sgc" (flips) or "canonical" (swaps)
    T: float = 800.0
    mu: float = 0.0
    sweeps: float = 100.0
    seed: int = 0
    eci: Optional[Dict[str, float]] = None
    occ: Optional[np.ndarray] = None
    composition: Optional[List[float]] = None
    settings: Optional[object] = None
    schedule: Optional[List[Tuple[float, float, float]]] = None
    job_id: int = -1
    arrival: float = 0.0
    admitted: float = float("nan")
    done: float = float("nan")
    result: Optional[dict] = None

    @property
    def latency(self) -> float:
        return self.done - self.arrival

    def segments(self) -> List[Tuple[float, float, float]]:
        if self.schedule:
            return [(float(sw), float(T), float(mu)) for sw, T, mu in self.schedule]
        return [(float(self.sweeps), float(self.T), float(self.mu))]


def group_bytes(geo: E.Geometry, model: CEModel, move: int, capacity: int) -> int:
    """Device bytes of a batch of ``capacity`` slots: per slot the occupation, (swaps) the site
    lists, correlation functions and ECIs, energy, temperature, trial counter, status, key,
    trial budget and running sums; the batch's recompute scratch; exact conflict tables for
    supercells above ``engine.STAMP_GLOBAL_SITES``."""
    n = model.n_sites
    per_slot = n + (8 * n if move == E.MOVE_SWAP else 0) + 16 * model.n_eci + 8 * E.ACCUM_DOUBLES + 48
    if move == E.MOVE_SWAP:
        per_slot += 8 * model.n_sym
    total = capacity * per_slot + 8 * max(geo.scratch_doubles(capacity), 1)
    if n > E.STAMP_GLOBAL_SITES:
        total += 4 * geo.stamp_words(capacity)
    return int(total)


class _Group:
    """Slots of one (geometry, move) pair resident on the device."""

    def __init__(self, server: "MCServer", key, model: CEModel, geo: E.Geometry, move: int, capacity: int):
        self.key = key
        self.model = model
        self.geo = geo
        self.move = move
        self.capacity = capacity
        self.stream = torch.cuda.Stream(device=geo.device)
        n = model.n_sites
        occ = np.zeros((capacity, n), dtype=np.int8)
        occ[:, : n // 2] = 1  # placeholder configurations (two species present) until slots fill
        with torch.cuda.stream(self.stream):
            self.cb = E.ChainBatch(geo, occ, np.zeros(model.n_eci), 1.0, move, seed=server.seed, stream=self.stream)
        self.jobs: List[Optional[Job]] = [None] * capacity
        self.remaining = np.zeros(capacity, dtype=np.int64)  # trials left in each slot's current segment
        self.seg = np.zeros(capacity, dtype=np.int64)        # index of each slot's current segment
        self.base_eci: List[Optional[np.ndarray]] = [None] * capacity
        self.seg_results: List[list] = [[] for _ in range(capacity)]
        self.last_used = time.perf_counter()
        self.chain_trials = torch.zeros(capacity, dtype=torch.int64, device=geo.device)
        self.bytes = group_bytes(geo, model, move, capacity)
        self.launched = False
        self.inflight = False
        self.ev_done = torch.cuda.Event()
        self.launch_trials = 0       # trials of the launch in flight
        self.quantum = max(1, int(round(max(server.quantum * n, server.quantum_trials))))  # trials per slot
        # Launch shape: small supercells on one SM per chain; large ones over a CTA pair (two
        # SMs, rounds twice as wide) when the pair's shared memory fits (cemc_run decides).
        self.warps, self.cluster = (server.warps, 1) if n < server.pair_sites else (server.warps, 0)
        self.dirty = []  # slots loaded since the last launch: recomputed together before it

    def free_slot(self) -> int:
        for i, j in enumerate(self.jobs):
            if j is None:
                return i
        return -1

    def active(self) -> int:
        return sum(j is not None for j in self.jobs)


class MCServer:
    """Request loop: admit, tick, retire.

    :param hbm_budget_gb: device memory the server may hold in chain state and tables.
    :param quantum_sweeps: at least this many sweeps per job per launch of its batch.
    :param quantum_trials: at least this many trials per job per launch of its batch.
    :param pair_sites: supercells of at least this many sites run a CTA pair per chain where the
        library finds it fits; smaller ones one CTA.
    :param capacity: slots per geometry batch (fewer for large supercells: about 2^20 sites per batch).
    :param capacity: slots per geometry batch.
    """

    def __init__(self, device="cuda", hbm_budget_gb: float = 120.0, quantum_sweeps: float = 10.0, capacity: int = 64,
                 precision: int = E.PREC_F32, warps: int = 16, seed: int = 2026, kB: float = KB_EV,
                 quantum_trials: int = 1 << 18, pair_sites: int = 8192):
        self.device = E.require_cuda(device)
        self.budget = hbm_budget_gb * 1e9
        self.used = 0.0
        self.quantum = float(quantum_sweeps)
        self.capacity = int(capacity)
        self.precision = precision
        self.warps = warps
        self.seed = int(seed)
        self.kB = kB
        self.groups: Dict[tuple, _Group] = {}
        self.models: Dict[tuple, Tuple[CEModel, E.Geometry, dict]] = {}
        self.pending: List[Job] = []
        self.finished: List[Job] = []
        self._ids = itertools.count()
        self._lock = threading.Lock()
        self.trials_done = 0
        self.t_start = None
        self.quantum_trials = int(quantum_trials)
        self.pair_sites = int(pair_sites)
        self.peak_used = 0.0
        self._settings_keys: Dict[int, tuple] = {}

    # -- submission ------------------------------------------------------------------
    def submit(self, job: Job) -> Job:
        with self._lock:
            if job.job_id < 0:
                job.job_id = next(self._ids)
            if not job.arrival:
                job.arrival = time.perf_counter()
            self.pending.append(job)
        return job

    def _model_key(self, job: Job):
        if job.settings is None:
            return (job.L, job.recipe)
        key = self._settings_keys.get(id(job.settings))
        if key is None:
            if job.eci is None:
                raise ValueError("a job with its own settings needs its ECIs")
            m = CEModel(job.settings, list(job.eci))
            h = hashlib.sha1()
            for arr in (m.gpu_table, m.term_eci, m.term_ref, m.term_size, m.term_nb, m.bf, m.eci_weight):
                h.update(np.ascontiguousarray(arr).tobytes())
            h.update(("|".join(m.eci_names) + "#" + "|".join(m.symbols)).encode())
            key = ("settings", h.hexdigest())
            self._settings_keys[id(job.settings)] = key
            self._built = (key, m, job.settings)  # reused by _model below
        return key

    def _model(self, job: Job):
        """The job's model and device geometry (built on first use); None while it does not fit the budget."""
        key = self._model_key(job)
        hit = self.models.get(key)
        if hit is None:
            built = getattr(self, "_built", None)
            if built is not None and built[0] == key:
                m, eci = built[1], dict(job.eci)
                self._built = None
            elif job.settings is not None:
                m, eci = CEModel(job.settings, list(job.eci)), dict(job.eci)
            else:
                ps, ts, qs, species = RECIPES[job.recipe]
                s = fcc_settings(job.L, ps, ts, qs, list(species))
                eci = seeded_ecis(s.cset, 0)
                m = CEModel(s, list(eci))
            geo = E.Geometry(m, self.device)
            nbytes = geo.device_bytes()
            if nbytes + group_bytes(geo, m, E.MOVE_FLIP, 1) > self.budget:
                geo.close()
                raise MemoryError("the job's geometry does not fit the device-memory budget")
            if self.used + nbytes > self.budget and not self._release_idle(nbytes):
                geo.close()
                return None
            self._account(nbytes)
            hit = (m, geo, eci, job.settings)
            self.models[key] = hit
        return hit[:3]

    def _account(self, nbytes: float):
        self.used += nbytes
        self.peak_used = max(self.peak_used, self.used)

    def _release_idle(self, need: float) -> bool:
        """Free batches without jobs (least recently used first), and geometries no batch uses, until
        ``need`` more bytes fit the budget; True when they do."""
        idle = sorted((g for g in self.groups.values() if not g.active() and not g.inflight),
                      key=lambda g: g.last_used)
        for grp in idle:
            if self.used + need <= self.budget:
                break
            del self.groups[grp.key]
            self.used -= grp.bytes
            gkey = grp.key[:-1]
            grp.cb = None
            if not any(k[:-1] == gkey for k in self.groups):
                m, geo, _, _ = self.models.pop(gkey)
                self.used -= geo.device_bytes()
                geo.close()
        return self.used + need <= self.budget

    def _capacity(self, m: CEModel) -> int:
        return int(min(self.capacity, max(4, (1 << 20) // m.n_sites)))

    def warm(self, jobs) -> float:
        """Build the geometries the given jobs need ahead of time (a warm server); returns seconds."""
        t0 = time.perf_counter()
        for job in jobs:
            if self._model(job) is None:
                break
        torch.cuda.synchronize()
        return time.perf_counter() - t0

    def _job_state(self, job: Job, m: CEModel, default_eci: dict):
        rng = np.random.default_rng(job.seed)
        if job.occ is not None:
            occ = np.asarray(job.occ, dtype=np.int8)
        else:
            comp = np.asarray(job.composition if job.composition is not None else [1.0] * m.n_sym, dtype=float)
            comp = comp / comp.sum()
            counts = np.floor(comp * m.n_sites).astype(int)
            counts[0] += m.n_sites - counts.sum()
            occ = np.repeat(np.arange(m.n_sym, dtype=np.int8), counts)
            rng.shuffle(occ)
        eci = dict(default_eci if job.eci is None else job.eci)
        return occ, m.eci_vector(eci)

    def _segment_eci(self, grp: _Group, slot: int, mu: float) -> np.ndarray:
        ev = grp.base_eci[slot].copy()
        if grp.jobs[slot].ensemble == "sgc":
            ev[grp.model.eci_names.index("c1_0")] -= mu  # sgc_montecarlo.py:239-261
        return ev

    def _admit(self):
        """Place pending jobs (arrival order) into free slots while memory allows."""
        with self._lock:
            pending = list(self.pending)
        admitted = []
        rejected = []
        for job in pending:
            try:
                hit = self._model(job)
            except MemoryError as exc:  # can never run within the budget: hand it back with the reason
                job.result = {"error": str(exc)}
                job.admitted = job.done = time.perf_counter()
                rejected.append(job)
                continue
            if hit is None:
                continue  # its geometry does not fit yet
            m, geo, eci0 = hit
            move = E.MOVE_FLIP if job.ensemble == "sgc" else E.MOVE_SWAP
            gkey = self._model_key(job) + (move,)
            grp = self.groups.get(gkey)
            if grp is None:
                need = group_bytes(geo, m, move, self._capacity(m))
                if need + geo.device_bytes() > self.budget:
                    job.result = {"error": "the job's batch does not fit the device-memory budget"}
                    job.admitted = job.done = time.perf_counter()
                    rejected.append(job)
                    continue
                if self.used + need > self.budget and not self._release_idle(need):
                    continue
                if gkey[:-1] not in self.models:  # the release took this job's own idle geometry
                    continue
                grp = _Group(self, gkey, m, geo, move, self._capacity(m))
                self.groups[gkey] = grp
                self._account(grp.bytes)
            slot = grp.free_slot()
            if slot < 0:
                continue
            occ, ev = self._job_state(job, m, eci0)
            self._load_slot(grp, slot, job, occ, ev)
            job.admitted = time.perf_counter()
            admitted.append(job)
        if admitted or rejected:
            self.finished.extend(rejected)
            with self._lock:
                ids = {j.job_id for j in admitted + rejected}
                self.pending = [j for j in self.pending if j.job_id not in ids]

    def _load_slot(self, grp: _Group, slot: int, job: Job, occ: np.ndarray, ev: np.ndarray):
        cb = grp.cb
        m = grp.model
        grp.jobs[slot] = job
        grp.base_eci[slot] = ev
        grp.seg[slot] = 0
        grp.seg_results[slot] = []
        sweeps, T, mu = job.segments()[0]
        with torch.cuda.stream(grp.stream):
            cb.occ[slot].copy_(torch.as_tensor(occ))
            cb.eci[slot].copy_(torch.as_tensor(self._segment_eci(grp, slot, mu)))
            cb.kT[slot] = self.kB * T
            cb.trial[slot] = 0
            # the stream of a job depends on its own seed only, never on its slot or arrival order
            cb.chain_key[slot] = (job.seed * 2654435761 + 97) & 0x7FFFFFFF
            if grp.move == E.MOVE_SWAP:
                from .engine import build_tracker
                trk, loc, start, count = build_tracker(occ[None], m.n_sym, m.background)
                cb.trk[slot].copy_(torch.as_tensor(trk[0]))
                cb.loc[slot].copy_(torch.as_tensor(loc[0]))
                cb.trk_start[slot].copy_(torch.as_tensor(start[0]))
                cb.trk_count[slot].copy_(torch.as_tensor(count[0]))
        grp.dirty.append(slot)
        grp.remaining[slot] = max(1, int(round(sweeps * m.n_sites)))

    # -- the loop ----------------------------------------------------------------------
    def _launch(self, grp: _Group):
        """One quantum of every occupied slot of a batch, asynchronous on its stream."""
        if grp.dirty:
            # newly loaded slots: one recompute of the batch (cf, energy), then fresh running sums
            with torch.cuda.stream(grp.stream):
                grp.cb.recompute()
                idx = torch.as_tensor(grp.dirty, device=grp.cb.accum.device)
                grp.cb.accum[idx] = 0.0
                grp.cb.accum[idx, E.A_EREF] = grp.cb.energy[idx]
            grp.dirty = []
        grp.last_used = time.perf_counter()
        per = np.minimum(grp.remaining, grp.quantum)
        per[[j is None for j in grp.jobs]] = 0
        n_max = int(per.max())
        if n_max == 0:
            return False
        with torch.cuda.stream(grp.stream):
            grp.chain_trials.copy_(torch.as_tensor(per), non_blocking=False)
            grp.cb.run(n_max, precision=self.precision, warps=grp.warps, chain_trials=grp.chain_trials,
                       cluster=grp.cluster)
            if not grp.cb.recomputed:
                grp.cb.recompute()
            grp.ev_done.record(grp.stream)
        grp.remaining -= per
        grp.launch_trials = int(per.sum())
        self.trials_done += grp.launch_trials
        grp.inflight = True
        return True

    def _finish(self, grp: _Group):
        """The batch's launch is done: hand out its finished jobs."""
        grp.inflight = False
        self._retire([grp])

    def _tick(self):
        """Relaunch every batch whose previous launch finished; returns the batches launched."""
        launched = []
        for grp in self.groups.values():
            if grp.inflight:
                if not grp.ev_done.query():
                    continue
                self._finish(grp)
            if grp.active() and self._launch(grp):
                launched.append(grp)
        return launched

    def _segment_result(self, grp: _Group, i: int, acc, energy, cf, kT, sweeps, mu) -> dict:
        a = acc[i]
        n = max(a[E.A_NSAMP], 1.0)
        mean = a[E.A_EREF] + a[E.A_SUM_E] / n
        T = kT[i] / self.kB
        return {"temperature": T, "mu": mu, "sweeps": sweeps, "energy": mean, "final_energy": float(energy[i]),
                "heat_capacity": (a[E.A_SUM_E2] / n - (a[E.A_SUM_E] / n) ** 2) / (self.kB * T * T),
                "singlet_c1_0": a[E.A_SUM_S] / n, "accept_rate": a[E.A_NACC] / n, "n_mc_steps": int(a[E.A_NSAMP]),
                "cf": cf[i].copy()}

    def _retire(self, groups: List[_Group]):
        """After a batch's launch: close finished segments, start the next one, hand out finished jobs."""
        for grp in groups:
            grp.stream.synchronize()
            grp.cb.check_status()
            ends = [i for i, j in enumerate(grp.jobs) if j is not None and grp.remaining[i] <= 0]
            if not ends:
                continue
            acc = grp.cb.accum_host()
            energy = grp.cb.energy.cpu().numpy()
            cf = grp.cb.cf.cpu().numpy()
            kT = grp.cb.kT.cpu().numpy()
            now = time.perf_counter()
            for i in ends:
                job = grp.jobs[i]
                segs = job.segments()
                k = int(grp.seg[i])
                res = self._segment_result(grp, i, acc, energy, cf, kT, segs[k][0], segs[k][2])
                grp.seg_results[i].append(res)
                if k + 1 < len(segs):
                    # next segment: its temperature and chemical potential, fresh running sums
                    sweeps, T, mu = segs[k + 1]
                    grp.seg[i] = k + 1
                    grp.remaining[i] = max(1, int(round(sweeps * grp.model.n_sites)))
                    with torch.cuda.stream(grp.stream):
                        grp.cb.kT[i] = self.kB * T
                        grp.cb.eci[i].copy_(torch.as_tensor(self._segment_eci(grp, i, mu)))
                    grp.dirty.append(i)
                    continue
                job.result = dict(res)
                job.result["occupation"] = grp.cb.occ[i].cpu().numpy().copy()
                if job.schedule:
                    job.result["segments"] = grp.seg_results[i]
                job.done = now
                grp.jobs[i] = None
                self.finished.append(job)

    def step(self) -> int:
        """Admit, relaunch finished batches, hand out results once; returns the number of active jobs."""
        if self.t_start is None:
            self.t_start = time.perf_counter()
        self._admit()
        launched = self._tick()
        if not launched:
            # nothing could start: wait for the first batch in flight instead of spinning
            busy = [g for g in self.groups.values() if g.inflight]
            if busy:
                for _ in range(200):
                    if any(g.ev_done.query() for g in busy):
                        break
                    time.sleep(0.0002)
        return sum(g.active() for g in self.groups.values())

    def run_until_idle(self, max_ticks: int = 10 ** 9):
        for _ in range(max_ticks):
            active = self.step()
            with self._lock:
                waiting = len(self.pending)
            if active == 0 and waiting == 0:
                break

    def stats(self) -> dict:
        lat = np.array([j.latency for j in self.finished]) if self.finished else np.zeros(1)
        wait = np.array([j.admitted - j.arrival for j in self.finished]) if self.finished else np.zeros(1)
        run = np.array([j.done - j.admitted for j in self.finished]) if self.finished else np.zeros(1)
        wall = (time.perf_counter() - self.t_start) if self.t_start else 0.0
        return {"jobs": len(self.finished), "p50_latency_s": float(np.percentile(lat, 50)),
                "p99_latency_s": float(np.percentile(lat, 99)),
                "p50_admission_wait_s": float(np.percentile(wait, 50)),
                "p99_admission_wait_s": float(np.percentile(wait, 99)),
                "p50_run_s": float(np.percentile(run, 50)), "p99_run_s": float(np.percentile(run, 99)),
                "trials": self.trials_done,
                "trials_per_s": self.trials_done / wall if wall > 0 else 0.0, "wall_s": wall,
                "hbm_used_gb": self.used / 1e9, "hbm_peak_gb": self.peak_used / 1e9}


def poisson_stream(n_jobs: int, rate: float, seed: int = 0, L_range=(4, 32), sweeps_range=(1e2, 1e4),
                   T_range=(300.0, 1200.0), recipes=("binary", "ternary", "binary6"), mu_range=(-0.2, 0.2)):
    """Synthetic served stream: Poisson arrivals, log-uniform supercells and budgets, uniform T."""
    rng = np.random.default_rng(seed)
    t = 0.0
    jobs = []
    for i in range(n_jobs):
        t += rng.exponential(1.0 / rate)
        L = int(round(math.exp(rng.uniform(math.log(L_range[0]), math.log(L_range[1])))))
        sweeps = float(math.exp(rng.uniform(math.log(sweeps_range[0]), math.log(sweeps_range[1]))))
        recipe = recipes[int(rng.integers(len(recipes)))]
        ens = "sgc" if rng.random() < 0.5 else "canonical"
        jobs.append(Job(L=max(L, 4), recipe=recipe, ensemble=ens, T=float(rng.uniform(*T_range)),
                        mu=float(rng.uniform(*mu_range)), sweeps=sweeps, seed=i + 1, arrival=t))
    return jobs
