"""Batched execution: many chains of one geometry stepped by one persistent launch.

A *step* is ``sweeps_per_step`` sweeps (sweep = n_sites trials) of every chain
in ONE ``cemc_run`` launch, followed by the FP64 full recompute that resets
the drift of the running correlation functions and energy (every
``recompute_every`` steps).  The step is captured once into a CUDA graph and
replayed, so a run of S steps issues S graph launches and nothing else.

This replaces the reference's one-Python-call-per-trial loop
(cemc/mcmc/montecarlo.py:802-837) for whole batches of independent chains.
"""
from __future__ import annotations

from typing import Dict, List, Optional, Sequence

import numpy as np
import torch

from . import engine as E
from .engine import ChainBatch, Geometry

KB_EV = 8.6173303e-5  # Boltzmann constant in eV/K (cpp/src/linear_vib_correction.cpp:3)


class BatchRunner:
    def __init__(self, geo: Geometry, occ, eci, temperatures, move: int, seed: int = 0,
                 precision: int = E.PREC_F32, warps: int = 0, sweeps_per_step: float = 1.0,
                 recompute_every: int = 1, graph: bool = True, chain_keys=None, kB: float = KB_EV,
                 stream: Optional[torch.cuda.Stream] = None, cluster: int = 0, kernel: int = E.KERNEL_AUTO):
        self.geo = geo
        self.kB = kB
        self.temperatures = np.broadcast_to(np.asarray(temperatures, dtype=np.float64),
                                            (np.asarray(occ).reshape(-1, geo.n_sites).shape[0],)).copy()
        self.stream = stream if stream is not None else torch.cuda.Stream(device=geo.device)
        with torch.cuda.stream(self.stream):
            self.cb = ChainBatch(geo, occ, eci, kB * self.temperatures, move, seed=seed, chain_keys=chain_keys,
                                 stream=self.stream)
        self.precision = int(precision)
        self.kernel = int(kernel)
        if warps == 0:
            from .autotune import best_config
            warps, cluster, self.kernel = best_config(geo, move, self.precision, self.cb.n_chains, batch=self.cb)
        self.warps = int(warps)
        self.cluster = int(cluster)  # CTAs per chain (0: chosen by the library)
        self.trials_per_step = max(1, int(round(sweeps_per_step * geo.n_sites)))
        self.recompute_every = max(0, int(recompute_every))
        self.use_graph = bool(graph)
        self._graph = None
        self.steps_done = 0

    @property
    def n_chains(self) -> int:
        return self.cb.n_chains

    def _step_body(self, with_recompute: bool):
        self.cb.run(self.trials_per_step, precision=self.precision, warps=self.warps, cluster=self.cluster,
                    kernel=self.kernel)
        if with_recompute and not self.cb.recomputed:
            self.cb.recompute()

    def capture(self):
        """Capture one step (MC launch + drift-reset recompute) as a CUDA graph."""
        if not self.use_graph or self._graph is not None:
            return
        # warm the launch path (shared-memory attributes, lazy loading) outside the capture; the
        # snapshot, the warm step and the restore are ordered on the runner's stream
        snapshot = self.snapshot()
        with torch.cuda.stream(self.stream):
            self._step_body(self.recompute_every == 1)
        self.restore(snapshot)
        self.stream.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=self.stream):
            self._step_body(self.recompute_every == 1)
        self._graph = g

    def step(self, n: int = 1):
        """Advance every chain by ``n`` steps (asynchronous on the runner's stream)."""
        for _ in range(n):
            self.steps_done += 1
            if self.use_graph and self.recompute_every == 1:
                if self._graph is None:
                    self.capture()
                with torch.cuda.stream(self.stream):  # replay() launches on the current stream
                    self._graph.replay()
            else:
                with torch.cuda.stream(self.stream):
                    rec = self.recompute_every > 0 and self.steps_done % self.recompute_every == 0
                    self._step_body(rec)

    def synchronize(self):
        self.stream.synchronize()

    # -- state transfer (the served / end-to-end path) -------------------------------
    def snapshot(self) -> Dict[str, torch.Tensor]:
        """Copies of the chain state, taken in order on the runner's stream (after its queued work)."""
        cb = self.cb
        names = ["occ", "cf", "energy", "eci", "kT", "trial", "accum"]
        if cb.trk is not None:
            names += ["trk", "loc"]
        with torch.cuda.stream(self.stream):
            return {n: getattr(cb, n).clone() for n in names}

    def restore(self, snap: Dict[str, torch.Tensor]):
        """Write a snapshot back, in order on the runner's stream: a launch still running there
        (the stream's own work) finishes before the state is overwritten."""
        with torch.cuda.stream(self.stream):
            for n, t in snap.items():
                getattr(self.cb, n).copy_(t)

    def load_state(self, occ: torch.Tensor, eci: Optional[torch.Tensor] = None, kT: Optional[torch.Tensor] = None):
        """Copy new configurations (host or device tensors) into the resident state and rebuild derived data."""
        cb = self.cb
        with torch.cuda.stream(self.stream):
            cb.occ.copy_(occ, non_blocking=True)
            if eci is not None:
                cb.eci.copy_(eci, non_blocking=True)
            if kT is not None:
                cb.kT.copy_(kT, non_blocking=True)
            cb.recompute()
            cb.reset_accumulators()

    # -- results ----------------------------------------------------------------------
    def thermodynamics(self) -> List[Dict[str, float]]:
        """Per-chain averages from the device running sums (Montecarlo.get_thermodynamic semantics)."""
        self.synchronize()
        acc = self.cb.accum_host()
        kT = self.cb.kT.cpu().numpy()
        out = []
        m = self.geo.model
        for c in range(self.n_chains):
            a = acc[c]
            n = max(a[E.A_NSAMP], 1.0)
            mean = a[E.A_EREF] + a[E.A_SUM_E] / n
            var = a[E.A_SUM_E2] / n - (a[E.A_SUM_E] / n) ** 2
            T = kT[c] / self.kB
            d = {"energy": mean, "heat_capacity": var / (self.kB * T * T), "temperature": T,
                 "accept_rate": a[E.A_NACC] / n, "n_mc_steps": int(a[E.A_NSAMP])}
            for b in range(m.n_bf):
                s = a[E.A_SUM_S + b] / n
                d["singlet_c1_%d" % b] = s
                d["var_singlet_c1_%d" % b] = a[E.A_SUM_S2 + b] / n - s * s
            out.append(d)
        return out


class MultiBatchRunner:
    """Chains of several supercells stepped together: one CUDA graph per step.

    Each group (one geometry and its chains) is a ``BatchRunner`` on its own
    stream.  The captured step forks every group's stream from a capture stream,
    records each group's MC launch and recompute on it, and joins them back, so
    ONE graph launch runs all groups' kernels concurrently on the device (uneven
    supercells do not wait for one another).  ``trials`` counts the step's
    trials over all groups.
    """

    def __init__(self, runners: Sequence[BatchRunner]):
        if not runners:
            raise ValueError("no groups")
        self.runners = list(runners)
        self.device = self.runners[0].geo.device
        self.stream = torch.cuda.Stream(device=self.device)
        self._graph = None
        self.trials_per_step = sum(r.n_chains * r.trials_per_step for r in self.runners)

    @property
    def n_chains(self) -> int:
        return sum(r.n_chains for r in self.runners)

    def _launch_order(self):
        """Groups by descending work per chain (longest first): the chains that set the step start
        before the short ones take the SMs, and the short ones fill the SMs around them."""
        return sorted(self.runners, key=lambda r: -r.trials_per_step * (2 if r.geo.model.n_sym > 2 else 1))

    def _body(self):
        start = torch.cuda.Event()
        start.record(self.stream)
        done = []
        for r in self._launch_order():
            r.stream.wait_event(start)
            with torch.cuda.stream(r.stream):
                r._step_body(r.recompute_every == 1)
            ev = torch.cuda.Event()
            ev.record(r.stream)
            done.append(ev)
        for ev in done:
            self.stream.wait_event(ev)

    def capture(self):
        if self._graph is not None:
            return
        snaps = [r.snapshot() for r in self.runners]
        with torch.cuda.stream(self.stream):
            self._body()  # warm the launch path outside the capture
        for r, snap in zip(self.runners, snaps):
            r.restore(snap)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=self.stream):
            self._body()
        self._graph = g

    def step(self, n: int = 1):
        """Advance every chain of every group by ``n`` steps (asynchronous on the runner's stream)."""
        if self._graph is None:
            self.capture()
        for _ in range(n):
            with torch.cuda.stream(self.stream):
                self._graph.replay()
            for r in self.runners:
                r.steps_done += 1

    def synchronize(self):
        self.stream.synchronize()


def sgc_grid(T_range=(300.0, 1200.0), mu_range=(-0.2, 0.2), n_T=8, n_mu=8):
    """Temperatures and chemical potentials of an n_T x n_mu semi-grand-canonical grid (T-major)."""
    Ts = np.repeat(np.linspace(T_range[0], T_range[1], n_T), n_mu)
    mus = np.tile(np.linspace(mu_range[0], mu_range[1], n_mu), n_T)
    return Ts, mus


def fold_chemical_potential(model, eci_vec: np.ndarray, mus: Sequence[float], singlet: str = "c1_0") -> np.ndarray:
    """ECIs per chain with mu folded into a singlet ECI, eci[c1] -= mu (sgc_montecarlo.py:239-261)."""
    ev = np.repeat(np.asarray(eci_vec, dtype=np.float64)[None], len(mus), 0)
    ev[:, model.eci_names.index(singlet)] -= np.asarray(mus, dtype=np.float64)
    return ev
