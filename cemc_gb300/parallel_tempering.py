"""Parallel tempering with every replica resident on one GPU.

Mirrors cemc/mcmc/parallel_tempering.py: a ladder of temperatures, Metropolis
sweeps of every replica, then neighbour exchanges accepted with probability
exp((1/kT_1 - 1/kT_2)(E_1 - E_2)) (parallel_tempering.py:138-175), "up" or
"down" pairings chosen at random each cycle (177-191).

Differences by design: all replicas advance together in one launch of the
fused kernel instead of one runMC after the other (177-191), and an accepted
exchange swaps the two chains' temperatures (and ladder positions) on the
device instead of copying whole configurations with set_symbols (146-151).
The two are statistically identical; ``replica_of`` records which chain sits
at each ladder position.
"""
from __future__ import annotations

import os
from typing import Dict, List, Optional, Sequence

import numpy as np
import torch

from . import engine as E
from .batch import KB_EV
from .rng import philox4x32_10


class ParallelTempering:
    """Temperature ladder over copies of one configuration.

    :param geo: device geometry (``engine.Geometry``).
    :param occ: initial occupation (n_sites,) or one per replica (n_replicas, n_sites).
    :param eci: ECI vector of the model.
    :param temperatures: ladder, or None to build a geometric ladder between Tmin and Tmax
        (or read it from ``temp_scheme_file``, one temperature per line, as the reference writes it).
    :param move: ``engine.MOVE_SWAP`` (canonical, the reference) or ``engine.MOVE_FLIP``.
    """

    def __init__(self, geo: E.Geometry, occ, eci, temperatures: Optional[Sequence[float]] = None, Tmax=1500.0,
                 Tmin=100.0, n_replicas: int = 16, temp_scheme_file: Optional[str] = None, move=E.MOVE_SWAP,
                 seed: int = 0, precision=E.PREC_F32, warps: int = 0, kB: float = KB_EV):
        if temperatures is None and temp_scheme_file and os.path.exists(temp_scheme_file):
            data = np.loadtxt(temp_scheme_file, delimiter=",", ndmin=2)
            temperatures = data[:, 0].tolist()
        if temperatures is None:
            temperatures = np.geomspace(Tmax, Tmin, n_replicas)
        self.temperatures = np.asarray(temperatures, dtype=np.float64)
        n = len(self.temperatures)
        occ = np.asarray(occ, dtype=np.int8)
        if occ.ndim == 1:
            occ = np.repeat(occ[None], n, 0)
        self.kB = kB
        self.seed = int(seed)
        self.precision = precision
        self.cb = E.ChainBatch(geo, occ, eci, kB * self.temperatures, move, seed=seed)
        if warps == 0:
            from .autotune import best_warps
            warps = best_warps(geo, move, precision, n)
        self.warps = warps
        dev = self.cb.occ.device
        self.replica_of = torch.arange(n, dtype=torch.int32, device=dev)
        # running sums are kept per ladder position (temperature), as in the reference where
        # each Montecarlo object of the ladder keeps its own averages
        self.position_of = torch.arange(n, dtype=torch.int32, device=dev)
        self.cb.accum_slot = self.position_of
        self.n_accept = torch.zeros(1, dtype=torch.int32, device=dev)
        self.exchange_round = 0
        self.accepted_exchanges: List[int] = []

    @property
    def temperature_scheme(self) -> List[float]:
        return self.temperatures.tolist()

    def save_temperature_scheme(self, fname="temp_scheme.csv"):
        np.savetxt(fname, np.vstack((self.temperatures, np.zeros_like(self.temperatures))).T, delimiter=",",
                   header="Temperature (K), Acceptance probabability")

    def _direction(self) -> int:
        w = philox4x32_10(self.exchange_round & 0xFFFFFFFF, self.exchange_round >> 32, 0xD1, 0, self.seed & 0xFFFFFFFF,
                          (self.seed >> 32) & 0xFFFFFFFF)
        return w[0] & 1  # 0 = "up", 1 = "down"

    def run(self, sweeps_per_cycle: float = 10.0, num_exchange_cycles: int = 10, recompute: bool = True,
            record: bool = False):
        """Alternate Metropolis sweeps of every replica and one exchange sweep, on the device."""
        n_sites = self.cb.geo.n_sites
        trials = max(1, int(round(sweeps_per_cycle * n_sites)))
        for _ in range(num_exchange_cycles):
            self.cb.run(trials, precision=self.precision, warps=self.warps)
            if recompute and not self.cb.recomputed:
                self.cb.recompute()
            E.pt_exchange(self.cb.energy, self.cb.kT, self.replica_of, self._direction(), self.seed,
                          self.exchange_round, self.n_accept, position_of=self.position_of)
            self.exchange_round += 1
            if record:
                self.accepted_exchanges.append(int(self.n_accept.item()))
        torch.cuda.synchronize()
        self.cb.check_status()

    def ladder(self) -> List[Dict[str, float]]:
        """Per ladder position: temperature, chain, current energy, running averages of that chain."""
        rep = self.replica_of.cpu().numpy()
        energy = self.cb.energy.cpu().numpy()
        acc = self.cb.accum_host()
        out = []
        for pos, c in enumerate(rep):
            a = acc[pos]
            n = max(a[E.A_NSAMP], 1.0)
            mean = a[E.A_EREF] + a[E.A_SUM_E] / n
            var = a[E.A_SUM_E2] / n - (a[E.A_SUM_E] / n) ** 2
            T = self.temperatures[pos]
            out.append({"position": pos, "temperature": T, "chain": int(c), "energy": float(energy[c]),
                        "mean_energy": mean, "heat_capacity": var / (self.kB * T * T),
                        "n_mc_steps": int(a[E.A_NSAMP])})
        return out
