"""Drop-in Metropolis drivers with the reference's runMC API, running on the GPU.

``Montecarlo`` (canonical swaps) and ``SGCMonteCarlo`` (semi-grand-canonical
flips) keep the constructor arguments, ``runMC`` signature, step accounting
and ``get_thermodynamic`` output of cemc/mcmc/montecarlo.py and
cemc/mcmc/sgc_montecarlo.py.  What changes is the inner loop: instead of one
Python -> C++ call per trial (montecarlo.py:970-1038), ``runMC`` hands whole
blocks of trials to the fused kernel, which proposes, evaluates, accepts and
commits in place on the calculator's device-resident configuration and keeps
the running sums the reference's ``Averager``s and ``SGCObserver`` keep.

Step accounting kept from the reference (montecarlo.py:732-844):
one trial before the loop, optional correlation-time estimate and
equilibration, a reset, 1000 trials to probe the energy bias followed by
``eci['c0'] -= E/N`` (178-217), a reset, then ``steps`` trials, then the bias is
added back to ``c0``.  Averages cover exactly the ``steps`` main-loop trials.

Trial proposals and uniforms come from the counter-based stream (seeded per
driver) rather than numpy's global generator; the proposal distributions are
the reference's (montecarlo.py:890-908, sgc_montecarlo.py:62-76).
"""
from __future__ import annotations

import logging
import time
from typing import Dict, List, Optional

import numpy as np
import torch

from . import engine as E
from .batch import KB_EV

kB = KB_EV


class DidNotReachEquillibriumError(Exception):
    pass


class TooFewElementsError(Exception):
    pass


class CanNotFindLegalMoveError(Exception):
    pass


class InvalidChemicalPotentialError(Exception):
    pass


_PREC = {"fp64": E.PREC_F64, "fp32": E.PREC_F32, E.PREC_F64: E.PREC_F64, E.PREC_F32: E.PREC_F32}


class Montecarlo:
    """Canonical Metropolis Monte Carlo (swap moves) on the GPU.

    :param atoms: atoms container with a ``cemc_gb300.calculator.CE`` attached.
    :param float temp: temperature in kelvin.
    :param int seed: seed of the counter-based trial stream (default: from os.urandom).
    :param precision: "fp64" (default, reference precision) or "fp32" (FP32 energy change, FP64 totals).
    :param int warps: speculation width of the kernel (0 = autotuned).
    :param int recompute_every_sweeps: FP64 full recompute (drift reset) interval.
    """

    move = E.MOVE_SWAP

    def __init__(self, atoms, temp, indeces=None, logfile="", plot_debug=False, min_acc_rate=0.0,
                 recycle_waste=False, max_constraint_attempts=10000, accept_first_trial_move_after_reset=False,
                 seed: Optional[int] = None, precision="fp64", warps: int = 0, recompute_every_sweeps: int = 100):
        self.name = "MonteCarlo"
        self.atoms = atoms
        self.T = float(temp)
        self.min_acc_rate = min_acc_rate
        # waste recycling (montecarlo.py:937-948): two-state acceptance and weighted sums on the device
        self.recycle_waste = bool(recycle_waste)
        # the next trial is accepted outright after construction, reset() and set_symbols()
        # (montecarlo.py:128-131, 294-295, 363-364, 932-935)
        self.accept_first_trial_move_after_reset = bool(accept_first_trial_move_after_reset)
        self.is_first = self.accept_first_trial_move_after_reset
        if max_constraint_attempts <= 0:
            raise ValueError("Max. constraint attempts has to be > 0!")
        self.indeces = range(len(atoms)) if indeces is None else indeces
        self.observers = []
        self.constraints = []
        self.max_allowed_constraint_pass_attempts = int(max_constraint_attempts)
        self._constraint_dev = None  # device masks of self.constraints, built on first use
        self.bias_potentials = []
        self.bias_energy = 0.0
        self.current_step = 0
        self.num_accepted = 0
        self.status_every_sec = 30
        self.energy_bias = 0.0
        self.correlation_info = None
        self.precision = _PREC[precision]
        self.warps = int(warps)
        self.recompute_every_sweeps = max(1, int(recompute_every_sweeps))
        if seed is None:
            seed = int.from_bytes(np.random.bytes(8), "little")
        self.seed = int(seed) & (2 ** 64 - 1)
        self.logfile = logfile
        self.logger = logging.getLogger("MonteCarlo")
        calc = self._calc()
        self.symbols = sorted(set(a.symbol for a in atoms))
        self.current_energy = calc.get_energy()
        self._chain: Optional[E.ChainBatch] = None
        self._trial = 0
        self._acc_base = np.zeros(E.ACCUM_DOUBLES)

    # -- plumbing -----------------------------------------------------------------
    def _calc(self):
        calc = self.atoms.get_calculator() if hasattr(self.atoms, "get_calculator") else self.atoms.calc
        if calc is None or not hasattr(calc, "updater"):
            raise TypeError("the atoms object needs a cemc_gb300.calculator.CE calculator attached")
        return calc

    def _kT(self):
        return kB * self.T

    def chain(self) -> E.ChainBatch:
        """The calculator's configuration viewed as a one-chain batch (built lazily, shares device memory)."""
        calc = self._calc()
        up = calc.updater
        if self._chain is None:
            self._chain = E.ChainBatch.wrap(up.geo, up.occ_d, up.cf_d, up.energy_d, up.eci_d, self._kT(), self.move,
                                            seed=self.seed, stream=up.stream)
        else:
            self._chain.set_temperature(self._kT())
        return self._chain

    def _invalidate_chain(self):
        self._chain = None

    def log(self, msg, mode="info"):
        if mode not in ("info", "warning"):
            raise ValueError("Mode has to be one of ['info', 'warning']")
        getattr(self.logger, mode)(msg)

    # -- the reference's public API ---------------------------------------------------
    def _check_symbols(self):
        """montecarlo.py:297-319."""
        symbs = [a.symbol for a in self.atoms]
        count = {}
        for s in symbs:
            count[s] = count.get(s, 0) + 1
        if len(count) < 2:
            raise TooFewElementsError("There is only one element in the given atoms object!")
        if sum(1 for v in count.values() if v >= 2) < 2:
            raise TooFewElementsError("There is only one element that has more than one atom")

    def update_current_energy(self):
        """Energy of the current state from the calculator plus every bias potential's value,
        computed from scratch (montecarlo.py:276-282)."""
        self.current_energy = self._calc().get_energy()
        self.bias_energy = 0.0
        for bias in self.bias_potentials:
            self.bias_energy += float(bias.calculate_from_scratch(self.atoms))
        self.current_energy += self.bias_energy

    def set_symbols(self, symbs):
        self._calc().set_symbols(symbs)
        self._invalidate_chain()
        self.symbols = sorted(set(symbs))
        self.update_current_energy()
        if self.accept_first_trial_move_after_reset:
            self.is_first = True

    def add_constraint(self, constraint):
        """Add a move constraint (montecarlo.py:386-392), enforced on the device.

        FixedElement, ConstrainElementByTag and FixEdgeLayers (this package's or the
        reference's objects) become per-site masks checked by the kernel's redraw loop;
        other constraints raise ``NotImplementedError`` (see ``mc_constraints``).
        """
        from .mc_constraints import device_masks
        m = self._calc().model
        device_masks(constraint, m.symbols, m.n_sites)
        self.constraints.append(constraint)
        self._constraint_dev = None

    def _no_constraint_violations(self, system_changes):
        """montecarlo.py:334-347."""
        for constraint in self.constraints:
            if not constraint(system_changes):
                return False
        return True

    def _first_arg(self):
        """Per-launch flags: waste recycling, and ``accept_first`` (consumes the pending first-trial
        acceptance)."""
        out = {"recycle_waste": True} if self.recycle_waste else {}
        if getattr(self, "is_first", False):
            self.is_first = False
            out["accept_first"] = True
        return out

    def _constraint_args(self):
        """Device masks and redraw limit of the constraints, as ``ChainBatch.run`` arguments."""
        if not self.constraints:
            return {}
        if self._constraint_dev is None:
            from .mc_constraints import combined_masks
            m = self._calc().model
            allow, frozen = combined_masks(self.constraints, m.symbols, m.n_sites)
            dev = self._calc().updater.occ_d.device
            self._constraint_dev = {
                "site_allow": None if allow is None else torch.as_tensor(allow[None, :]).to(dev),
                "frozen": torch.tensor([np.int32(np.uint32(frozen).view(np.int32))], dtype=torch.int32,
                                       device=dev) if frozen else None,
            }
        return dict(self._constraint_dev, max_attempts=self.max_allowed_constraint_pass_attempts)

    def insert_symbol(self, symb, indices):
        """Put ``symb`` on the given sites (montecarlo.py:219-233); each change must pass the constraints."""
        calc = self._calc()
        for indx in indices:
            change = (int(indx), self.atoms[indx].symbol, symb)
            if not self._no_constraint_violations([change]):
                raise ValueError("The indices given results in an update that violate one or more constraints!")
            calc.update_cf(change)
        calc.clear_history()
        self._invalidate_chain()
        self.symbols = sorted(set(a.symbol for a in self.atoms) | set(self.symbols))
        self.update_current_energy()

    def insert_symbol_random_places(self, symbol, num=1, swap_symbs=()):
        """Put ``symbol`` on ``num`` random sites holding one of ``swap_symbs`` (montecarlo.py:235-275).

        Draws from numpy's global generator where the reference uses Python's ``random``.
        """
        calc = self._calc()
        symbs = [a.symbol for a in self.atoms]
        swap_symbs = list(swap_symbs) if swap_symbs else sorted(set(symbs))
        max_attempts = 10 * len(self.atoms)
        num_inserted = attempts = 0
        while num_inserted < num and attempts < max_attempts:
            attempts += 1
            old_symb = swap_symbs[np.random.randint(len(swap_symbs))]
            if old_symb == symbol:
                continue
            sites = [i for i, a in enumerate(self.atoms) if a.symbol == old_symb]
            if not sites:
                continue
            indx = sites[np.random.randint(len(sites))]
            change = (indx, old_symb, symbol)
            if not self._no_constraint_violations([change]):
                continue
            calc.update_cf(change)
            num_inserted += 1
        calc.clear_history()
        self._invalidate_chain()
        self.symbols = sorted(set(a.symbol for a in self.atoms) | set(self.symbols))
        self.update_current_energy()
        if attempts == max_attempts:
            raise RuntimeError("Could insert {} {} atoms!".format(num, symbol))

    def add_bias(self, potential):
        """Add a bias potential (montecarlo.py:394-401).

        A bias is any object with the reference's ``BiasPotential`` interface
        (cemc/mcmc/bias_potential.py:4-31): ``potential(system_changes)`` returns its value
        for the state after the proposed changes, which the acceptance test adds to that
        state's energy (montecarlo.py:925-930); ``calculate_from_scratch(atoms)`` gives its
        value for the current state.  Arbitrary host code cannot run inside the kernel, so a
        driver with biases evaluates its trials one at a time on the host (``_run_biased``):
        the same counter-based proposals and uniforms as the kernel, the energy change from the
        device calculator, the biases, then the reference's acceptance test.
        """
        if not callable(potential) or not hasattr(potential, "calculate_from_scratch"):
            raise TypeError("potential has to be of type BiasPotential")
        if self.recycle_waste:
            raise NotImplementedError("waste recycling together with bias potentials is not supported")
        self.bias_potentials.append(potential)

    def attach(self, obs, interval=1):
        """Call ``obs(system_changes)`` every ``interval`` trials (montecarlo.py:403-415).

        The trials between two observed steps run on the device as one launch, so a large
        interval costs nothing; interval 1 turns every trial into its own launch.
        """
        if not callable(obs):
            raise ValueError("The observer has to be a callable class!")
        self.observers.append((interval, obs))

    def reset(self):
        """Zero the step counter and averages (montecarlo.py:349-364)."""
        for _, obs in self.observers:
            if hasattr(obs, "reset"):
                obs.reset()
        self.current_step = 0
        self.num_accepted = 0
        if self.accept_first_trial_move_after_reset:
            self.is_first = True
        ch = self.chain()
        ch.reset_accumulators()

    def count_atoms(self):
        occ = self._calc().updater.occupation()
        m = self._calc().model
        cnt = np.bincount(occ.astype(np.int64), minlength=m.n_sym)
        return {m.symbols[i]: int(cnt[i]) for i in range(m.n_sym) if m.symbols[i] in self.symbols}

    def _run_trials(self, n: int, trace: bool = False):
        """n trials through the fused kernel; drift reset every recompute_every_sweeps sweeps.

        Attached observers are called like the reference's ``_mc_step`` calls them
        (montecarlo.py:1031-1036): after every trial whose step number is a multiple of
        the observer's interval, with that trial's changes (``(site, old, new)``, or
        ``(site, old, old)`` when it was rejected).  The trials between two such steps
        run as one launch; the observed trial runs alone, traced.
        """
        if self.bias_potentials:
            return self._run_biased(n, trace)
        traces = []
        done = 0
        while done < n:
            gap = self._steps_to_next_observation()
            if gap is None or gap > n - done:
                traces += self._run_block(n - done, trace)
                break
            if gap > 1:
                traces += self._run_block(gap - 1, trace)
            traces += self._observed_trial(trace)
            done += gap
        return traces

    def _steps_to_next_observation(self):
        """Trials until the next step at which an observer is due (None without observers)."""
        gaps = [int(iv) - self.current_step % int(iv) for iv, _ in self.observers if int(iv) > 0]
        return min(gaps) if gaps else None

    def _run_block(self, n: int, trace: bool = False):
        ch = self.chain()
        m = self._calc().model
        block = self.recompute_every_sweeps * m.n_sites
        traces = []
        done = 0
        while done < n:
            k = min(block, n - done)
            tr = ch.run(k, precision=self.precision, warps=self._warps(), trace=trace, **self._constraint_args(),
                        **self._first_arg())
            if trace:
                traces.append(tr)
            if k == block:
                ch.recompute()
            done += k
        self.current_step += n
        self._sync_after_run()
        return traces

    def _observed_trial(self, trace: bool = False):
        """One traced trial, then the observers due at this step get its changes."""
        calc = self._calc()
        syms = calc.model.symbols_of(calc.updater.occupation())
        ch = self.chain()
        tr = ch.run(1, precision=self.precision, warps=1, trace=True, **self._constraint_args(), **self._first_arg())
        self.current_step += 1
        self._sync_after_run()
        sites, acc, _ = (t.cpu().numpy() for t in tr)
        a, b = int(sites[0, 0, 0]), int(sites[0, 0, 1])
        accepted = bool(acc[0, 0])
        if self.move == E.MOVE_SWAP:
            sa, sb = syms[a], syms[b]
            changes = [(a, sa, sb), (b, sb, sa)] if accepted else [(a, sa, sa), (b, sb, sb)]
        else:
            new = calc.model.symbols[b]
            changes = [(a, syms[a], new)] if accepted else [(a, syms[a], syms[a])]
        for interval, obs in self.observers:
            if int(interval) > 0 and self.current_step % int(interval) == 0:
                obs(changes)
        return [tr] if trace else []

    def _run_biased(self, n: int, trace: bool = False):
        """n trials of a driver with bias potentials, one at a time (the reference's _mc_step and
        _accept, montecarlo.py:910-1038).

        Trial t draws its proposal and uniform from the same counter-based stream as the kernel
        (proposal k of a redrawn trial from streams 2k, 2k + 1), so a biased run continues the
        chain an unbiased launch would continue, and the device trial counter, swap site lists
        and running sums stay valid.  Per trial: the energy change from the device calculator
        (``cemc_delta_e``), the atoms object updated to the proposed state and each bias called
        with the changes, then accept when new < current or u <= exp(-(new - current) / kT)
        (the first trial after a reset is accepted outright when asked), commit on the device
        (``cemc_apply_changes``).  The running sums take the energy with its bias, as the
        reference's averages do.
        """
        from .rng import below, trial_draw, u01_53
        calc = self._calc()
        up = calc.updater
        m = calc.model
        ch = self.chain()
        torch.cuda.synchronize(ch.occ.device)
        key = int(ch.chain_key[0].item())
        t = int(ch.trial[0].item())
        occ = up.occupation().astype(np.int64)
        swap = self.move == E.MOVE_SWAP
        if swap:
            trk, loc = ch.trk[0].cpu().numpy().copy(), ch.loc[0].cpu().numpy().copy()
            start, count = ch.trk_start[0].cpu().numpy(), ch.trk_count[0].cpu().numpy()
            present = [s for s in range(m.n_sym) if count[s] > 0]
        movable = np.asarray(m.movable, dtype=np.int64)
        every_site = len(movable) == m.n_sites
        syms = m.symbols
        e_ref = float(ch.accum_host()[0, E.A_EREF])
        cf = up.cf()
        sing_idx = [int(k) for k in m.singlet_eci[:m.n_bf]]
        sing = np.array([cf[k] for k in sing_idx], dtype=np.float64)
        e_ce = up.energy()
        sums = np.zeros(E.A_NSAMP - 1)  # sum_e, sum_e2, sum_s[4], sum_s2[4], sum_se[4]
        n_acc = 0
        kT = self._kT()
        max_att = self.max_allowed_constraint_pass_attempts
        tr_sites, tr_acc, tr_de = [], [], []

        def proposal(k):
            w = trial_draw(self.seed, key, t, 2 * k)
            if swap:
                x = trial_draw(self.seed, key, t, 2 * k + 1)
                npres = len(present)
                ia = below(w[0], npres)
                ib = below(w[1], npres - 1)
                ib += ib >= ia
                A, B = present[ia], present[ib]
                a = int(trk[start[A] + below(w[2], int(count[A]))])
                b = int(trk[start[B] + below(w[3], int(count[B]))])
                return [(a, A, B), (b, B, A)], x[0], x[1]
            a = int(below(w[0], m.n_sites)) if every_site else int(movable[below(w[0], len(movable))])
            old = int(occ[a])
            kk = below(w[1], m.n_sym - 1)
            return [(a, old, kk + (kk >= old))], w[2], w[3]

        for _ in range(n):
            self.current_step += 1
            k = 0
            ids, ua, ub = proposal(0)
            while not self._no_constraint_violations([(s, syms[o], syms[v]) for s, o, v in ids]) and k < max_att:
                k += 1
                ids, ua, ub = proposal(k)
            if k == max_att:
                raise CanNotFindLegalMoveError("Did not manage to produce a trial move that does not violate any "
                                               "of the constraints")
            t += 1
            changes = [(s, syms[o], syms[v]) for s, o, v in ids]
            if swap:
                de, dcf = up.delta_swap(ids[0][0], ids[1][0])
            else:
                de, dcf = up.delta_flip(ids[0][0], ids[0][2])
            # the biases see the system with the proposed changes in place (montecarlo.py:925-930)
            for s, _, v in changes:
                self.atoms[s].symbol = v
            bias_new = 0.0
            for bias in self.bias_potentials:
                bias_new += float(bias(changes))
            new_energy = e_ce + de + bias_new
            if self.is_first:
                self.is_first = False
                accept = True
            elif new_energy < self.current_energy:
                accept = True
            else:
                accept = u01_53(ua, ub) <= np.exp(-(new_energy - self.current_energy) / kT)
            tr_sites.append((ids[0][0], ids[1][0] if swap else ids[0][2]))
            tr_acc.append(int(accept))
            tr_de.append(new_energy - self.current_energy)
            if accept:
                up.apply(ids, record=False)
                e_ce += de
                self.current_energy = new_energy
                self.bias_energy = bias_new
                for s, _, v in ids:
                    occ[s] = v
                if swap:  # the site lists as the kernel's commit leaves them
                    (a, A, B), (b, _, _) = ids
                    la, lb = int(loc[a]), int(loc[b])
                    trk[start[A] + la] = b
                    loc[b] = la
                    trk[start[B] + lb] = a
                    loc[a] = lb
                sing += np.array([dcf[k] for k in sing_idx])
                n_acc += 1
                obs_changes = changes
            else:
                for s, o, _ in changes:
                    self.atoms[s].symbol = o
                obs_changes = [(s, o, o) for s, o, _ in changes]
            e = self.current_energy - e_ref
            sums[0] += e
            sums[1] += e * e
            for b in range(m.n_bf):
                sums[2 + b] += sing[b]
                sums[2 + E._lib.MAX_BF + b] += sing[b] * sing[b]
                sums[2 + 2 * E._lib.MAX_BF + b] += sing[b] * e
            for interval, obs in self.observers:
                if int(interval) > 0 and self.current_step % int(interval) == 0:
                    obs(obs_changes)
        # hand the chain back to the device path: trial counter, site lists, running sums
        raw = ch.accum.cpu().numpy().copy()
        raw[0, E.A_SUM_E:E.A_NSAMP] += sums
        counters = raw[0, E.A_NSAMP:E.A_NACC + 1].view(np.uint64)
        counters += np.array([n, n_acc], dtype=np.uint64)
        ch.accum.copy_(torch.as_tensor(raw))
        ch.trial.fill_(t)
        if swap:
            ch.trk[0].copy_(torch.as_tensor(trk))
            ch.loc[0].copy_(torch.as_tensor(loc))
        up.clear()
        self.num_accepted = int(ch.accum_host()[0, E.A_NACC])
        if not trace:
            return []
        sites = torch.tensor(tr_sites, dtype=torch.int32).view(1, n, 2)
        return [(sites, torch.tensor(tr_acc, dtype=torch.int8).view(1, n),
                 torch.tensor(tr_de, dtype=torch.float64).view(1, n))]

    def _warps(self):
        if self.warps:
            return self.warps
        from .autotune import best_warps
        m = self._calc().model
        self.warps = best_warps(self._calc().geometry, self.move, self.precision, 1)
        return self.warps

    def _sync_after_run(self):
        ch = self._chain
        torch.cuda.synchronize(ch.occ.device)
        try:
            ch.check_status()
        except E._lib.CemcError as exc:
            if exc.code == E._lib.ERR_NO_MOVE:
                ch.status.zero_()
                raise CanNotFindLegalMoveError("Did not manage to produce a trial move that does not violate any "
                                               "of the constraints") from exc
            raise
        calc = self._calc()
        # mirror the new configuration into the atoms object (background sites keep their symbol)
        # and drop the undo buffer
        syms = calc.model.symbols_of(calc.updater.occupation())
        for a, s in zip(self.atoms, syms):
            if a.symbol != s:
                a.symbol = s
        calc.updater.clear()
        acc = ch.accum_host()[0]
        self.num_accepted = int(acc[E.A_NACC])
        self.current_energy = calc.get_energy()

    def _mc_step(self, verbose=False):
        """One trial (the reference's _mc_step, observers included); returns (energy, accepted)."""
        if self.bias_potentials:
            (_, acc, _), = self._run_biased(1, trace=True)
        else:
            (_, acc, _), = self._observed_trial(trace=True)
        return self.current_energy, bool(acc.cpu().numpy()[0, 0])

    def _probe_energy_bias(self, num_steps=1000):
        """montecarlo.py:178-211."""
        self.log("Probing energy bias using {} MC steps...".format(num_steps))
        self._run_trials(num_steps)
        self.energy_bias = self.current_energy
        self._remove_bias_from_empty_eci(self.energy_bias)

    def _remove_bias_from_empty_eci(self, bias):
        calc = self._calc()
        eci = calc.eci
        eci["c0"] = eci["c0"] - bias / len(self.atoms)
        calc.update_ecis(eci)
        self.current_energy = calc.get_energy()
        if abs(self.current_energy) > 1e-6:
            raise RuntimeError("Energy is not 0 after subtracting the bias. Got {}".format(self.current_energy))

    def _undo_energy_bias_from_eci(self):
        calc = self._calc()
        eci = calc.eci
        eci["c0"] += self.energy_bias / len(self.atoms)
        calc.update_ecis(eci)
        self.current_energy = calc.get_energy()

    def _window_stats(self, n):
        """Mean and variance of the energy over the next n trials (fresh accumulators)."""
        ch = self.chain()
        ch.reset_accumulators()
        self._run_trials(n)
        a = ch.accum_host()[0]
        cnt = max(a[E.A_NSAMP], 1.0)
        mean = a[E.A_EREF] + a[E.A_SUM_E] / cnt
        var = a[E.A_SUM_E2] / cnt - (a[E.A_SUM_E] / cnt) ** 2
        return mean, var, cnt

    def _estimate_correlation_time(self, window_length=1000, restart=False):
        """montecarlo.py:461-526 from a per-trial energy trace of the kernel."""
        ch = self.chain()
        e0 = self.current_energy
        tr = self._run_trials(window_length, trace=True)
        _, acc, de = tr[0] if len(tr) == 1 else (None, torch.cat([t[1] for t in tr], 1),
                                                 torch.cat([t[2] for t in tr], 1))
        acc = acc.cpu().numpy()[0].astype(bool)
        de = de.cpu().numpy()[0]
        energies = e0 + np.cumsum(np.where(acc, de, 0.0))
        info = {"correlation_time_found": False, "correlation_time": 0.0, "msg": ""}
        dev = energies - energies.mean()
        var = np.var(dev)
        if var == 0.0:
            info.update(correlation_time_found=True, correlation_time=window_length,
                        msg="Zero variance leads to infinite correlation time")
            self.correlation_info = info
            return info
        ac = np.correlate(dev, dev, mode="full")
        ac = ac[len(ac) // 2:] / (window_length * var)
        if np.min(ac) > 0.5:
            info.update(correlation_time=window_length, msg="Window is too short. Add more samples")
            self.correlation_info = info
            return info
        indx = int(np.argmax(ac < 0.5))
        rho = 2.0 ** (-1.0 / indx)
        info.update(correlation_time=-1.0 / np.log(rho), correlation_time_found=True)
        self.correlation_info = info
        return info

    def _get_var_average_energy(self):
        """montecarlo.py:429-459."""
        a = self.chain().accum_host()[0]
        n = max(a[E.A_NSAMP], 1.0)
        var = abs(a[E.A_SUM_E2] / n - (a[E.A_SUM_E] / n) ** 2)
        steps = max(self.current_step, 1)
        info = self.correlation_info
        if info is None or not info["correlation_time_found"]:
            return var / steps
        tau = max(info["correlation_time"], 1.0)
        return 2.0 * var * tau / steps

    def _composition_reached_equillibrium(self, prev_composition, var_prev, confidence_level=0.05):
        return True, prev_composition, var_prev, 0.0

    def _equillibriate(self, window_length="auto", confidence_level=0.05, maxiter=1000, mode="stat_equiv"):
        """montecarlo.py:541-697: windows of 10 N trials until the window means agree (z-test)."""
        from scipy import stats
        if mode not in ("stat_equiv", "fixed"):
            raise ValueError("Equilibration mode has to be one of ['stat_equiv', 'fixed']")
        if window_length == "auto":
            window_length = 10 * len(self.atoms)
        self.reset()
        if mode == "fixed":
            self._run_trials(window_length)
            return
        lo, hi = stats.norm.ppf(confidence_level), stats.norm.ppf(1.0 - confidence_level)
        E_prev = var_prev = None
        composition, var_comp = [], []
        for _ in range(maxiter):
            self.reset()
            E_new, var, n = self._window_stats(window_length)
            var_E_new = self._get_var_average_energy()
            comp_conv, composition, var_comp, _ = self._composition_reached_equillibrium(
                composition, var_comp, confidence_level=confidence_level)
            if E_prev is None:
                E_prev, var_prev = E_new, var_E_new
                continue
            var_diff = var_E_new + var_prev
            if var_diff < 1e-6:
                z = 0.0
                comp_conv = True
            else:
                z = (E_new - E_prev) / np.sqrt(var_diff)
            if lo < z < hi and comp_conv:
                self.current_step = 0
                return
            E_prev, var_prev = E_new, var_E_new
        raise DidNotReachEquillibriumError("Did not manage to reach equillibrium!")

    def _include_vib(self):
        self._calc().include_linvib_in_ecis(self.T)

    def runMC(self, mode="fixed", steps=10, verbose=False, equil=True, equil_params=None, prec=0.01,
              prec_confidence=0.05):
        """Run the Monte Carlo simulation (montecarlo.py:732-844)."""
        equil_params = equil_params or {}
        if mode not in ("fixed", "prec"):
            raise ValueError("Mode has to be one of ['fixed', 'prec']")
        self._check_symbols()
        self.update_current_energy()
        self._include_vib()
        self._run_trials(1)
        totalenergies = [self.current_energy]
        self.current_step = 0
        if equil:
            res = self._estimate_correlation_time()
            if not res["correlation_time_found"]:
                res["correlation_time"] = 1000
                res["correlation_time_found"] = True
            self._equillibriate(**equil_params)
        check_every = None
        if mode == "prec":
            res = self._estimate_correlation_time()
            while not res["correlation_time_found"]:
                res = self._estimate_correlation_time()
            check_every = max(1, int(10 * self.correlation_info["correlation_time"]))
        self.reset()
        self._probe_energy_bias()
        self.reset()
        self.chain().reset_accumulators(e_ref=0.0)
        start = time.time()
        if mode == "fixed":
            self._run_trials(int(steps))
        else:
            from scipy import stats
            percentile = stats.norm.ppf(1.0 - prec_confidence)
            while self.current_step < steps:
                self._run_trials(min(check_every, int(steps) - self.current_step))
                if self._get_var_average_energy() < (prec / percentile) ** 2:
                    break
        if self.current_step >= steps:
            self.log("Reached maximum number of steps ({} mc steps)".format(steps))
        self.elapsed = time.time() - start
        self._undo_energy_bias_from_eci()
        return totalenergies

    # -- checkpoint / restart (montecarlo.py:1040-1074) ---------------------------------
    _CHECKPOINT_ATTRS = ("T", "min_acc_rate", "current_step", "num_accepted", "status_every_sec", "energy_bias",
                         "correlation_info", "precision", "warps", "recompute_every_sweeps", "seed", "symbols",
                         "current_energy", "logfile", "name", "max_allowed_constraint_pass_attempts",
                         "accept_first_trial_move_after_reset", "is_first", "recycle_waste")

    def _checkpoint_attrs(self):
        return self._CHECKPOINT_ATTRS

    def save(self, fname):
        """Store the run so that ``load`` continues it exactly where it stopped.

        The reference pickles the whole driver with dill (montecarlo.py:1040-1056).
        Here the file (a pickle of plain data) holds the driver's attributes, the
        calculator's settings object, ECIs and symbols, and the chain's device state
        (``ChainBatch.state_dict``: occupation, correlation functions, energy, the
        trial counter of the counter-based stream, the running sums and the swap
        site lists), so a loaded driver draws the same trials and reaches
        bit-identical states.  Observers and constraints are not stored: like the
        reference does for those it cannot serialise, the caller attaches them again.
        """
        import pickle
        calc = self._calc()
        state = {"format": "cemc_gb300.montecarlo/1", "class": type(self).__name__,
                 "attrs": {k: getattr(self, k) for k in self._checkpoint_attrs()},
                 "settings": calc.BC, "eci": dict(calc.eci), "symbols": [a.symbol for a in self.atoms],
                 "chain": self.chain().state_dict()}
        with open(fname, "wb") as f:
            pickle.dump(state, f, protocol=4)

    @staticmethod
    def load(fname, atoms=None, device="cuda"):
        """Rebuild a driver saved by ``save`` (montecarlo.py:1058-1074).

        ``atoms``: container to attach the calculator to (its symbols are set
        from the file); default a ``SimpleAtoms`` of the saved symbols.
        """
        import pickle
        from .calculator import CE, SimpleAtoms
        with open(fname, "rb") as f:
            state = pickle.load(f)
        if state.get("format") != "cemc_gb300.montecarlo/1":
            raise ValueError("%s is not a Monte Carlo checkpoint of this library" % fname)
        klass = {"Montecarlo": Montecarlo, "SGCMonteCarlo": SGCMonteCarlo}[state["class"]]
        if atoms is None:
            atoms = SimpleAtoms(state["symbols"])
        else:
            for a, sym in zip(atoms, state["symbols"]):
                a.symbol = sym
        ch_state = state["chain"]
        names = sorted(state["eci"])  # the calculator keeps its correlation functions in sorted-name order
        CE(atoms, state["settings"], eci=dict(state["eci"]),
           initial_cf=dict(zip(names, np.asarray(ch_state["cf"], dtype=np.float64).reshape(-1).tolist())),
           device=device)
        a = state["attrs"]
        mc = klass(atoms, a["T"], seed=a["seed"], precision=a["precision"], warps=a["warps"],
                   recompute_every_sweeps=a["recompute_every_sweeps"])
        for k, v in a.items():
            setattr(mc, k, v)
        mc.chain().load_state_dict(ch_state)
        return mc

    @property
    def meta_info(self):
        import datetime
        import sys
        v = sys.version_info
        return {"timestamp": datetime.datetime.now().strftime("%Y-%m-%d %H:%M:%S"),
                "python_version": "{}.{}.{}".format(v.major, v.minor, v.micro)}

    def get_thermodynamic(self):
        """montecarlo.py:861-888."""
        a = self.chain().accum_host()[0]
        n = max(a[E.A_NSAMP], 1.0)
        mean = a[E.A_EREF] + a[E.A_SUM_E] / n
        mean_sq = a[E.A_SUM_E2] / n
        q = {"energy": mean + self.energy_bias,
             "heat_capacity": (mean_sq - (a[E.A_SUM_E] / n) ** 2) / (kB * self.T ** 2),
             "energy_std": float(np.sqrt(self._get_var_average_energy())),
             "temperature": self.T}
        for key, value in self.count_atoms().items():
            q["{}_conc".format(key)] = float(value) / len(self.atoms)
        q.update(self.meta_info)
        for _, obs in self.observers:
            if hasattr(obs, "get_averages"):
                q.update(obs.get_averages())
        q["accept_rate"] = a[E.A_NACC] / n
        return q


class SGCMonteCarlo(Montecarlo):
    """Semi-grand-canonical Monte Carlo (single-site flips) on the GPU (sgc_montecarlo.py)."""

    move = E.MOVE_FLIP

    def __init__(self, atoms, temp, indeces=None, symbols=None, logfile="", plot_debug=False, min_acc_rate=0.0,
                 recycle_waste=False, **kwargs):
        Montecarlo.__init__(self, atoms, temp, indeces=indeces, logfile=logfile, plot_debug=plot_debug,
                            min_acc_rate=min_acc_rate, recycle_waste=recycle_waste, **kwargs)
        species = list(self._calc().model.symbols)
        if symbols is not None:
            if sorted(symbols) != species:
                raise NotImplementedError("flips to a subset of the species are not supported by the GPU drivers")
        self.symbols = species
        if len(self.symbols) <= 1:
            raise ValueError("At least 2 symbols have to be specified")
        self.name = "SGCMonteCarlo"
        self._chemical_potential = None
        self.chem_pots: List[float] = []
        self.chem_pot_names: List[str] = []
        self.chem_pot_in_ecis = False

    def _check_symbols(self):
        pass

    _CHECKPOINT_ATTRS = Montecarlo._CHECKPOINT_ATTRS + ("chem_pots", "chem_pot_names", "chem_pot_in_ecis",
                                                        "_chemical_potential")

    @property
    def chemical_potential(self):
        return self._chemical_potential

    @chemical_potential.setter
    def chemical_potential(self, chem_pot: Dict[str, float]):
        """sgc_montecarlo.py:223-261: eci[k] -= mu_k."""
        calc = self._calc()
        eci = calc.eci
        if any(k not in eci for k in chem_pot):
            raise InvalidChemicalPotentialError("A chemical potential that is currently not tracked is added.")
        self._chemical_potential = chem_pot
        if self.chem_pot_in_ecis:
            self._reset_eci_to_original(eci)
        self.chem_pots, self.chem_pot_names = [], []
        for key in sorted(chem_pot):
            self.chem_pots.append(chem_pot[key])
            self.chem_pot_names.append(key)
            eci[key] = eci.get(key, 0.0) - chem_pot[key]
        calc.update_ecis(eci)
        self.chem_pot_in_ecis = True
        self.current_energy = calc.get_energy()

    def _reset_eci_to_original(self, eci_with_chem_pot):
        for name, val in zip(self.chem_pot_names, self.chem_pots):
            eci_with_chem_pot[name] += val
        self._calc().update_ecis(eci_with_chem_pot)
        self.chem_pot_in_ecis = False
        self.current_energy = self._calc().get_energy()
        return eci_with_chem_pot

    def reset_ecis(self):
        if self.chem_pot_in_ecis:
            self._reset_eci_to_original(self._calc().eci)

    def runMC(self, mode="fixed", steps=10, verbose=False, chem_potential=None, equil=True, equil_params=None,
              prec_confidence=0.05, prec=0.01):
        """sgc_montecarlo.py:336-374."""
        if chem_potential is None and self.chemical_potential is None:
            raise ValueError("No chemicalpotentials given. Has to be dictionary of the form "
                             "{'c1_1': -0.1, 'c1_2': 0.05}")
        if chem_potential is not None:
            self.chemical_potential = chem_potential
        self.reset()
        self._include_vib()
        if equil:
            res = self._estimate_correlation_time()
            if not res["correlation_time_found"]:
                res["correlation_time_found"] = True
                res["correlation_time"] = 1000
            self._equillibriate(**(equil_params or {}))
        self.reset()
        return Montecarlo.runMC(self, mode=mode, steps=steps, verbose=verbose, equil=False,
                                prec=prec, prec_confidence=prec_confidence)

    def singlet2composition(self, avg_singlets):
        """sgc_montecarlo.py:376-396."""
        bf = self._calc().BC.basis_functions
        n = len(self.symbols)
        index = {s: i for i, s in enumerate(self.symbols)}
        matrix = np.zeros((n, n))
        for i, b in enumerate(bf):
            for s, col in index.items():
                matrix[i, col] = b[s]
        matrix[-1, :] = 1.0
        rhs = np.zeros(n)
        rhs[:-1] = avg_singlets
        rhs[-1] = 1.0
        x = np.linalg.solve(matrix, rhs)
        return {s + "_conc": x[i] for s, i in index.items()}

    def get_thermodynamic(self, reset_ecis=True):
        """sgc_montecarlo.py:398-448."""
        a = self.chain().accum_host()[0]
        m = self._calc().model
        N = max(a[E.A_NSAMP], 1.0)
        nb = m.n_bf
        singlets = a[E.A_SUM_S:E.A_SUM_S + nb] / N
        singlets_sq = a[E.A_SUM_S2:E.A_SUM_S2 + nb] / N
        mean = a[E.A_EREF] + a[E.A_SUM_E] / N
        q = {"sgc_energy": mean + self.energy_bias,
             "sgc_heat_capacity": (a[E.A_SUM_E2] / N - (a[E.A_SUM_E] / N) ** 2) / (kB * self.T ** 2),
             "energy": mean + self.energy_bias}
        natoms = len(self.atoms)
        name_to_bf = {"c1_%d" % b: b for b in range(nb)}
        for mu, name in zip(self.chem_pots, self.chem_pot_names):
            q["energy"] += mu * singlets[name_to_bf[name]] * natoms
        q["temperature"] = self.T
        q["n_mc_steps"] = int(a[E.A_NSAMP])
        for mu, name in zip(self.chem_pots, self.chem_pot_names):
            b = name_to_bf[name]
            q["singlet_{}".format(name)] = singlets[b]
            q["var_singlet_{}".format(name)] = singlets_sq[b] - singlets[b] ** 2
            q["mu_{}".format(name)] = mu
        q.update(self.meta_info)
        try:
            q.update(self.singlet2composition(singlets))
        except Exception:
            pass
        q["accept_rate"] = a[E.A_NACC] / N
        if reset_ecis:
            self._reset_eci_to_original(self._calc().eci)
        return q
