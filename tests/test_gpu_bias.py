"""Bias potentials on the GPU drivers against a restatement of the reference's biased acceptance.

The reference adds, for every trial, the value of each bias potential for the
state after the proposed move to that state's energy, and keeps the current
state's bias in its current energy (cemc/mcmc/montecarlo.py:276-282, 919-956,
993-998).  The restatement below runs the same trials (same counter-based
proposals and uniforms, same swap site lists) with the oracle's FP64 updater
for the cluster-expansion energies and the same bias object, and the drivers
must reproduce its decisions bit for bit, its final occupation, its current
energy and its running sums (1e-9 relative).
"""
import numpy as np
import pytest

from conftest import KB

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


class BlockCountBias:
    """lam * n^2 / block with n the atoms of `symbol` on sites [0, block): a bias on a local order
    parameter, so it depends on where atoms sit, not only on the composition.  The reference's
    BiasPotential interface: __call__(system_changes) on the system with the changes applied,
    calculate_from_scratch(atoms)."""

    def __init__(self, atoms, lam, symbol="Mg", block=64):
        self.atoms, self.lam, self.symbol, self.block = atoms, lam, symbol, block

    def calculate_from_scratch(self, atoms):
        n = sum(1 for i in range(self.block) if atoms[i].symbol == self.symbol)
        return self.lam * n * n / self.block

    def __call__(self, system_changes):
        return self.calculate_from_scratch(self.atoms)


def _calc(seed=0):
    from cemc_gb300.calculator import CE, SimpleAtoms
    from cemc_gb300.lattice import fcc_settings, seeded_ecis
    s = fcc_settings(4, 4, 2, 1, ["Al", "Mg"])
    eci = seeded_ecis(s.cset, 0)
    rng = np.random.default_rng(seed)
    atoms = SimpleAtoms([["Al", "Mg"][i] for i in rng.integers(0, 2, s.n_sites)])
    return atoms, CE(atoms, s, eci=dict(eci))


def _restated_run(oracle_mod, m, occ0, ev, T, seed, n, swap, lam, first=False):
    """The reference's biased _mc_step loop over the same stream, energies from the oracle."""
    from cemc_gb300.calculator import SimpleAtoms
    from cemc_gb300.engine import build_tracker
    from cemc_gb300.rng import below, trial_draw, u01_53
    orc = oracle_mod.Oracle(m)
    occ = occ0.astype(np.int64).copy()
    cf = orc.full_cf(occ.astype(np.int8))
    e_ce = orc.energy(ev, cf)
    atoms = SimpleAtoms([m.symbols[i] for i in occ])
    bias = BlockCountBias(atoms, lam)
    current = e_ce + bias.calculate_from_scratch(atoms)
    trk, loc, start, count = (x[0] for x in build_tracker(occ[None].astype(np.int8), m.n_sym, m.background))
    present = [s for s in range(m.n_sym) if count[s] > 0]
    kT = KB * T
    acc_out = np.zeros(n, dtype=np.int8)
    sums = np.zeros(2)
    e_ref = e_ce
    for t in range(n):
        w = trial_draw(seed, 0, t, 0)
        if swap:
            x = trial_draw(seed, 0, t, 1)
            ia = below(w[0], len(present))
            ib = below(w[1], len(present) - 1)
            ib += ib >= ia
            A, B = present[ia], present[ib]
            a = int(trk[start[A] + below(w[2], int(count[A]))])
            b = int(trk[start[B] + below(w[3], int(count[B]))])
            ids = [(a, A, B), (b, B, A)]
            ua, ub = x[0], x[1]
        else:
            a = int(below(w[0], m.n_sites))
            kk = below(w[1], m.n_sym - 1)
            ids = [(a, int(occ[a]), kk + (kk >= occ[a]))]
            ua, ub = w[2], w[3]
        o2, c2 = occ.copy(), cf
        for s, _, v in ids:
            c2 = orc.update_cf(o2.astype(np.int8), s, v, c2)
            o2[s] = v
        e_new_ce = orc.energy(ev, c2)
        for s, _, v in ids:
            atoms[s].symbol = m.symbols[v]
        new = e_new_ce + bias([(s, m.symbols[o], m.symbols[v]) for s, o, v in ids])
        if first and t == 0:
            accept = True
        elif new < current:
            accept = True
        else:
            accept = u01_53(ua, ub) <= np.exp(-(new - current) / kT)
        if accept:
            occ, cf, e_ce, current = o2, c2, e_new_ce, new
            if swap:
                (a, A, B), (b, _, _) = ids
                la, lb = int(loc[a]), int(loc[b])
                trk[start[A] + la], loc[b] = b, la
                trk[start[B] + lb], loc[a] = a, lb
        else:
            for s, o, _ in ids:
                atoms[s].symbol = m.symbols[o]
        acc_out[t] = accept
        sums += [current - e_ref, (current - e_ref) ** 2]
    return acc_out, occ, current, sums


@pytest.mark.parametrize("sgc", [False, True])
def test_biased_driver_matches_restated_reference(sgc, torch_cuda, oracle_mod):
    from cemc_gb300 import engine as E
    from cemc_gb300.mcmc import Montecarlo, SGCMonteCarlo
    atoms, calc = _calc(seed=3)
    m = calc.model
    T, seed, n, lam = 500.0, 123, 600, 0.05
    if sgc:
        mc = SGCMonteCarlo(atoms, T, seed=seed)
        mc.chemical_potential = {"c1_0": 0.01}
    else:
        mc = Montecarlo(atoms, T, seed=seed)
    mc.add_bias(BlockCountBias(atoms, lam))
    occ0 = m.occupation([a.symbol for a in atoms])
    ev = m.eci_vector(calc.eci)
    mc.update_current_energy()
    (sites, acc, de), = mc._run_trials(n, trace=True)
    acc = acc.numpy()[0]
    ref_acc, ref_occ, ref_current, ref_sums = _restated_run(oracle_mod, m, occ0, ev, T, seed, n, not sgc, lam)
    assert 0 < acc.sum() < n
    assert np.array_equal(acc, ref_acc)
    assert np.array_equal(calc.updater.occupation(), ref_occ)
    assert [a.symbol for a in atoms] == [m.symbols[i] for i in ref_occ]
    assert mc.current_energy == pytest.approx(ref_current, rel=1e-9, abs=1e-9)
    h = mc.chain().accum_host()[0]
    assert h[E.A_NSAMP] == n and h[E.A_NACC] == acc.sum()
    # both sums are taken relative to the cluster-expansion energy of the starting state
    assert h[E.A_SUM_E] == pytest.approx(ref_sums[0], rel=1e-9, abs=1e-7)
    assert h[E.A_SUM_E2] == pytest.approx(ref_sums[1], rel=1e-9, abs=1e-7)


def test_biased_run_continues_the_device_chain(torch_cuda, oracle_mod):
    """Trials after the bias is removed continue the same counter-based chain on the kernel path."""
    from cemc_gb300.mcmc import Montecarlo
    atoms, calc = _calc(seed=5)
    m = calc.model
    mc = Montecarlo(atoms, 700.0, seed=9)
    mc.add_bias(BlockCountBias(atoms, 0.0))  # a zero bias: same decisions as the unbiased chain
    mc.update_current_energy()
    occ0 = m.occupation([a.symbol for a in atoms])
    mc._run_trials(300)
    mc.bias_potentials.clear()
    mc._run_trials(700)
    orc = oracle_mod.Oracle(m)
    st = orc.new_chain_state(occ0, m.eci_vector(calc.eci), KB * 700.0, oracle_mod.MOVE_SWAP)
    orc.run(st, seed=9, chain_id=0, t_begin=0, n_trials=1000)
    assert np.array_equal(calc.updater.occupation(), st.occ)
    assert np.allclose(calc.updater.cf(), st.cf, rtol=1e-9, atol=1e-13)
