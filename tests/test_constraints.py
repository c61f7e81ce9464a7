"""Move constraints: this package's classes and device masks against the reference's own verdicts
(tests/golden/constraints_verdicts.npz, recorded from cemc/mcmc/mc_constraints.py), and the oracle's
redraw loop against a restatement of the reference's loop (montecarlo.py:976-988) on the host."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, KB


def _fixture():
    d = np.load(os.path.join(GOLDEN, "constraints_verdicts.npz"), allow_pickle=False)
    return {k: d[k] for k in d.files}


class _Atom:
    def __init__(self, index, tag):
        self.index, self.tag = index, tag


def _atoms(g):
    class Atoms(list):
        def get_cell(self):
            return g["cell"]

        def get_positions(self):
            return g["positions"]

    return Atoms(_Atom(i, int(t)) for i, t in enumerate(g["tags"]))


def _ours(g):
    from cemc_gb300.mc_constraints import ConstrainElementByTag, FixEdgeLayers, FixedElement
    atoms = _atoms(g)
    ebt = [str(e).split("|") for e in g["element_by_tag"]]
    return [FixedElement(element=str(g["fixed_element"])), ConstrainElementByTag(atoms, ebt),
            FixEdgeLayers(thickness=float(g["thickness"]), atoms=atoms)]


def _changes(g, k):
    syms = [str(s) for s in g["symbols"]]
    return [(int(c[0]), syms[c[1]], syms[c[2]]) for c in g["moves"][k] if c[0] >= 0]


def test_constraint_classes_match_reference_verdicts():
    g = _fixture()
    cons = _ours(g)
    for k in range(len(g["moves"])):
        ch = _changes(g, k)
        for q, c in enumerate(cons):
            assert bool(c(ch)) == bool(g["verdict"][k, q]), (k, g["constraint_names"][q])


def test_device_masks_match_reference_verdicts():
    """A move is legal on the device when every change's old species is not frozen and its new species
    is allowed at its site: the same verdicts as the reference's objects, one constraint at a time."""
    from cemc_gb300.mc_constraints import PairConstraint, device_masks
    g = _fixture()
    syms = [str(s) for s in g["symbols"]]
    n = len(g["tags"])
    for q, c in enumerate(_ours(g)):
        allow, frozen = device_masks(c, syms, n)
        for k in range(len(g["moves"])):
            legal = True
            for site, old, new in (tuple(int(x) for x in m) for m in g["moves"][k] if m[0] >= 0):
                if (frozen >> old) & 1 or (allow is not None and not (int(allow[site]) >> new) & 1):
                    legal = False
            assert legal == bool(g["verdict"][k, q]), (k, g["constraint_names"][q])
    # PairConstraint as the reference ships it accepts every move (see its docstring)
    pc = PairConstraint(calc=object(), cluster_name="c2_d0000_0", elements=["Al", "Mg"])
    assert pc([(0, "Al", "Mg")]) and device_masks(pc, syms, n) == (None, 0)
    with pytest.raises(ValueError):
        PairConstraint(calc=object(), cluster_name="c3_d0000_0", elements=["Al", "Mg"])

    class Custom:
        def __call__(self, changes):
            return True

    with pytest.raises(NotImplementedError):
        device_masks(Custom(), syms, n)


def _redraw_flip(rng_mod, seed, key, t, occ, movable, n_sym, allow, frozen, max_att):
    """Host restatement of the device redraw loop for a flip (proposal k from counter stream 2k)."""
    att = 0
    while True:
        w = rng_mod.trial_draw(seed, key, t, 2 * att)
        site = int(movable[rng_mod.below(w[0], len(movable))])
        old = int(occ[site])
        k = rng_mod.below(w[1], n_sym - 1)
        new = k + (k >= old)
        legal = not (frozen >> old) & 1 and (allow is None or (int(allow[site]) >> new) & 1)
        if legal or att == max_att:
            return site, new, att == max_att
        att += 1


def test_oracle_redraw_loop_follows_the_reference(oracle_mod):
    """Every trial of a constrained oracle run proposes the first legal redraw (or fails after
    max_attempts, then rejected); the chain never changes a frozen or disallowed site."""
    from cemc_gb300 import rng as R
    from cemc_gb300.lattice import fcc_settings, seeded_ecis
    from cemc_gb300.tables import CEModel
    s = fcc_settings(4, 3, 2, 0, ["Al", "Mg", "Si"])
    eci = seeded_ecis(s.cset, 0)
    m = CEModel(s, list(eci))
    orc = oracle_mod.Oracle(m)
    rng = np.random.default_rng(4)
    occ0 = rng.integers(0, 3, m.n_sites).astype(np.int8)
    # Mg sites never change and no Mg is inserted (FixedElement alone lets the element in but never
    # out, which freezes ever more sites), 60 fixed sites, no Si on one sublattice
    allow = np.full(m.n_sites, 0b101, dtype=np.uint8)
    allow[rng.choice(m.n_sites, 60, replace=False)] = 0
    allow[np.arange(m.n_sites) % 4 == 1] &= 0b001
    frozen = 1 << 1
    st = orc.new_chain_state(occ0, m.eci_vector(eci), KB * 900.0, 0, allow=allow, frozen=frozen, max_attempts=50)
    occ = occ0.copy()
    n = 3000
    tr = orc.run(st, seed=9, chain_id=3, t_begin=0, n_trials=n, trace=True)
    for t in range(n):
        site, new, failed = _redraw_flip(R, 9, 3, t, occ, m.movable, m.n_sym, allow, frozen, 50)
        assert (tr.site[2 * t], tr.site[2 * t + 1]) == (site, new)
        assert not failed
        if tr.acc[t]:
            occ[site] = new
    assert np.array_equal(st.occ, occ)
    changed = occ != occ0
    assert not np.any(changed & (allow == 0)) and not np.any(changed & (occ0 == 1))
    assert not np.any((occ == 2) & (occ0 != 2) & (np.arange(m.n_sites) % 4 == 1))


def test_oracle_reports_exhausted_redraws(oracle_mod):
    """No legal move at all: every trial fails after max_attempts redraws and is rejected."""
    from cemc_gb300.lattice import fcc_settings, seeded_ecis
    from cemc_gb300.tables import CEModel
    s = fcc_settings(4, 3, 2, 0, ["Al", "Mg"])
    eci = seeded_ecis(s.cset, 0)
    m = CEModel(s, list(eci))
    orc = oracle_mod.Oracle(m)
    occ = (np.arange(m.n_sites) % 2).astype(np.int8)
    st = orc.new_chain_state(occ, m.eci_vector(eci), KB * 900.0, 1, frozen=0b01, max_attempts=5)
    with pytest.raises(oracle_mod.NoLegalMove) as ei:
        orc.run(st, seed=1, chain_id=0, t_begin=0, n_trials=20, trace=True)
    assert not ei.value.trace.acc.any()
    assert np.array_equal(st.occ, occ)


def test_oracle_accepts_the_first_trial_when_asked(oracle_mod):
    """accept_first_trial_move_after_reset (montecarlo.py:932-935): the run's first trial is accepted
    whatever its energy change; the rest follow Metropolis."""
    from cemc_gb300.lattice import fcc_settings, seeded_ecis
    from cemc_gb300.tables import CEModel
    s = fcc_settings(4, 3, 2, 0, ["Al", "Mg"])
    eci = seeded_ecis(s.cset, 0)
    m = CEModel(s, list(eci))
    orc = oracle_mod.Oracle(m)
    occ = np.random.default_rng(8).integers(0, 2, m.n_sites).astype(np.int8)
    for seed in range(50):  # a stream whose first proposal raises the energy
        plain = orc.new_chain_state(occ, m.eci_vector(eci), KB * 5.0, 1)
        tr0 = orc.run(plain, seed=seed, chain_id=0, t_begin=0, n_trials=50, trace=True)
        if tr0.de[0] > 0:
            break
    assert tr0.de[0] > 0 and tr0.acc[0] == 0
    first = orc.new_chain_state(occ, m.eci_vector(eci), KB * 5.0, 1, accept_first=1)
    tr1 = orc.run(first, seed=seed, chain_id=0, t_begin=0, n_trials=50, trace=True)
    assert tr1.acc[0] == 1 and tr1.de[0] == tr0.de[0]
    assert np.array_equal(tr0.site[:2], tr1.site[:2])


@pytest.mark.parametrize("move", [0, 1])
def test_oracle_waste_recycling_follows_the_reference(move, oracle_mod):
    """Waste recycling (montecarlo.py:937-948, util.py:41-63, mc_observers.py:231-258): acceptance
    u > w0 / (w0 + w1) with w = exp(-(E - min E) / kT) over (current, proposed); every trial adds
    w-weighted energies of the current and proposed states and the calculator's singlets before and
    after the step.  Replayed here from the trace with the reference's own formulas."""
    from cemc_gb300.lattice import fcc_settings, seeded_ecis
    from cemc_gb300.tables import CEModel
    s = fcc_settings(4, 3, 2, 0, ["Al", "Mg"])
    eci = seeded_ecis(s.cset, 0)
    m = CEModel(s, list(eci))
    orc = oracle_mod.Oracle(m)
    occ = np.random.default_rng(2).integers(0, 2, m.n_sites).astype(np.int8)
    kT = KB * 700.0
    st = orc.new_chain_state(occ, m.eci_vector(eci), kT, move, recycle=1)
    e0 = float(st.energy[0])
    e_ref = float(st.acc[0]["e_ref"])
    bf = m.bf[0]
    s_cur = float(np.mean(bf[occ]))
    n = 1500
    tr = orc.run(st, seed=3, chain_id=1, t_begin=0, n_trials=n, trace=True)

    def recycled(obs, energies):  # util.waste_recycled_average
        w = np.exp(-(energies - energies.min()) / kT)
        return float(obs.dot(w) / w.sum())

    e_cur = e0
    cur = occ.copy()
    sums = np.zeros(5)
    for t in range(n):
        energies = np.array([e_cur, e_cur + tr.de[t]])
        w = np.exp(-(energies - energies.min()) / kT)
        assert bool(tr.acc[t]) == bool(tr.u[t] > (w / w.sum())[0])
        a, b = int(tr.site[2 * t]), int(tr.site[2 * t + 1])
        s_new = s_cur
        if tr.acc[t]:
            if move == 0:
                s_new += (bf[b] - bf[cur[a]]) / m.n_sites
                cur[a] = b
            else:
                cur[a], cur[b] = cur[b], cur[a]
        sl = np.array([s_cur, s_new])
        rel = energies - e_ref
        sums += [recycled(rel, energies), recycled(rel ** 2, energies), recycled(sl, energies),
                 recycled(sl ** 2, energies), recycled(sl * rel, energies)]
        if tr.acc[t]:
            e_cur += tr.de[t]
            s_cur = s_new
    o = st.acc[0]
    got = np.array([o["sum_e"], o["sum_e2"], o["sum_s"][0], o["sum_s2"][0], o["sum_se"][0]])
    assert np.allclose(got, sums, rtol=1e-9, atol=1e-9)
    assert np.array_equal(st.occ, cur)
