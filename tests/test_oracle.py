"""The CPU oracle against the reference: golden fixtures (always) and the live compiled reference (when built here)."""
import math

import numpy as np
import pytest

from conftest import KB, golden_cases, golden_model, load_golden


@pytest.mark.parametrize("case", golden_cases())
def test_oracle_reproduces_reference_fixture(case, oracle_mod):
    """Replaying the fixture's trials, the oracle matches the reference bit for bit."""
    from golden.make_golden import model_hash
    g = load_golden(case)
    s, m, eci = golden_model(g)
    assert model_hash(m) == str(g["model_hash"]), "cluster generator output changed"
    assert list(m.eci_names) == [str(x) for x in g["eci_names"]]
    orc = oracle_mod.Oracle(m)
    move = int(g["move"])
    st = orc.new_chain_state(g["occ0"], g["eci"], float(g["kT"]), move)
    assert np.array_equal(st.cf, g["cf0"])
    n = int(g["n_trials"])
    tr = orc.run(st, seed=int(g["seed"]), chain_id=0, t_begin=0, n_trials=n, trace=True)
    assert np.array_equal(tr.site.reshape(n, 2), g["sites"])
    assert np.array_equal(tr.u, g["u"])
    assert np.array_equal(tr.acc, g["ref_acc"])
    assert np.array_equal(tr.de, g["ref_de"])
    assert np.array_equal(st.occ, g["occ_final"])
    assert np.array_equal(st.cf, g["cf_final"])
    assert st.energy[0] == float(g["energy_final"])


@pytest.mark.parametrize("case", golden_cases())
def test_oracle_single_updates_match_reference_fixture(case, oracle_mod):
    g = load_golden(case)
    s, m, eci = golden_model(g)
    orc = oracle_mod.Oracle(m)
    occ = g["occ0"].copy()
    cf = g["cf0"].copy()
    for i, site in enumerate(g["upd_sites"]):
        cf = orc.update_cf(occ, int(site), int(g["upd_new"][i]), cf)
        occ[site] = g["upd_new"][i]
        assert np.array_equal(cf, g["upd_cf"][i])
        assert orc.energy(g["eci"], cf) == g["upd_energy"][i]


@pytest.mark.parametrize("recipe", [(4, 4, 2, 1, ["Al", "Mg"]), (4, 5, 3, 1, ["Al", "Mg", "Si"])])
def test_incremental_equals_full_recompute(recipe, oracle_mod):
    """The reference's own test invariant (tests/test_CE_updater.py:40-115): incremental == brute force."""
    from cemc_gb300.lattice import fcc_settings, seeded_ecis
    from cemc_gb300.tables import CEModel
    L, ps, ts, qs, syms = recipe
    s = fcc_settings(L, ps, ts, qs, syms)
    eci = seeded_ecis(s.cset, 0)
    m = CEModel(s, list(eci))
    orc = oracle_mod.Oracle(m)
    rng = np.random.default_rng(0)
    occ = rng.integers(0, len(syms), m.n_sites).astype(np.int8)
    cf = orc.full_cf(occ)
    for _ in range(40):
        site = int(rng.integers(m.n_sites))
        new = int((occ[site] + 1 + rng.integers(len(syms) - 1)) % len(syms))
        cf = orc.update_cf(occ, site, new, cf)
        occ[site] = new
    assert np.allclose(cf, orc.full_cf(occ), rtol=0, atol=1e-12)


def test_oracle_chain_runs_are_resumable(oracle_mod):
    """Two runs of n/2 trials equal one run of n (counter-based stream)."""
    g = load_golden("binary_swap")
    s, m, eci = golden_model(g)
    orc = oracle_mod.Oracle(m)
    a = orc.new_chain_state(g["occ0"], g["eci"], float(g["kT"]), 1)
    b = orc.new_chain_state(g["occ0"], g["eci"], float(g["kT"]), 1)
    orc.run(a, seed=3, chain_id=2, t_begin=0, n_trials=1000)
    orc.run(b, seed=3, chain_id=2, t_begin=0, n_trials=500)
    orc.run(b, seed=3, chain_id=2, t_begin=500, n_trials=500)
    assert np.array_equal(a.occ, b.occ) and np.array_equal(a.cf, b.cf)
    assert a.acc["sum_e"][0] == pytest.approx(b.acc["sum_e"][0], rel=1e-12)


def test_oracle_many_threads_equal_serial(oracle_mod):
    g = load_golden("binary_flip")
    s, m, eci = golden_model(g)
    orc = oracle_mod.Oracle(m)
    rng = np.random.default_rng(4)
    occs = rng.integers(0, 2, (6, m.n_sites)).astype(np.int8)
    ser = [orc.new_chain_state(o, g["eci"], KB * 600, 0) for o in occs]
    par = [orc.new_chain_state(o, g["eci"], KB * 600, 0) for o in occs]
    for i, st in enumerate(ser):
        orc.run(st, seed=9, chain_id=i, t_begin=0, n_trials=700)
    orc.run_many(par, seed=9, chain_ids=list(range(6)), t_begin=0, n_trials=700, n_threads=3)
    for a, b in zip(ser, par):
        assert np.array_equal(a.occ, b.occ) and np.array_equal(a.cf, b.cf)


def test_oracle_accumulators_match_python_restatement(oracle_mod):
    """Running sums equal the per-step averages the reference's runMC / SGCObserver keep."""
    g = load_golden("binary_flip")
    s, m, eci = golden_model(g)
    orc = oracle_mod.Oracle(m)
    st = orc.new_chain_state(g["occ0"], g["eci"], float(g["kT"]), 0)
    e0 = st.energy[0]
    n = 400
    tr = orc.run(st, seed=int(g["seed"]), chain_id=0, t_begin=0, n_trials=n, trace=True)
    e = e0
    es = []
    for i in range(n):
        if tr.acc[i]:
            e += tr.de[i]
        es.append(e)
    es = np.array(es) - e0
    assert st.acc["n_samples"][0] == n
    assert st.acc["sum_e"][0] == pytest.approx(es.sum(), rel=1e-9, abs=1e-9)
    assert st.acc["sum_e2"][0] == pytest.approx((es ** 2).sum(), rel=1e-9)
    assert st.acc["n_accept"][0] == int(tr.acc.sum())


def _live_reference(oracle_mod):
    mod = oracle_mod.reference_module()
    if mod is None:
        pytest.skip("reference CEUpdater not built here (oracle/build_ref.sh needs the reference sources)")
    return mod


@pytest.mark.parametrize("syms", [["Al", "Mg"], ["Al", "Mg", "Si"]])
def test_oracle_equals_live_reference_on_random_sequences(syms, oracle_mod):
    _live_reference(oracle_mod)
    from cemc_gb300.lattice import fcc_settings, seeded_ecis
    from cemc_gb300.tables import CEModel
    s = fcc_settings(4, 4 if len(syms) == 2 else 5, 2 if len(syms) == 2 else 3, 1, syms)
    eci = seeded_ecis(s.cset, 7)
    m = CEModel(s, list(eci))
    orc = oracle_mod.Oracle(m)
    rng = np.random.default_rng(8)
    occ = rng.integers(0, len(syms), m.n_sites).astype(np.int8)
    cf = orc.full_cf(occ)
    upd, _ = oracle_mod.make_reference_updater(s, m.symbols_of(occ), dict(zip(m.eci_names, cf)), eci)
    for it in range(60):
        a, b = (int(x) for x in rng.choice(m.n_sites, 2, replace=False))
        if it % 2 and occ[a] != occ[b]:
            changes = [(a, m.symbols[occ[a]], m.symbols[occ[b]]), (b, m.symbols[occ[b]], m.symbols[occ[a]])]
        else:
            new = int((occ[a] + 1 + rng.integers(len(syms) - 1)) % len(syms))
            changes = [(a, m.symbols[occ[a]], m.symbols[new])]
        e_ref = upd.calculate(changes)
        for site, _, nw in changes:
            nid = m.symbols.index(nw)
            cf = orc.update_cf(occ, site, nid, cf)
            occ[site] = nid
        assert e_ref == orc.energy(m.eci_vector(eci), cf)
        if it % 3 == 0:
            upd.undo_changes()
            for site, old, _ in reversed(changes):
                occ[site] = m.symbols.index(old)
            cf = np.array([upd.get_cf()[k] for k in m.eci_names])
        else:
            upd.clear_history()
        ref = upd.get_cf()
        assert np.array_equal(cf, [ref[k] for k in m.eci_names])


def test_reference_rejects_background_move_like_oracle(oracle_mod):
    from cemc_gb300.tables import CEModel
    from cemc_gb300.lattice import fcc_settings, seeded_ecis
    s = fcc_settings(4, 4, 2, 1, ["Al", "Mg"])
    eci = seeded_ecis(s.cset, 0)
    s.index_by_trans_symm = [list(range(1, s.n_sites))]
    s.background_indices = [0]
    m = CEModel(s, list(eci))
    orc = oracle_mod.Oracle(m)
    occ = np.zeros(m.n_sites, dtype=np.int8)
    with pytest.raises(RuntimeError, match="background"):
        orc.update_cf(occ, 0, 1, orc.full_cf(occ))
