"""Drop-in calculator and drivers on the GPU: the reference's call sequences, its test invariants, serving."""
import math

import numpy as np
import pytest

from conftest import KB, golden_model, load_golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _calc(recipe=(4, 4, 2, 1, ("Al", "Mg")), seed=0, eci_seed=0):
    from cemc_gb300.calculator import CE, SimpleAtoms
    from cemc_gb300.lattice import fcc_settings, seeded_ecis
    L, ps, ts, qs, syms = recipe
    s = fcc_settings(L, ps, ts, qs, list(syms))
    eci = seeded_ecis(s.cset, eci_seed)
    rng = np.random.default_rng(seed)
    symbols = [syms[i] for i in rng.integers(0, len(syms), s.n_sites)]
    atoms = SimpleAtoms(symbols)
    calc = CE(atoms, s, eci=dict(eci))
    return atoms, calc, s, eci


def test_calculator_swap_sequences_match_full_recompute(torch_cuda, oracle_mod):
    """tests/test_CE_updater.py:86-115 (double swaps): incremental cf == brute force after each swap."""
    atoms, calc, s, eci = _calc(recipe=(4, 5, 3, 1, ("Al", "Mg", "Si")))
    m = calc.model
    orc = oracle_mod.Oracle(m)
    rng = np.random.default_rng(1)
    for _ in range(15):
        i1 = int(rng.integers(m.n_sites))
        s1 = atoms[i1].symbol
        i2, s2 = i1, s1
        while s2 == s1:
            i2 = int(rng.integers(m.n_sites))
            s2 = atoms[i2].symbol
        e = calc.calculate(atoms, ["energy"], [(i1, s1, s2), (i2, s2, s1)])
        cf = calc.get_cf()
        brute = orc.full_cf(m.occupation([a.symbol for a in atoms]))
        assert np.allclose([cf[k] for k in m.eci_names], brute, rtol=1e-9, atol=1e-13)
        assert e == pytest.approx(orc.energy(m.eci_vector(eci), brute), rel=1e-9)
        calc.clear_history()


def test_calculator_undo_restores_state(torch_cuda):
    atoms, calc, s, eci = _calc()
    cf0 = calc.get_cf()
    e0 = calc.get_energy()
    sym0 = [a.symbol for a in atoms]
    calc.calculate(atoms, ["energy"], [(0, atoms[0].symbol, "Mg" if atoms[0].symbol == "Al" else "Al")])
    calc.calculate(atoms, ["energy"], [(5, atoms[5].symbol, "Mg" if atoms[5].symbol == "Al" else "Al")])
    calc.calculate(atoms, ["energy"], [(0, atoms[0].symbol, "Mg" if atoms[0].symbol == "Al" else "Al")])
    assert calc.get_energy() != e0
    calc.undo_changes()
    assert [a.symbol for a in atoms] == sym0
    assert calc.get_cf() == cf0 and calc.get_energy() == e0


def test_calculator_rejects_inconsistent_move(torch_cuda):
    atoms, calc, s, eci = _calc()
    wrong = "Mg" if atoms[3].symbol == "Al" else "Al"
    with pytest.raises(RuntimeError):
        calc.calculate(atoms, ["energy"], [(3, wrong, atoms[3].symbol)])


def test_calculator_singlets_update_ecis_and_set_symbols(torch_cuda, oracle_mod):
    atoms, calc, s, eci = _calc()
    m = calc.model
    sing = calc.get_singlets()
    occ = m.occupation([a.symbol for a in atoms])
    assert sing[0] == pytest.approx(np.mean(np.where(occ == 0, 1.0, -1.0)), abs=1e-14)
    new = dict(eci)
    new["c1_0"] += 0.05
    calc.update_ecis(new)
    cf = calc.get_cf()
    assert calc.get_energy() == pytest.approx(m.n_sites * sum(new[k] * cf[k] for k in m.eci_names), rel=1e-12)
    calc.set_composition({"Al": 0.75, "Mg": 0.25})
    assert sum(a.symbol == "Mg" for a in atoms) == m.n_sites // 4
    orc = oracle_mod.Oracle(m)
    brute = orc.full_cf(m.occupation([a.symbol for a in atoms]))
    assert np.allclose([calc.get_cf()[k] for k in m.eci_names], brute, atol=1e-13)


def test_montecarlo_runmc_accounting_and_thermodynamics(torch_cuda, oracle_mod):
    from cemc_gb300.mcmc import Montecarlo
    atoms, calc, s, eci = _calc(recipe=(4, 4, 2, 1, ("Al", "Mg")))
    c0 = calc.eci["c0"]
    mc = Montecarlo(atoms, 600.0, seed=5)
    mc.runMC(mode="fixed", steps=5000, equil=False)
    q = mc.get_thermodynamic()
    for key in ("energy", "heat_capacity", "energy_std", "temperature", "Al_conc", "Mg_conc"):
        assert key in q
    assert mc.current_step == 5000
    assert calc.eci["c0"] == pytest.approx(c0, abs=1e-12)  # bias added back (montecarlo.py:213-217)
    # composition is conserved by swaps; energy consistent with a recompute
    m = calc.model
    orc = oracle_mod.Oracle(m)
    occ = calc.updater.occupation()
    assert np.array_equal(occ, m.occupation([a.symbol for a in atoms]))
    brute = orc.full_cf(occ)
    assert calc.get_energy() == pytest.approx(orc.energy(m.eci_vector(calc.eci), brute), rel=1e-9)
    assert q["heat_capacity"] >= 0.0


def test_montecarlo_equilibration_and_prec_mode(torch_cuda):
    from cemc_gb300.mcmc import Montecarlo
    atoms, calc, s, eci = _calc(recipe=(4, 4, 2, 1, ("Al", "Mg")))
    mc = Montecarlo(atoms, 2000.0, seed=7)
    mc.runMC(mode="prec", steps=20000, equil=True, prec=1.0)
    q = mc.get_thermodynamic()
    assert np.isfinite(q["energy"]) and mc.current_step <= 20000


def test_sgc_runmc_and_thermodynamics(torch_cuda):
    from cemc_gb300.mcmc import SGCMonteCarlo
    atoms, calc, s, eci = _calc(recipe=(4, 4, 2, 1, ("Al", "Mg")))
    c1 = calc.eci["c1_0"]
    mc = SGCMonteCarlo(atoms, 800.0, seed=3)
    mc.runMC(mode="fixed", steps=8000, chem_potential={"c1_0": 0.15}, equil=False)
    q = mc.get_thermodynamic()
    for key in ("sgc_energy", "sgc_heat_capacity", "energy", "temperature", "n_mc_steps", "singlet_c1_0",
                "var_singlet_c1_0", "mu_c1_0", "Al_conc", "Mg_conc"):
        assert key in q, key
    assert q["n_mc_steps"] == 8000
    assert q["Al_conc"] + q["Mg_conc"] == pytest.approx(1.0)
    assert calc.eci["c1_0"] == pytest.approx(c1, abs=1e-12)  # chemical potential removed again
    # energy = sgc_energy + mu * <singlet> * N (sgc_montecarlo.py:419-422)
    assert q["energy"] == pytest.approx(q["sgc_energy"] + 0.15 * q["singlet_c1_0"] * len(atoms), rel=1e-12)


def test_sgc_chemical_potential_shifts_composition(torch_cuda):
    """A positive mu on c1_0 favours the species with bf = +1 (thermodynamic sanity, sgc_montecarlo.py:239-261)."""
    from cemc_gb300.mcmc import SGCMonteCarlo
    res = []
    for mu in (-0.3, 0.3):
        atoms, calc, s, eci = _calc(recipe=(4, 4, 2, 1, ("Al", "Mg")), seed=4)
        mc = SGCMonteCarlo(atoms, 1000.0, seed=11)
        mc.runMC(steps=20000, chem_potential={"c1_0": mu}, equil=False)
        res.append(mc.get_thermodynamic()["singlet_c1_0"])
    assert res[1] > res[0]


def test_parallel_tempering_ladder(torch_cuda):
    from cemc_gb300 import engine as E
    from cemc_gb300.parallel_tempering import ParallelTempering
    from cemc_gb300.lattice import fcc_settings, seeded_ecis
    from cemc_gb300.tables import CEModel
    s = fcc_settings(4, 4, 2, 1, ["Al", "Mg"])
    eci = seeded_ecis(s.cset, 0)
    m = CEModel(s, list(eci))
    geo = E.Geometry(m)
    occ = np.zeros(m.n_sites, dtype=np.int8)
    occ[: m.n_sites // 2] = 1
    pt = ParallelTempering(geo, occ, m.eci_vector(eci), temperatures=np.geomspace(200, 1500, 8), seed=1, warps=8)
    pt.run(sweeps_per_cycle=2, num_exchange_cycles=6, record=True)
    lad = pt.ladder()
    assert sorted(x["chain"] for x in lad) == list(range(8))
    kT = pt.cb.kT.cpu().numpy()
    for x in lad:
        assert kT[x["chain"]] == pytest.approx(KB * x["temperature"])
        assert x["n_mc_steps"] == 6 * 2 * m.n_sites
    assert sum(pt.accepted_exchanges) > 0
    # composition conserved in every replica (canonical swaps)
    assert np.all(pt.cb.occ.cpu().numpy().sum(axis=1) == m.n_sites // 2)


def test_server_result_same_alone_and_in_a_mix(torch_cuda):
    """North-star serving property: a job's result does not depend on what else is on the GPU."""
    from cemc_gb300.server import Job, MCServer
    def make(seed, L=4, recipe="binary", ens="sgc", sweeps=30):
        return Job(L=L, recipe=recipe, ensemble=ens, T=700.0, mu=0.05, sweeps=sweeps, seed=seed)
    alone = MCServer(quantum_sweeps=7, capacity=8)
    a = alone.submit(make(42))
    alone.run_until_idle()
    mixed = MCServer(quantum_sweeps=7, capacity=8)
    others = [make(100 + i, L=4 + (i % 2), recipe=("binary", "ternary")[i % 2], ens=("sgc", "canonical")[i % 2],
                   sweeps=10 + 13 * i) for i in range(9)]
    for j in others[:4]:
        mixed.submit(j)
    b = mixed.submit(make(42))
    mixed.step()
    for j in others[4:]:
        mixed.submit(j)
    mixed.run_until_idle()
    assert a.result is not None and b.result is not None
    assert np.array_equal(a.result["occupation"], b.result["occupation"])
    assert np.array_equal(a.result["cf"], b.result["cf"])
    assert a.result["energy"] == b.result["energy"]
    st = mixed.stats()
    assert st["jobs"] == 10 and st["p99_latency_s"] >= st["p50_latency_s"] > 0
    for j in others:
        assert j.result["n_mc_steps"] == int(round(j.sweeps * (4 * j.L ** 3)))


def test_server_budget_binds_with_schedules_and_own_settings(torch_cuda):
    """A device-memory budget that holds one batch at a time: jobs of other batches wait, idle batches
    (and their geometries) are released for them, memory use never exceeds the budget, and every result
    -- a job with its own settings object (a BCC cell) and a two-segment T / mu schedule among them --
    equals the job's result alone on an unconstrained server."""
    from cemc_gb300.lattice import cubic_settings, seeded_ecis
    from cemc_gb300.server import Job, MCServer, group_bytes
    bcc = cubic_settings("bcc", 4, 3, 2, 0, ["Al", "Mg"])
    bcc_eci = dict(seeded_ecis(bcc.cset, 1))

    def jobs():
        return [Job(L=4, recipe="binary", ensemble="sgc", T=900.0, mu=0.02, sweeps=20, seed=1),
                Job(L=4, recipe="binary", ensemble="canonical", T=700.0, sweeps=15, seed=2),
                Job(L=0, settings=bcc, eci=bcc_eci, ensemble="sgc", schedule=[(10, 1200.0, 0.0), (12, 500.0, 0.05)],
                    seed=3),
                Job(L=6, recipe="binary", ensemble="sgc", T=800.0, sweeps=10, seed=4)]

    kw = dict(capacity=4, quantum_sweeps=3.0, quantum_trials=1)
    alone = []
    for j in jobs():
        srv = MCServer(hbm_budget_gb=8.0, **kw)
        srv.submit(j)
        srv.run_until_idle()
        alone.append(j)
    probe = MCServer(hbm_budget_gb=8.0, **kw)
    sizes = []
    for j in jobs():
        m, geo, _ = probe._model(j)
        move = 0 if j.ensemble == "sgc" else 1
        sizes.append(geo.device_bytes() + group_bytes(geo, m, move, probe._capacity(m)))
    big = int(np.argmax(sizes))
    budget = 1.02 * sizes[big]
    assert budget < sizes[big] + min(sizes[:big] + sizes[big + 1:])  # the largest batch only fits alone
    srv = MCServer(hbm_budget_gb=budget / 1e9, **kw)
    js = [srv.submit(j) for j in jobs()]
    srv.run_until_idle()
    assert len(srv.finished) == 4 and all("error" not in j.result for j in js)
    assert srv.peak_used <= srv.budget
    others = [j for k, j in enumerate(js) if k != big]
    assert js[big].admitted >= max(j.done for j in others)  # it waited until the others' memory was released
    for a, b in zip(alone, js):
        assert np.array_equal(a.result["occupation"], b.result["occupation"])
        assert np.array_equal(a.result["cf"], b.result["cf"])
        assert a.result["energy"] == b.result["energy"]
    seg = js[2].result["segments"]
    assert [round(x["temperature"]) for x in seg] == [1200, 500] and [x["mu"] for x in seg] == [0.0, 0.05]
    assert [x["n_mc_steps"] for x in seg] == [10 * 128, 12 * 128]
    small = MCServer(hbm_budget_gb=1e-6, **kw)
    j = small.submit(jobs()[0])
    small.run_until_idle()
    assert "error" in j.result


def test_fp32_drift_and_recompute_at_benchmark_size(torch_cuda):
    """64 chains x 16384 sites, FP32 energy changes: incremental cf/energy vs the FP64 recompute after 3 sweeps."""
    import torch
    from cemc_gb300 import engine as E
    from cemc_gb300.batch import fold_chemical_potential, sgc_grid
    from cemc_gb300.lattice import fcc_settings, seeded_ecis
    from cemc_gb300.tables import CEModel
    s = fcc_settings(16, 4, 2, 1, ["Al", "Mg"])
    eci = seeded_ecis(s.cset, 0)
    m = CEModel(s, list(eci))
    geo = E.Geometry(m)
    rng = np.random.default_rng(0)
    occ = rng.integers(0, 2, (64, m.n_sites)).astype(np.int8)
    Ts, mus = sgc_grid()
    ev = fold_chemical_potential(m, m.eci_vector(eci), mus)
    cb = E.ChainBatch(geo, occ, ev, KB * Ts, E.MOVE_FLIP, seed=3)
    cb.run(3 * m.n_sites, precision=E.PREC_F32, warps=16)
    torch.cuda.synchronize()
    cf_inc, e_inc = cb.cf.cpu().numpy().copy(), cb.energy.cpu().numpy().copy()
    cb.recompute()
    torch.cuda.synchronize()
    cf_full, e_full = cb.cf.cpu().numpy(), cb.energy.cpu().numpy()
    assert np.max(np.abs(cf_inc - cf_full)) < 1e-9  # binary products are exact in FP32
    assert np.max(np.abs(e_inc - e_full)) < 1e-6
    # singlet = mean spin (a size-independent identity)
    spins = np.where(cb.occ.cpu().numpy() == 0, 1.0, -1.0).mean(axis=1)
    assert np.allclose(cf_full[:, m.eci_names.index("c1_0")], spins, atol=1e-14)


def test_multi_geometry_graph_equals_separate_batches(torch_cuda):
    """One CUDA graph over chains of three supercell sizes (and both move types) steps each
    group exactly as its own batch runner does."""
    from cemc_gb300 import engine as E
    from cemc_gb300.batch import BatchRunner, MultiBatchRunner
    from cemc_gb300.lattice import fcc_settings, seeded_ecis
    from cemc_gb300.tables import CEModel
    specs = [(4, (4, 2, 1), ("Al", "Mg"), E.MOVE_FLIP), (5, (5, 3, 1), ("Al", "Mg", "Si"), E.MOVE_SWAP),
             (6, (4, 2, 1), ("Al", "Mg"), E.MOVE_SWAP)]

    def runners():
        out = []
        for L, sh, syms, move in specs:
            s = fcc_settings(L, *sh, list(syms))
            eci = seeded_ecis(s.cset, L)
            m = CEModel(s, list(eci))
            geo = E.Geometry(m)
            rng = np.random.default_rng(L)
            occ = rng.integers(0, len(syms), (3, m.n_sites)).astype(np.int8)
            out.append(BatchRunner(geo, occ, m.eci_vector(eci), [500.0, 900.0, 1300.0], move, seed=3 + L,
                                   precision=E.PREC_F32, warps=8, sweeps_per_step=2.0, graph=True))
        return out

    alone = runners()
    for r in alone:
        r.step(3)
        r.synchronize()
    multi = MultiBatchRunner(runners())
    multi.step(3)
    multi.synchronize()
    for a, b in zip(alone, multi.runners):
        a.cb.check_status()
        b.cb.check_status()
        assert np.array_equal(a.cb.occ.cpu().numpy(), b.cb.occ.cpu().numpy())
        assert np.array_equal(a.cb.cf.cpu().numpy(), b.cb.cf.cpu().numpy())
        assert np.array_equal(a.cb.accum_host(), b.cb.accum_host())


def test_table_form_leaves_exact_correlation_functions(torch_cuda, oracle_mod):
    """The table form ends cemc_run with the full recompute: CFs and energy equal the oracle's
    full recompute of the final occupation, and callers see kernel_used = table."""
    from cemc_gb300 import engine as E
    from cemc_gb300.lattice import fcc_settings, seeded_ecis
    from cemc_gb300.tables import CEModel
    s = fcc_settings(5, 5, 3, 1, ["Al", "Mg", "Si"])
    eci = seeded_ecis(s.cset, 2)
    m = CEModel(s, list(eci))
    geo = E.Geometry(m)
    orc = oracle_mod.Oracle(m)
    rng = np.random.default_rng(4)
    occ = rng.integers(0, 3, (4, m.n_sites)).astype(np.int8)
    for move in (E.MOVE_FLIP, E.MOVE_SWAP):
        cb = E.ChainBatch(geo, occ, m.eci_vector(eci), KB * 700.0, move, seed=9)
        cb.run(4 * m.n_sites, precision=E.PREC_F32, warps=12, kernel=E.KERNEL_TABLE)
        torch_cuda.cuda.synchronize()
        assert cb.last_kernel == E.KERNEL_TABLE and cb.recomputed
        for c in range(4):
            o = cb.occ.cpu().numpy()[c]
            full = orc.full_cf(o)
            assert np.allclose(cb.cf.cpu().numpy()[c], full, rtol=1e-12, atol=1e-15)
            assert abs(cb.energy.cpu().numpy()[c] - orc.energy(m.eci_vector(eci), full)) < 1e-9 * abs(
                orc.energy(m.eci_vector(eci), full))


@pytest.mark.parametrize("driver", ["canonical", "sgc"])
def test_montecarlo_checkpoint_resume_is_exact(driver, torch_cuda, tmp_path):
    """A driver saved mid-run and loaded again continues bit for bit like one that never stopped
    (Montecarlo.save / load, montecarlo.py:1040-1074)."""
    torch = torch_cuda
    from cemc_gb300.mcmc import Montecarlo, SGCMonteCarlo

    def make():
        atoms, calc, s, eci = _calc(recipe=(4, 4, 2, 1, ("Al", "Mg")), seed=2)
        if driver == "sgc":
            mc = SGCMonteCarlo(atoms, 900.0, seed=21)
            mc.chemical_potential = {"c1_0": 0.05}
        else:
            mc = Montecarlo(atoms, 700.0, seed=21)
        return mc

    a = make()
    a._run_trials(7000)
    path = str(tmp_path / "mc.ckpt")
    a.save(path)
    a._run_trials(9000)
    b = Montecarlo.load(path)
    assert type(b) is type(a) and b.current_step == 7000
    b._run_trials(9000)
    ca, cb = a.chain(), b.chain()
    for name in ("occ", "cf", "energy", "trial", "accum", "eci", "kT"):
        assert torch.equal(getattr(ca, name), getattr(cb, name)), name
    if driver == "canonical":
        assert torch.equal(ca.trk, cb.trk) and torch.equal(ca.loc, cb.loc)
    assert [x.symbol for x in a.atoms] == [x.symbol for x in b.atoms]
    qa, qb = a.get_thermodynamic(), b.get_thermodynamic()
    for k, v in qa.items():
        if k != "timestamp":
            assert qb[k] == v, k


@pytest.mark.parametrize("move", [0, 1])
def test_chain_batch_checkpoint_resume_is_exact(move, torch_cuda, tmp_path):
    """ChainBatch.save / load: a batch restored from a checkpoint continues identically."""
    torch = torch_cuda
    from cemc_gb300 import engine as E
    g = load_golden("ternary_swap")
    s, m, eci = golden_model(g)
    geo = E.Geometry(m)
    rng = np.random.default_rng(3)
    occ = rng.integers(0, m.n_sym, (5, m.n_sites)).astype(np.int8)
    kT = KB * np.linspace(500, 1500, 5)
    a = E.ChainBatch(geo, occ, g["eci"], kT, move, seed=77, chain_keys=[4, 1, 9, 2, 6])
    a.run(3000, warps=8)
    path = str(tmp_path / "batch.npz")
    a.save(path)
    a.run(4000, warps=8)
    b = E.ChainBatch(geo, occ, g["eci"], KB * 300.0, move, seed=1)
    b.load(path)
    b.run(4000, warps=8)
    torch.cuda.synchronize()
    for name in ("occ", "cf", "energy", "trial", "accum", "kT", "chain_key"):
        assert torch.equal(getattr(a, name), getattr(b, name)), name
    with pytest.raises(ValueError):
        E.ChainBatch(geo, occ[:2], g["eci"], kT[:2], move, seed=1).load(path)


def _check_swap_state(cb, occ0, oracle_mod=None):
    """Compositions conserved and the per-species site lists (trk / loc) equal to the occupation."""
    m = cb.geo.model
    occ = cb.occ.cpu().numpy()
    trk, loc = cb.trk.cpu().numpy(), cb.loc.cpu().numpy()
    start, count = cb.trk_start.cpu().numpy(), cb.trk_count.cpu().numpy()
    for c in range(cb.n_chains):
        assert np.array_equal(np.bincount(occ[c], minlength=m.n_sym), np.bincount(occ0[c], minlength=m.n_sym))
        for sp in range(m.n_sym):
            lst = trk[c, start[c, sp]:start[c, sp] + count[c, sp]]
            assert set(lst.tolist()) == set(np.nonzero(occ[c] == sp)[0].tolist())
            assert np.array_equal(loc[c, lst], np.arange(count[c, sp]))
    if oracle_mod is not None:
        orc = oracle_mod.Oracle(m)
        cf = cb.cf.cpu().numpy()
        for c in range(cb.n_chains):
            assert np.allclose(cf[c], orc.full_cf(occ[c]), rtol=1e-9, atol=1e-12)


def test_graph_capture_keeps_swap_state_consistent(torch_cuda, oracle_mod):
    """Capturing a runner's step runs one warm step and restores the state; both must be ordered on the
    runner's stream, or the restore lands in the middle of the (long) warm kernel and leaves site lists
    that disagree with the occupation."""
    from cemc_gb300 import engine as E
    from cemc_gb300.batch import BatchRunner, MultiBatchRunner
    from cemc_gb300.lattice import fcc_settings, seeded_ecis
    from cemc_gb300.tables import CEModel
    rng = np.random.default_rng(8)
    runners, occs = [], []
    for L in (12, 6):
        s = fcc_settings(L, 5, 3, 1, ["Al", "Mg", "Si"])
        eci = seeded_ecis(s.cset, 0)
        m = CEModel(s, list(eci))
        geo = E.Geometry(m)
        occ = rng.integers(0, 3, (3, m.n_sites)).astype(np.int8)
        occs.append(occ)
        runners.append(BatchRunner(geo, occ, m.eci_vector(eci), 800.0, E.MOVE_SWAP, seed=2, precision=E.PREC_F32,
                                   warps=16, cluster=1, sweeps_per_step=20, graph=True))
    r0 = runners[0]
    r0.capture()
    r0.step(2)
    r0.synchronize()
    _check_swap_state(r0.cb, occs[0], oracle_mod)
    multi = MultiBatchRunner(runners)
    multi.step(2)
    multi.synchronize()
    for r, occ in zip(runners, occs):
        _check_swap_state(r.cb, occ, oracle_mod)


def test_rocksalt_canonical_run_with_fixed_background_element(torch_cuda):
    """The reference's tests/test_sgc_mc.py:140-191: Li/V on one sublattice, O on the other (background),
    some V replaced by Li, Montecarlo with FixedElement("O"), a short fixed-mode runMC; O never moves."""
    from cemc_gb300.calculator import CE, SimpleAtoms
    from cemc_gb300.lattice import fcc_settings, seeded_ecis, with_background
    from cemc_gb300.mc_constraints import FixedElement
    from cemc_gb300.mcmc import Montecarlo
    s = with_background(fcc_settings(3, 3, 2, 1, ["Li", "V"]), "O")
    eci = seeded_ecis(s.base.cset, 0)
    atoms = SimpleAtoms(s.symbols_with_background(["V"] * s.base.n_sites))
    CE(atoms, s, eci=dict(eci))
    mc = Montecarlo(atoms, 800, seed=4)
    mc.add_constraint(FixedElement(element="O"))
    mc.insert_symbol("Li", [i for i, a in enumerate(atoms) if a.symbol == "V"][:5])
    mc.runMC(steps=100, equil=False, mode="fixed")
    syms = [a.symbol for a in atoms]
    assert all(syms[i] == "O" for i in s.background_indices)
    assert sum(1 for x in syms if x == "Li") == 5


def test_sgc_constraints_by_tag_and_fixed_element(torch_cuda):
    """SGC flips under ConstrainElementByTag (Si only placed on one sublattice, Mg nowhere) and
    FixedElement("Mg") (sites holding Mg never change): after runMC every site obeys both.  (FixedElement
    alone lets Mg in but never out, so without the tag constraint Mg would take over the cell.)"""
    from cemc_gb300.mc_constraints import ConstrainElementByTag, FixedElement
    from cemc_gb300.mcmc import CanNotFindLegalMoveError, SGCMonteCarlo
    atoms, calc, s, eci = _calc(recipe=(4, 3, 2, 0, ("Al", "Mg", "Si")), seed=6)
    for a in atoms:
        a.tag = a.index % 4
    before = [a.symbol for a in atoms]
    mc = SGCMonteCarlo(atoms, 1000.0, seed=12)
    mc.add_constraint(ConstrainElementByTag(atoms, [["Al", "Si"], ["Al"], ["Al"], ["Al"]]))
    mc.add_constraint(FixedElement(element="Mg"))
    mc.runMC(steps=4000, chem_potential={"c1_0": 0.0, "c1_1": 0.0}, equil=False)
    after = [a.symbol for a in atoms]
    assert sum(1 for b, x in zip(before, after) if b != x) > 0
    for i, (b, x) in enumerate(zip(before, after)):
        if b == "Mg":
            assert x == "Mg"
        if x != b:
            assert x == "Al" or (x == "Si" and i % 4 == 0)
    # no legal move at all: every species frozen
    mc2 = SGCMonteCarlo(atoms, 1000.0, seed=1)
    for sym in ("Al", "Mg", "Si"):
        mc2.add_constraint(FixedElement(element=sym))
    with pytest.raises(CanNotFindLegalMoveError):
        mc2._run_trials(10)


@pytest.mark.parametrize("sgc", [False, True])
def test_observers_called_at_their_interval(sgc, torch_cuda):
    """Observers run every `interval` trials with that trial's changes (montecarlo.py:1031-1036): the
    swap / flip tuples, no-op tuples after a rejection, and the atoms already showing the new symbols."""
    from cemc_gb300.mcmc import Montecarlo, SGCMonteCarlo
    atoms, calc, s, eci = _calc()
    mc = SGCMonteCarlo(atoms, 900.0, seed=3) if sgc else Montecarlo(atoms, 900.0, seed=3)
    calls = []

    class Obs:
        def __call__(self, changes):
            calls.append((mc.current_step, list(changes), [atoms[c[0]].symbol for c in changes],
                          calc.get_energy()))

    mc.attach(Obs(), interval=250)
    if sgc:
        mc.runMC(steps=2000, chem_potential={"c1_0": 0.02}, equil=False)
    else:
        mc.runMC(steps=2000, equil=False)
    assert len(calls) == 12  # 4 during the 1000-trial bias probe, 8 in the main loop
    n_changed = 0
    for step, changes, now, energy in calls:
        assert step % 250 == 0 and len(changes) == (1 if sgc else 2)
        for (site, old, new), cur in zip(changes, now):
            assert cur == new
            n_changed += old != new
        if not sgc:
            (a, sa, sb), (b, sb2, sa2) = changes
            assert (sa, sb) == (sa2, sb2) or (sa == sb and sa2 == sb2)
    assert n_changed > 0


def test_accept_first_trial_move_after_reset(torch_cuda):
    """montecarlo.py:128-131, 363-364, 932-935: after construction and after every reset the next trial is
    accepted whatever its energy change."""
    from cemc_gb300.mcmc import Montecarlo
    atoms, calc, s, eci = _calc()
    mc = Montecarlo(atoms, 1.0, seed=2, accept_first_trial_move_after_reset=True)
    for _ in range(3):
        e0 = mc.current_energy
        _, accepted = mc._mc_step()
        assert accepted
        mc.reset()
    mc2 = Montecarlo(atoms, 1.0, seed=2)
    assert sum(mc2._mc_step()[1] for _ in range(5)) <= 5


@pytest.mark.parametrize("sgc", [False, True])
def test_drivers_with_waste_recycling(sgc, torch_cuda):
    """recycle_waste=True (montecarlo.py:50-68, 937-948): the runs complete and their averages are finite."""
    from cemc_gb300.mcmc import Montecarlo, SGCMonteCarlo
    atoms, calc, s, eci = _calc()
    if sgc:
        mc = SGCMonteCarlo(atoms, 900.0, seed=4, recycle_waste=True)
        mc.runMC(steps=3000, chem_potential={"c1_0": 0.01}, equil=False)
        q = mc.get_thermodynamic()
        assert np.isfinite(q["singlet_c1_0"]) and -1.0 <= q["singlet_c1_0"] <= 1.0
    else:
        mc = Montecarlo(atoms, 900.0, seed=4, recycle_waste=True)
        mc.runMC(steps=3000, equil=False)
        q = mc.get_thermodynamic()
    assert np.isfinite(q["energy"]) and q["heat_capacity" if not sgc else "sgc_heat_capacity"] >= 0.0
