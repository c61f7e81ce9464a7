"""GPU kernels against the reference (golden fixtures) and the CPU oracle.

Bar: bit-exact decisions and occupations; correlation functions and energies
within 1e-9 relative in FP64; in FP32-energy-change mode, decisions bit-exact
outside the near-threshold band |dE/kT + ln u| < FP32_BAND and energy-change
error at most 1e-5 eV.
"""
import math

import numpy as np
import pytest

from conftest import KB, golden_cases, golden_model, load_golden, settings_for

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-9
FP32_DE_TOL = 1e-5  # eV, per trial


@pytest.fixture(scope="module")
def E():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from cemc_gb300 import engine
    return engine


def _sync():
    import torch
    torch.cuda.synchronize()


def _rel(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))


def _cf_close(a, b, rtol=FP64_RTOL, atol=1e-14):
    return np.allclose(a, b, rtol=rtol, atol=atol)


def _run_shape(cb, n, E, **kw):
    """cb.run, skipping when an explicitly requested CTA pair does not fit in shared memory."""
    from cemc_gb300._lib import CemcError
    try:
        return cb.run(n, **kw)
    except CemcError as exc:
        if kw.get("cluster") == 2 and exc.code == 5:
            pytest.skip("CTA pair of this shape exceeds shared memory: %s" % exc)
        raise


def _kernel_ok(m, kernel, E, move=0, cluster=0):
    """The spin-basis kernels only take binary +1/-1 geometries of one translation group; the half-warp one
    only flips."""
    if kernel in (E.KERNEL_SPIN, E.KERNEL_SPIN_HALFWARP) and not (
            m.n_sym == 2 and sorted(m.bf[0].tolist()) == [-1.0, 1.0] and m.n_groups == 1):
        pytest.skip("spin-basis kernel needs a binary +1/-1 basis and one translation group")
    if kernel == E.KERNEL_SPIN_HALFWARP and move != 0:
        pytest.skip("the half-warp spin kernel runs flips")
    if kernel == E.KERNEL_TABLE and np.any(np.asarray(m.group_scale) != 1.0):
        pytest.skip("the table kernel needs translation groups of equal size")
    if kernel == E.KERNEL_SPIN_QUARTER:
        if not (m.n_sym == 2 and sorted(m.bf[0].tolist()) == [-1.0, 1.0] and m.n_groups == 1
                and int((np.asarray(m.eci_kind) == 2).sum()) <= 8):
            pytest.skip("the quarter-warp spin kernel needs a binary +1/-1 basis, one group, <= 8 cluster ECIs")
        if move != 0 or cluster == 2:
            pytest.skip("the quarter-warp spin kernel runs flips on one CTA per chain")
    if kernel == E.KERNEL_FIELD:
        if not (m.n_sym == 2 and sorted(m.bf[0].tolist()) == [-1.0, 1.0] and m.n_groups == 1
                and len(m.movable) == m.n_sites):
            pytest.skip("the local-field kernel needs a binary +1/-1 basis, one translation group, no background")
        if move != 0 or cluster == 2:
            pytest.skip("the local-field kernel runs flips on one CTA per chain")


KERNELS = [1, 2, 3, 4, 5, 6]  # generic, spin, spin half-warp, table, local field, spin quarter-warp
CLUSTERS = [1, 2]  # CTAs per chain


@pytest.mark.parametrize("cluster", CLUSTERS)
@pytest.mark.parametrize("kernel", KERNELS)
@pytest.mark.parametrize("warps", [1, 9, 16])
@pytest.mark.parametrize("case", golden_cases())
def test_gpu_replays_reference_fixture_fp64(case, warps, kernel, cluster, E):
    g = load_golden(case)
    s, m, eci = golden_model(g)
    _kernel_ok(m, kernel, E, int(g["move"]), cluster)
    geo = E.Geometry(m)
    move = int(g["move"])
    cb = E.ChainBatch(geo, g["occ0"][None], g["eci"], float(g["kT"]), move, seed=int(g["seed"]))
    assert _cf_close(cb.cf.cpu().numpy()[0], g["cf0"], atol=1e-15)
    n = int(g["n_trials"])
    sites, acc, de = _run_shape(cb, n, E, precision=E.PREC_F64, warps=warps, trace=True, kernel=kernel,
                                cluster=cluster)
    _sync()
    cb.check_status()
    assert np.array_equal(sites.cpu().numpy()[0], g["sites"])
    assert np.array_equal(acc.cpu().numpy()[0], g["ref_acc"])
    assert np.array_equal(cb.occ.cpu().numpy()[0], g["occ_final"])
    assert _cf_close(cb.cf.cpu().numpy()[0], g["cf_final"])
    assert _rel(cb.energy.cpu().numpy()[0], g["energy_final"]) < FP64_RTOL
    assert np.max(np.abs(de.cpu().numpy()[0] - g["ref_de"])) < 1e-9


@pytest.mark.parametrize("cluster", CLUSTERS)
@pytest.mark.parametrize("kernel", KERNELS)
@pytest.mark.parametrize("case", golden_cases())
def test_gpu_fp32_energy_change_against_reference_fixture(case, kernel, cluster, E):
    g = load_golden(case)
    s, m, eci = golden_model(g)
    _kernel_ok(m, kernel, E, int(g["move"]), cluster)
    geo = E.Geometry(m)
    cb = E.ChainBatch(geo, g["occ0"][None], g["eci"], float(g["kT"]), int(g["move"]), seed=int(g["seed"]))
    n = int(g["n_trials"])
    sites, acc, de = _run_shape(cb, n, E, precision=E.PREC_F32, warps=16, trace=True, kernel=kernel,
                                cluster=cluster)
    _sync()
    acc = acc.cpu().numpy()[0]
    de = de.cpu().numpy()[0]
    kT = float(g["kT"])
    margin = np.abs(g["ref_de"] / kT + np.log(np.maximum(g["u"], 1e-300)))
    band = FP32_DE_TOL / kT
    near = margin < band
    mism = acc != g["ref_acc"]
    assert not np.any(mism & ~near), "decision differs outside the FP32 band"
    if not np.any(mism):
        assert np.array_equal(cb.occ.cpu().numpy()[0], g["occ_final"])
        assert np.max(np.abs(de - g["ref_de"])) < FP32_DE_TOL
        assert _cf_close(cb.cf.cpu().numpy()[0], g["cf_final"], rtol=1e-6, atol=1e-7)


@pytest.mark.parametrize("case", golden_cases())
def test_gpu_calculator_kernels_match_reference_updates(case, E):
    """cemc_apply_changes reproduces the reference's update_cf known answers."""
    import torch
    g = load_golden(case)
    s, m, eci = golden_model(g)
    geo = E.Geometry(m)
    from cemc_gb300.calculator import DeviceUpdater
    up = DeviceUpdater(geo, g["occ0"], g["eci"], cf=g["cf0"])
    for i, site in enumerate(g["upd_sites"]):
        up.apply([(int(site), int(up.occupation()[site]), int(g["upd_new"][i]))])
        assert _cf_close(up.cf(), g["upd_cf"][i])
        assert _rel(up.energy(), g["upd_energy"][i]) < FP64_RTOL


def test_gpu_delta_e_matches_oracle(E, oracle_mod):
    g = load_golden("ternary_swap")
    s, m, eci = golden_model(g)
    geo = E.Geometry(m)
    orc = oracle_mod.Oracle(m)
    from cemc_gb300.calculator import DeviceUpdater
    up = DeviceUpdater(geo, g["occ0"], g["eci"], cf=g["cf0"])
    occ = g["occ0"].copy()
    rng = np.random.default_rng(1)
    e0 = orc.energy(g["eci"], g["cf0"])
    for _ in range(20):
        a, b = (int(x) for x in rng.choice(m.n_sites, 2, replace=False))
        if occ[a] == occ[b]:
            continue
        de, dcf = up.delta_swap(a, b)
        c1 = orc.update_cf(occ, a, occ[b], g["cf0"])
        o2 = occ.copy()
        o2[a] = occ[b]
        c2 = orc.update_cf(o2, b, occ[a], c1)
        assert abs(de - (orc.energy(g["eci"], c2) - e0)) < 1e-9
        assert np.allclose(dcf, c2 - g["cf0"], atol=1e-13)


@pytest.mark.parametrize("recipe", [(6, 4, 2, 1, ["Al", "Mg"], "fcc"), (4, 5, 3, 1, ["Al", "Mg", "Si"], "fcc"),
                                    (4, 4, 2, 1, ["Al", "Mg"], "l12"), (3, 3, 2, 0, ["Al", "Mg", "Si"], "l12"),
                                    (4, 4, 2, 1, ["Al", "Mg"], "l12:0111")])
def test_gpu_full_recompute_matches_oracle(recipe, E, oracle_mod):
    from cemc_gb300.lattice import seeded_ecis
    from cemc_gb300.tables import CEModel
    L, ps, ts, qs, syms, lattice = recipe
    s = settings_for(lattice, L, ps, ts, qs, syms)
    eci = seeded_ecis(s.cset, 2)
    m = CEModel(s, list(eci))
    orc = oracle_mod.Oracle(m)
    geo = E.Geometry(m)
    rng = np.random.default_rng(5)
    occ = rng.integers(0, len(syms), (5, m.n_sites)).astype(np.int8)
    cb = E.ChainBatch(geo, occ, m.eci_vector(eci), KB * 700, E.MOVE_FLIP)
    _sync()
    for c in range(5):
        full = orc.full_cf(occ[c])
        assert np.allclose(cb.cf.cpu().numpy()[c], full, rtol=1e-12, atol=1e-15)
        assert _rel(cb.energy.cpu().numpy()[c], orc.energy(m.eci_vector(eci), full)) < 1e-12


@pytest.mark.parametrize("cluster", CLUSTERS)
@pytest.mark.parametrize("kernel", KERNELS)
@pytest.mark.parametrize("move", [0, 1])
@pytest.mark.parametrize("prec", [0, 1])
def test_gpu_batch_equals_oracle_per_chain(move, prec, kernel, cluster, E, oracle_mod):
    """Many chains in one launch, each equal to the oracle run of that chain (keys, temperatures, mu differ)."""
    g = load_golden("binary_flip")
    s, m, eci = golden_model(g)
    _kernel_ok(m, kernel, E, move, cluster)
    geo = E.Geometry(m)
    orc = oracle_mod.Oracle(m)
    rng = np.random.default_rng(7)
    n_chains = 6
    occ = rng.integers(0, 2, (n_chains, m.n_sites)).astype(np.int8)
    Ts = np.linspace(300, 1500, n_chains)
    ev = np.repeat(g["eci"][None], n_chains, 0)
    ev[:, m.eci_names.index("c1_0")] += np.linspace(-0.1, 0.1, n_chains)
    keys = [11, 5, 7, 3, 13, 2]
    cb = E.ChainBatch(geo, occ, ev, KB * Ts, move, seed=99, chain_keys=keys)
    n = 2500
    _, acc, de = _run_shape(cb, n, E, precision=prec, warps=8, trace=True, kernel=kernel, cluster=cluster)
    _sync()
    acc = acc.cpu().numpy()
    de = de.cpu().numpy()
    for c in range(n_chains):
        st = orc.new_chain_state(occ[c], ev[c], KB * Ts[c], move)
        tr = orc.run(st, seed=99, chain_id=keys[c], t_begin=0, n_trials=n, trace=True)
        if prec == 0:
            assert np.array_equal(acc[c], tr.acc)
            assert np.array_equal(cb.occ.cpu().numpy()[c], st.occ)
            assert _cf_close(cb.cf.cpu().numpy()[c], st.cf)
        else:
            margin = np.abs(tr.de / (KB * Ts[c]) + np.log(np.maximum(tr.u, 1e-300)))
            mism = acc[c] != tr.acc
            assert not np.any(mism & (margin >= FP32_DE_TOL / (KB * Ts[c])))
            if not np.any(mism):
                assert np.max(np.abs(de[c] - tr.de)) < FP32_DE_TOL
                assert np.array_equal(cb.occ.cpu().numpy()[c], st.occ)


@pytest.mark.parametrize("kernel", KERNELS)
def test_gpu_launch_splitting_is_invisible(kernel, E):
    """k launches of n/k trials equal one launch of n (counter-based proposals, resident state),
    whatever the launch shape of each piece (warps, CTAs per chain, trials per warp)."""
    flips_only = kernel in (E.KERNEL_SPIN_HALFWARP, E.KERNEL_FIELD, E.KERNEL_SPIN_QUARTER)
    g = load_golden("binary_flip" if flips_only else "binary_swap")
    move = 0 if flips_only else 1
    s, m, eci = golden_model(g)
    geo = E.Geometry(m)
    a = E.ChainBatch(geo, g["occ0"][None], g["eci"], float(g["kT"]), move, seed=4)
    b = E.ChainBatch(geo, g["occ0"][None], g["eci"], float(g["kT"]), move, seed=4)
    a.run(3000, precision=0, warps=16, kernel=kernel, cluster=1)
    for i in range(3):
        if i == 1 and kernel in (E.KERNEL_FIELD, E.KERNEL_SPIN_QUARTER):  # another form on a CTA pair
            b.run(1000, precision=0, warps=7, kernel=E.KERNEL_SPIN_HALFWARP, cluster=2)
        elif i == 1:  # the middle piece on a CTA pair
            b.run(1000, precision=0, warps=7, kernel=kernel, cluster=2)
        else:
            b.run(1000, precision=0, warps=7, kernel=kernel, cluster=1)
    _sync()
    assert np.array_equal(a.occ.cpu().numpy(), b.occ.cpu().numpy())
    assert np.allclose(a.cf.cpu().numpy(), b.cf.cpu().numpy(), rtol=1e-12, atol=1e-15)
    ha, hb = a.accum_host(), b.accum_host()
    assert ha[0, E.A_NSAMP] == hb[0, E.A_NSAMP] == 3000
    assert ha[0, E.A_NACC] == hb[0, E.A_NACC]
    assert np.allclose(ha[0, :E.A_NSAMP], hb[0, :E.A_NSAMP], rtol=1e-10, atol=1e-12)


@pytest.mark.parametrize("cluster", CLUSTERS)
@pytest.mark.parametrize("kernel", KERNELS)
def test_gpu_accumulators_match_oracle(kernel, cluster, E, oracle_mod):
    g = load_golden("binary_flip")
    s, m, eci = golden_model(g)
    _kernel_ok(m, kernel, E, 0, cluster)
    geo = E.Geometry(m)
    orc = oracle_mod.Oracle(m)
    for prec in (0, 1):
        cb = E.ChainBatch(geo, g["occ0"][None], g["eci"], float(g["kT"]), 0, seed=int(g["seed"]))
        _run_shape(cb, 3000, E, precision=prec, warps=16, kernel=kernel, cluster=cluster)
        _sync()
        st = orc.new_chain_state(g["occ0"], g["eci"], float(g["kT"]), 0)
        orc.run(st, seed=int(g["seed"]), chain_id=0, t_begin=0, n_trials=3000)
        h = cb.accum_host()[0]
        o = st.acc[0]
        tol = 1e-9 if prec == 0 else 1e-5
        assert h[E.A_NSAMP] == o["n_samples"] and h[E.A_NACC] == o["n_accept"]
        n = o["n_samples"]
        assert abs(h[E.A_SUM_E] - o["sum_e"]) / n < tol
        assert abs(h[E.A_SUM_E2] - o["sum_e2"]) / n < tol * max(1.0, abs(o["sum_e2"] / n))
        assert abs(h[E.A_SUM_S] - o["sum_s"][0]) / n < tol
        assert abs(h[E.A_SUM_S2] - o["sum_s2"][0]) / n < tol
        assert abs(h[E.A_SUM_SE] - o["sum_se"][0]) / n < tol


def test_gpu_replica_exchange_matches_restatement(E):
    """cemc_pt_exchange against a Python restatement of parallel_tempering.py:138-175."""
    import torch
    from cemc_gb300.rng import pt_uniform
    n = 9
    rng = np.random.default_rng(3)
    energy = rng.normal(-100, 2, n)
    Ts = np.geomspace(200, 1500, n)
    for direction in (0, 1):
        for rnd in range(4):
            kT = KB * Ts.copy()
            rep = np.arange(n, dtype=np.int32)
            en_d = torch.tensor(energy, device="cuda")
            kT_d = torch.tensor(kT, device="cuda")
            rep_d = torch.tensor(rep, device="cuda")
            nacc = torch.zeros(1, dtype=torch.int32, device="cuda")
            from cemc_gb300.engine import pt_exchange
            pt_exchange(en_d, kT_d, rep_d, direction, seed=17, round_index=rnd, n_accept=nacc)
            _sync()
            pairs = [(i, i + 1) for i in range(0, n - 1, 2)] if direction == 0 else \
                    [(i, i - 1) for i in range(n - 1, 0, -2)]
            acc = 0
            for p, q in pairs:
                ci, cj = rep[p], rep[q]
                prob = math.exp((1 / kT[ci] - 1 / kT[cj]) * (energy[ci] - energy[cj]))
                u = pt_uniform(17, rnd, p)
                if u < prob:
                    kT[ci], kT[cj] = kT[cj], kT[ci]
                    rep[p], rep[q] = cj, ci
                    acc += 1
            assert np.array_equal(rep_d.cpu().numpy(), rep)
            assert np.array_equal(kT_d.cpu().numpy(), kT)
            assert int(nacc.item()) == acc


@pytest.mark.parametrize("case", ["l12_swap", "l12_merged_swap", "l12_ternary_swap"])
@pytest.mark.parametrize("kernel", [1, 4])
@pytest.mark.parametrize("move", [0, 1])
def test_gpu_multi_group_batch_equals_oracle(case, kernel, move, E, oracle_mod):
    """Several translation groups: chains with their own keys, temperatures and occupations, flips
    and swaps (within and across groups), each equal to the oracle's run of that chain."""
    g = load_golden(case)
    s, m, eci = golden_model(g)
    assert m.n_groups > 1
    _kernel_ok(m, kernel, E, move)
    geo = E.Geometry(m)
    orc = oracle_mod.Oracle(m)
    rng = np.random.default_rng(17)
    n_chains = 4
    occ = rng.integers(0, m.n_sym, (n_chains, m.n_sites)).astype(np.int8)
    Ts = np.linspace(400, 1600, n_chains)
    ev = np.repeat(g["eci"][None], n_chains, 0)
    keys = [3, 9, 4, 21]
    cb = E.ChainBatch(geo, occ, ev, KB * Ts, move, seed=5, chain_keys=keys)
    n = 2000
    _, acc, de = cb.run(n, precision=E.PREC_F64, warps=12, trace=True, kernel=kernel)
    _sync()
    cb.check_status()
    assert cb.last_kernel == kernel
    acc = acc.cpu().numpy()
    de = de.cpu().numpy()
    for c in range(n_chains):
        st = orc.new_chain_state(occ[c], ev[c], KB * Ts[c], move)
        tr = orc.run(st, seed=5, chain_id=keys[c], t_begin=0, n_trials=n, trace=True)
        assert np.array_equal(acc[c], tr.acc)
        assert np.max(np.abs(de[c] - tr.de)) < 1e-9
        assert np.array_equal(cb.occ.cpu().numpy()[c], st.occ)
        assert _cf_close(cb.cf.cpu().numpy()[c], st.cf)


def test_gpu_multi_group_kernel_selection(E):
    """Four equal groups run the table form by default; unequal groups the generic form, and neither
    takes the spin form."""
    from cemc_gb300._lib import CemcError
    for case, auto_kernel in (("l12_swap", E.KERNEL_TABLE), ("l12_merged_swap", E.KERNEL_GENERIC)):
        g = load_golden(case)
        s, m, eci = golden_model(g)
        geo = E.Geometry(m)
        cb = E.ChainBatch(geo, g["occ0"][None], g["eci"], float(g["kT"]), 1, seed=1)
        cb.run(100)
        _sync()
        assert cb.last_kernel == auto_kernel
        with pytest.raises(CemcError) as ei:
            cb.run(10, kernel=E.KERNEL_SPIN)
        assert ei.value.code == 1
        if auto_kernel == E.KERNEL_GENERIC:
            with pytest.raises(CemcError) as ei:
                cb.run(10, kernel=E.KERNEL_TABLE)
            assert ei.value.code == 5


def test_gpu_multi_group_delta_e_matches_oracle(E, oracle_mod):
    """The calculator's energy change of swaps between sites of different translation groups."""
    g = load_golden("l12_ternary_swap")
    s, m, eci = golden_model(g)
    geo = E.Geometry(m)
    orc = oracle_mod.Oracle(m)
    from cemc_gb300.calculator import DeviceUpdater
    up = DeviceUpdater(geo, g["occ0"], g["eci"], cf=g["cf0"])
    occ = g["occ0"].copy()
    rng = np.random.default_rng(3)
    e0 = orc.energy(g["eci"], g["cf0"])
    n_cross = 0
    for _ in range(40):
        a, b = (int(x) for x in rng.choice(m.n_sites, 2, replace=False))
        if occ[a] == occ[b]:
            continue
        n_cross += int(m.site_group[a] != m.site_group[b])
        de, dcf = up.delta_swap(a, b)
        c1 = orc.update_cf(occ, a, occ[b], g["cf0"])
        o2 = occ.copy()
        o2[a] = occ[b]
        c2 = orc.update_cf(o2, b, occ[a], c1)
        assert abs(de - (orc.energy(g["eci"], c2) - e0)) < 1e-9
        assert np.allclose(dcf, c2 - g["cf0"], atol=1e-13)
    assert n_cross > 5


def test_gpu_spin_kernel_rejects_ternary(E):
    g = load_golden("ternary_flip")
    s, m, eci = golden_model(g)
    geo = E.Geometry(m)
    cb = E.ChainBatch(geo, g["occ0"][None], g["eci"], float(g["kT"]), 0, seed=1)
    from cemc_gb300._lib import CemcError
    with pytest.raises(CemcError):
        cb.run(10, kernel=E.KERNEL_SPIN)


@pytest.mark.parametrize("move", [0, 1])
def test_gpu_global_stamp_tables_match_oracle(move, E, oracle_mod, monkeypatch):
    """55296 sites: the exact conflict table only fits in device memory; with it (exact) and
    without it (hashed shared-memory table) the chain equals the oracle's."""
    from cemc_gb300.lattice import fcc_settings, seeded_ecis
    from cemc_gb300.tables import CEModel
    s = fcc_settings(24, 4, 2, 1, ["Al", "Mg"])
    eci = seeded_ecis(s.cset, 3)
    m = CEModel(s, list(eci))
    geo = E.Geometry(m)
    orc = oracle_mod.Oracle(m)
    rng = np.random.default_rng(5)
    occ = rng.integers(0, 2, m.n_sites).astype(np.int8)
    ev = m.eci_vector(eci)
    kT = KB * 900.0
    n = 20000
    st = orc.new_chain_state(occ, ev, kT, move)
    tr = orc.run(st, seed=31, chain_id=0, t_begin=0, n_trials=n, trace=True)
    for global_tables in (True, False):
        monkeypatch.setattr(E, "STAMP_GLOBAL_SITES", 0 if global_tables else 1 << 30)
        cb = E.ChainBatch(geo, occ[None], ev, kT, move, seed=31)
        _, acc, _ = cb.run(n, precision=E.PREC_F64, warps=16, trace=True, cluster=1)
        _sync()
        cb.check_status()
        assert (cb._stamp_buf is not None) == global_tables
        assert np.array_equal(acc.cpu().numpy()[0], tr.acc)
        assert np.array_equal(cb.occ.cpu().numpy()[0], st.occ)
        assert _cf_close(cb.cf.cpu().numpy()[0], st.cf)


def _constraint_masks(m, n_chains, rng):
    """Per-chain constraints: fixed sites; no species 1 on one sublattice; (ternary) species 0 frozen and
    never placed; the last chain unconstrained."""
    full = (1 << m.n_sym) - 1
    allow = np.full((n_chains, m.n_sites), full, dtype=np.uint8)
    frozen = np.zeros(n_chains, dtype=np.int32)
    allow[0, rng.choice(m.n_sites, m.n_sites // 5, replace=False)] = 0
    allow[1, np.arange(m.n_sites) % 4 == 0] &= np.uint8(full & ~0b10)
    if m.n_sym > 2:
        frozen[1] = 0b1
        allow[1] &= np.uint8(full & ~0b1)
    return allow, frozen


@pytest.mark.parametrize("kernel", [1, 2, 4])
@pytest.mark.parametrize("move", [0, 1])
@pytest.mark.parametrize("case", ["binary_flip", "ternary_swap"])
def test_gpu_constrained_runs_match_oracle(case, move, kernel, E, oracle_mod):
    """Move constraints (redraw loop of montecarlo.py:976-988 on per-site masks): every chain's
    proposals, decisions, occupation and correlation functions equal the oracle's."""
    import torch
    g = load_golden(case)
    s, m, eci = golden_model(g)
    _kernel_ok(m, kernel, E, move)
    geo = E.Geometry(m)
    rng = np.random.default_rng(11)
    n_chains = 3
    occ = rng.integers(0, m.n_sym, (n_chains, m.n_sites)).astype(np.int8)
    allow, frozen = _constraint_masks(m, n_chains, rng)
    Ts = np.array([600.0, 900.0, 1200.0])
    keys = [5, 8, 2]
    cb = E.ChainBatch(geo, occ, g["eci"], KB * Ts, move, seed=41, chain_keys=keys)
    n = 2000
    sites, acc, de = cb.run(n, precision=E.PREC_F64, warps=8, trace=True, kernel=kernel,
                            site_allow=torch.as_tensor(allow).cuda(), frozen=torch.as_tensor(frozen).cuda(),
                            max_attempts=300)
    _sync()
    cb.check_status()
    assert cb.last_kernel == kernel
    sites, acc = sites.cpu().numpy(), acc.cpu().numpy()
    for c in range(n_chains):
        st = orc_state = oracle_mod.Oracle(m).new_chain_state(
            occ[c], g["eci"], KB * Ts[c], move, allow=None if c == 2 else allow[c], frozen=int(frozen[c]),
            max_attempts=300)
        tr = oracle_mod.Oracle(m).run(orc_state, seed=41, chain_id=keys[c], t_begin=0, n_trials=n, trace=True)
        assert np.array_equal(sites[c].reshape(-1), tr.site), c
        assert np.array_equal(acc[c], tr.acc), c
        assert np.array_equal(cb.occ.cpu().numpy()[c], st.occ), c
        assert _cf_close(cb.cf.cpu().numpy()[c], st.cf), c
        changed = st.occ != occ[c]
        assert not np.any(changed & (allow[c] == 0))


@pytest.mark.parametrize("kernel", [1, 4])
def test_gpu_constraints_without_legal_move_report_status(kernel, E, oracle_mod):
    """A binary canonical chain with one species frozen has no legal swap: every trial is rejected after
    max_attempts redraws, the chain is untouched and its status is CEMC_ERR_NO_MOVE."""
    import torch
    from cemc_gb300._lib import CemcError, ERR_NO_MOVE
    g = load_golden("binary_swap")
    s, m, eci = golden_model(g)
    geo = E.Geometry(m)
    occ = g["occ0"][None]
    cb = E.ChainBatch(geo, occ, g["eci"], float(g["kT"]), 1, seed=3)
    cf0 = cb.cf.clone()
    _, acc, _ = cb.run(50, precision=E.PREC_F64, warps=4, trace=True, kernel=kernel,
                       frozen=torch.tensor([0b01], dtype=torch.int32, device="cuda"), max_attempts=7)
    _sync()
    with pytest.raises(CemcError) as ei:
        cb.check_status()
    assert ei.value.code == ERR_NO_MOVE
    assert not acc.cpu().numpy().any()
    assert np.array_equal(cb.occ.cpu().numpy(), occ)
    assert torch.equal(cb.cf, cf0)
    st = oracle_mod.Oracle(m).new_chain_state(occ[0], g["eci"], float(g["kT"]), 1, frozen=0b01, max_attempts=7)
    with pytest.raises(oracle_mod.NoLegalMove):
        oracle_mod.Oracle(m).run(st, seed=3, chain_id=0, t_begin=0, n_trials=50)


@pytest.mark.parametrize("kernel", [1, 2, 4])
@pytest.mark.parametrize("move", [0, 1])
def test_gpu_accept_first_matches_oracle(move, kernel, E, oracle_mod):
    """The call's first trial is accepted outright on every chain (accept_first_trial_move_after_reset),
    at a temperature where it would be rejected; the chains then equal the oracle's."""
    g = load_golden("binary_flip")
    s, m, eci = golden_model(g)
    _kernel_ok(m, kernel, E, move)
    geo = E.Geometry(m)
    rng = np.random.default_rng(21)
    occ = rng.integers(0, 2, (3, m.n_sites)).astype(np.int8)
    keys = [1, 4, 9]
    cb = E.ChainBatch(geo, occ, g["eci"], KB * 20.0, move, seed=6, chain_keys=keys)
    _, acc, _ = cb.run(400, precision=E.PREC_F64, warps=8, trace=True, kernel=kernel, accept_first=True)
    _sync()
    acc = acc.cpu().numpy()
    for c in range(3):
        st = oracle_mod.Oracle(m).new_chain_state(occ[c], g["eci"], KB * 20.0, move, accept_first=1)
        tr = oracle_mod.Oracle(m).run(st, seed=6, chain_id=keys[c], t_begin=0, n_trials=400, trace=True)
        assert acc[c, 0] == 1 and np.array_equal(acc[c], tr.acc)
        assert np.array_equal(cb.occ.cpu().numpy()[c], st.occ)
        assert _cf_close(cb.cf.cpu().numpy()[c], st.cf)


@pytest.mark.parametrize("move", [0, 1])
@pytest.mark.parametrize("prec", [0, 1])
def test_gpu_waste_recycling_matches_oracle(prec, move, E, oracle_mod):
    """Waste recycling (generic form, one CTA): decisions u > 1 / (1 + exp(-dE / kT)) and the weighted
    running sums equal the oracle's (FP64 bit-exact decisions, sums to 1e-9; FP32 decisions outside the
    near-threshold band, sums to 1e-5)."""
    g = load_golden("ternary_swap")
    s, m, eci = golden_model(g)
    geo = E.Geometry(m)
    orc = oracle_mod.Oracle(m)
    rng = np.random.default_rng(12)
    occ = rng.integers(0, m.n_sym, (2, m.n_sites)).astype(np.int8)
    keys = [3, 8]
    kT = KB * np.array([600.0, 1100.0])
    cb = E.ChainBatch(geo, occ, g["eci"], kT, move, seed=17, chain_keys=keys)
    n = 2500
    _, acc, de = cb.run(n, precision=prec, warps=12, trace=True, recycle_waste=True)
    _sync()
    cb.check_status()
    assert cb.last_kernel == E.KERNEL_GENERIC
    acc, de = acc.cpu().numpy(), de.cpu().numpy()
    h = cb.accum_host()
    for c in range(2):
        st = orc.new_chain_state(occ[c], g["eci"], kT[c], move, recycle=1)
        tr = orc.run(st, seed=17, chain_id=keys[c], t_begin=0, n_trials=n, trace=True)
        if prec == 1:
            x = tr.de / kT[c]
            p0 = 1.0 / (1.0 + np.exp(-x))
            near = np.abs(tr.u - p0) < 1e-5 * np.maximum(p0 * (1 - p0), 1e-300) / kT[c] + 1e-12
            assert not np.any((acc[c] != tr.acc) & ~near)
            if np.any(acc[c] != tr.acc):
                continue
        assert np.array_equal(acc[c], tr.acc)
        assert np.array_equal(cb.occ.cpu().numpy()[c], st.occ)
        o = st.acc[0]
        nn = o["n_samples"]
        tol = 1e-9 if prec == 0 else 1e-5
        assert h[c, E.A_NSAMP] == nn and h[c, E.A_NACC] == o["n_accept"]
        assert abs(h[c, E.A_SUM_E] - o["sum_e"]) / nn < tol * max(1.0, abs(o["sum_e"] / nn))
        assert abs(h[c, E.A_SUM_E2] - o["sum_e2"]) / nn < tol * max(1.0, abs(o["sum_e2"] / nn))
        for b in range(m.n_bf):
            assert abs(h[c, E.A_SUM_S + b] - o["sum_s"][b]) / nn < tol
            assert abs(h[c, E.A_SUM_S2 + b] - o["sum_s2"][b]) / nn < tol
            assert abs(h[c, E.A_SUM_SE + b] - o["sum_se"][b]) / nn < tol * max(1.0, abs(o["sum_se"][b] / nn))


def test_gpu_table_form_scratch_rules(E):
    """cemc_run's table form ends with a full recompute: with no scratch buffer it uses the library's fixed
    array and gives the same chains as with a caller buffer; a caller buffer that is too small is refused
    (CEMC_ERR_ARG) before anything is launched."""
    import torch
    from cemc_gb300._lib import CemcError, ERR_ARG
    g = load_golden("ternary_swap")
    s, m, eci = golden_model(g)
    geo = E.Geometry(m)
    rng = np.random.default_rng(31)
    occ = rng.integers(0, m.n_sym, (3, m.n_sites)).astype(np.int8)
    a = E.ChainBatch(geo, occ, g["eci"], KB * 900.0, 1, seed=12)
    b = E.ChainBatch(geo, occ, g["eci"], KB * 900.0, 1, seed=12)
    a.run(3000, precision=E.PREC_F32, warps=8, kernel=E.KERNEL_TABLE)
    b.scratch = None  # the fixed array
    b.run(3000, precision=E.PREC_F32, warps=8, kernel=E.KERNEL_TABLE)
    _sync()
    assert a.last_kernel == b.last_kernel == E.KERNEL_TABLE
    assert torch.equal(a.occ, b.occ)
    assert torch.equal(a.cf, b.cf) and torch.equal(a.energy, b.energy)
    c = E.ChainBatch(geo, occ, g["eci"], KB * 900.0, 1, seed=12)
    occ_before = c.occ.clone()
    c.scratch = torch.empty(1, dtype=torch.float64, device="cuda")
    with pytest.raises(CemcError) as ei:
        c.run(3000, precision=E.PREC_F32, warps=8, kernel=E.KERNEL_TABLE)
    assert ei.value.code == ERR_ARG
    _sync()
    assert torch.equal(c.occ, occ_before)
