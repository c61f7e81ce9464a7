"""Every benchmark workload at its own size, in the launch shape the benchmark times, against the oracle.

The small-cell fixture tests pin the kernels to the reference; these tests pin
the configurations that are measured: the same supercells, cluster sets,
chain counts, temperatures, seeds, chain keys, kernel forms, warps per CTA,
CTAs per chain, conflict tables and CUDA-graph capture as ``bench.py``.

  * 64 SGC chains x 16384 sites (FP32 energy changes, half-warp spin form, the
    autotuned shape, graph-captured steps) -- the headline;
  * one canonical FP64 chain of 2048 sites with the library's default shape;
  * one 131072-site replica of the tempering ladder (table form, the CTA-pair
    and device-memory conflict-table choices the library makes for it);
  * ternary chains of 4^3 and 24^3 cells stepped together by one multi-size
    graph (table form).

Bar: FP64 decisions and occupations bit-exact, correlation functions and
energies within 1e-9 relative; FP32 energy-change runs, decisions bit-exact
outside the near-threshold band |dE/kT + ln u| < 1e-5 eV / kT (and then the
occupations equal and the energies within 1e-9 after the FP64 recompute), the
per-trial energy change within 1e-5 eV.
"""
import os
import sys

import numpy as np
import pytest

from conftest import KB, ROOT

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-9
FP32_DE_TOL = 1e-5  # eV


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


def _check_fp32(acc_gpu, de_gpu, tr, kT):
    """FP32 decisions against the oracle's FP64 ones; True when every decision agrees."""
    margin = np.abs(tr.de / kT + np.log(np.maximum(tr.u, 1e-300)))
    mism = acc_gpu != tr.acc
    assert not np.any(mism & (margin >= FP32_DE_TOL / kT)), "decision differs outside the FP32 band"
    if np.any(mism):
        return False
    assert np.max(np.abs(de_gpu - tr.de)) < FP32_DE_TOL
    return True


def _bench():
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    import bench
    return bench


def test_gpu_headline_sgc64_matches_oracle(E, oracle_mod):
    """The headline batch (64 chains x 16384 sites): one graph-captured step of one sweep in the
    benchmark's own runner and shape, then a traced sweep of every chain in that shape."""
    import torch
    bench = _bench()
    from cemc_gb300.batch import BatchRunner
    s, m, occ, ev, Ts = bench.workload(0)
    geo = E.Geometry(m)
    keys = np.arange(bench.N_CHAINS)
    runner = BatchRunner(geo, occ, ev, Ts, E.MOVE_FLIP, seed=2026, precision=E.PREC_F32, warps=0, cluster=0,
                         sweeps_per_step=1, recompute_every=1, graph=True, chain_keys=keys)
    runner.capture()
    runner.step()
    runner.synchronize()
    runner.cb.check_status()
    assert runner.cb.last_kernel in (E.KERNEL_SPIN_QUARTER, E.KERNEL_SPIN_HALFWARP, E.KERNEL_SPIN, E.KERNEL_FIELD)
    orc = oracle_mod.Oracle(m)
    n = m.n_sites
    occ_gpu = runner.cb.occ.cpu().numpy()
    cf_gpu = runner.cb.cf.cpu().numpy()
    en_gpu = runner.cb.energy.cpu().numpy()
    for c in (0, 27, 63):  # coldest / lowest mu, a middle chain, hottest / highest mu
        kT = KB * Ts[c]
        st = orc.new_chain_state(occ[c], ev[c], kT, oracle_mod.MOVE_FLIP)
        tr = orc.run(st, seed=2026, chain_id=int(keys[c]), t_begin=0, n_trials=n, trace=True)
        margin = np.abs(tr.de / kT + np.log(np.maximum(tr.u, 1e-300)))
        if np.any(margin < FP32_DE_TOL / kT):
            continue  # a near-threshold trial may legitimately differ; the traced sweep below checks it
        assert np.array_equal(occ_gpu[c], st.occ), c
        assert np.allclose(cf_gpu[c], st.cf, rtol=FP64_RTOL, atol=1e-14), c
        assert _rel(en_gpu[c], st.energy[0]) < FP64_RTOL, c

    # traced sweep of all 64 chains from the same start, same warps / CTAs per chain / form as the runner
    cb = E.ChainBatch(geo, occ, ev, KB * Ts, E.MOVE_FLIP, seed=2026, chain_keys=keys)
    _, acc, de = cb.run(n, precision=E.PREC_F32, warps=runner.warps, cluster=runner.cluster, kernel=runner.kernel,
                        trace=True)
    cb.recompute()
    _sync()
    assert cb.last_kernel == runner.cb.last_kernel
    acc, de = acc.cpu().numpy(), de.cpu().numpy()
    occ_t, cf_t = cb.occ.cpu().numpy(), cb.cf.cpu().numpy()
    agreed = 0
    for c in range(bench.N_CHAINS):
        kT = KB * Ts[c]
        st = orc.new_chain_state(occ[c], ev[c], kT, oracle_mod.MOVE_FLIP)
        tr = orc.run(st, seed=2026, chain_id=int(keys[c]), t_begin=0, n_trials=n, trace=True)
        if _check_fp32(acc[c], de[c], tr, kT):
            agreed += 1
            assert np.array_equal(occ_t[c], st.occ), c
            assert np.allclose(cf_t[c], st.cf, rtol=FP64_RTOL, atol=1e-14), c
    assert agreed >= bench.N_CHAINS - 2  # near-threshold trials are rare (none expected at 1e-5 eV)


def test_gpu_canonical_single_chain_fp64_bit_exact(E, oracle_mod):
    """One FP64 canonical chain of 2048 sites (binary FCC 8^3, the headline cluster set), the library's
    default launch shape, 2048 x 20 swaps: decisions, occupations and correlation functions exact."""
    bench = _bench()
    from cemc_gb300.lattice import fcc_settings, seeded_ecis
    from cemc_gb300.tables import CEModel
    s = fcc_settings(8, *bench.SHELLS, bench.SPECIES)
    eci = seeded_ecis(s.cset, 0)
    m = CEModel(s, list(eci))
    geo = E.Geometry(m)
    rng = np.random.default_rng(0)
    occ = np.zeros(m.n_sites, dtype=np.int8)
    occ[rng.permutation(m.n_sites)[: m.n_sites // 2]] = 1
    ev = m.eci_vector(eci)
    kT = KB * 800.0
    cb = E.ChainBatch(geo, occ[None], ev, kT, E.MOVE_SWAP, seed=0)
    n = m.n_sites * 20
    sites, acc, de = cb.run(n, precision=E.PREC_F64, warps=0, trace=True)
    _sync()
    cb.check_status()
    orc = oracle_mod.Oracle(m)
    st = orc.new_chain_state(occ, ev, kT, oracle_mod.MOVE_SWAP)
    tr = orc.run(st, seed=0, chain_id=0, t_begin=0, n_trials=n, trace=True)
    assert np.array_equal(sites.cpu().numpy()[0].reshape(-1), tr.site)
    assert np.array_equal(acc.cpu().numpy()[0], tr.acc)
    assert np.array_equal(cb.occ.cpu().numpy()[0], st.occ)
    assert np.allclose(cb.cf.cpu().numpy()[0], st.cf, rtol=FP64_RTOL, atol=1e-14)
    assert _rel(cb.energy.cpu().numpy()[0], st.energy[0]) < FP64_RTOL
    assert np.max(np.abs(de.cpu().numpy()[0] - tr.de)) < 1e-9


def test_gpu_tempering_replica_131072_sites(E, oracle_mod):
    """Replicas of the tempering ladder's cell (binary FCC 32^3 = 131072 sites, pairs to the 6th shell):
    one sweep of swaps in FP32 with the shape the ladder runs (table form, the library's choice of CTAs
    per chain, exact conflict tables in device memory), each replica against the oracle."""
    bench = _bench()
    from cemc_gb300.lattice import fcc_settings, seeded_ecis
    from cemc_gb300.tables import CEModel
    s = fcc_settings(32, 6, 2, 1, bench.SPECIES)
    eci = seeded_ecis(s.cset, 0)
    m = CEModel(s, list(eci))
    geo = E.Geometry(m)
    rng = np.random.default_rng(0)
    occ = np.zeros(m.n_sites, dtype=np.int8)
    occ[rng.permutation(m.n_sites)[: m.n_sites // 2]] = 1
    Ts = np.array([200.0, 1500.0])
    ev = m.eci_vector(eci)
    cb = E.ChainBatch(geo, np.repeat(occ[None], 2, 0), ev, KB * Ts, E.MOVE_SWAP, seed=11)
    assert cb._stamps() is not None  # exact conflict tables in device memory
    n = m.n_sites
    _, acc, de = cb.run(n, precision=E.PREC_F32, warps=0, trace=True)
    _sync()
    cb.check_status()
    assert cb.last_kernel == E.KERNEL_TABLE
    orc = oracle_mod.Oracle(m)
    acc, de = acc.cpu().numpy(), de.cpu().numpy()
    for c in range(2):
        st = orc.new_chain_state(occ, ev, KB * Ts[c], oracle_mod.MOVE_SWAP)
        tr = orc.run(st, seed=11, chain_id=c, t_begin=0, n_trials=n, trace=True)
        if _check_fp32(acc[c], de[c], tr, KB * Ts[c]):
            assert np.array_equal(cb.occ.cpu().numpy()[c], st.occ), c
            assert np.allclose(cb.cf.cpu().numpy()[c], st.cf, rtol=FP64_RTOL, atol=1e-14), c


def test_gpu_ternary_uneven_graph_matches_oracle(E, oracle_mod):
    """Ternary canonical chains of a 4^3 and a 24^3 cell (256 and 55296 sites; pairs to the 5th shell,
    triplets to the 3rd, the tetrahedron), Dirichlet compositions, stepped together by one CUDA graph
    with one stream per size, in the benchmark's launch shapes (the large cell on a CTA pair) and
    launch order; every chain against the oracle."""
    from cemc_gb300.batch import BatchRunner, MultiBatchRunner
    from cemc_gb300.lattice import fcc_settings, seeded_ecis
    from cemc_gb300.tables import CEModel
    rng = np.random.default_rng(1000)
    runners, cases = [], []
    for L, n_chains in ((4, 2), (24, 1)):
        s = fcc_settings(L, 5, 3, 1, ["Al", "Mg", "Si"])
        eci = seeded_ecis(s.cset, 0)
        m = CEModel(s, list(eci))
        geo = E.Geometry(m)
        occ = np.zeros((n_chains, m.n_sites), dtype=np.int8)
        for c in range(n_chains):
            comp = rng.dirichlet([2.0, 2.0, 2.0])
            counts = np.floor(comp * m.n_sites).astype(int)
            counts[0] += m.n_sites - counts.sum()
            occ[c] = rng.permutation(np.repeat(np.arange(3), counts))
        keys = np.arange(n_chains) + 1000 * L
        warps, cluster = _bench().ternary_shape(m)
        runners.append(BatchRunner(geo, occ, m.eci_vector(eci), 800.0, E.MOVE_SWAP, seed=7 + L,
                                   precision=E.PREC_F32, warps=warps, cluster=cluster, sweeps_per_step=1,
                                   recompute_every=1, graph=True, chain_keys=keys))
        cases.append((m, occ, m.eci_vector(eci), keys, 7 + L))
    multi = MultiBatchRunner(runners)
    multi.capture()
    multi.step()
    multi.synchronize()
    for r, (m, occ, ev, keys, seed) in zip(runners, cases):
        r.cb.check_status()
        assert r.cb.last_kernel == E.KERNEL_TABLE
        orc = oracle_mod.Oracle(m)
        kT = KB * 800.0
        for c in range(len(keys)):
            st = orc.new_chain_state(occ[c], ev, kT, oracle_mod.MOVE_SWAP)
            tr = orc.run(st, seed=seed, chain_id=int(keys[c]), t_begin=0, n_trials=m.n_sites, trace=True)
            margin = np.abs(tr.de / kT + np.log(np.maximum(tr.u, 1e-300)))
            if np.any(margin < FP32_DE_TOL / kT):
                continue
            assert np.array_equal(r.cb.occ.cpu().numpy()[c], st.occ), (m.n_sites, c)
            assert np.allclose(r.cb.cf.cpu().numpy()[c], st.cf, rtol=FP64_RTOL, atol=1e-14), (m.n_sites, c)
            assert _rel(r.cb.energy.cpu().numpy()[c], st.energy[0]) < FP64_RTOL
