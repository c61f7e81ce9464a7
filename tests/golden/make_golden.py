"""Generate the golden fixtures of the hot path from the reference's own CEUpdater.

Run in a checkout where the reference has been compiled by
``oracle/build_ref.sh`` (it needs the reference sources).  For each case it

1. builds an FCC supercell and cluster set with ``cemc_gb300.lattice``;
2. draws a random occupation and computes its correlation functions with the
   oracle's full recompute (the reference has no full recompute of its own;
   its tests compare against CLEASE's, which is unavailable);
3. lets the oracle propose ``n_trials`` moves and uniforms from the shared
   counter-based stream (seed, chain 0), and replays exactly those moves and
   uniforms through the reference's ``PyCEUpdater.calculate`` /
   ``clear_history`` / ``undo_changes`` with the reference's Metropolis rule
   (cemc/mcmc/montecarlo.py:950-956, 1014-1017);
4. records the reference's decisions, energy changes, final occupation,
   correlation functions and energy, plus the reference's correlation
   functions after each of a few explicit single-site updates.

The fixtures then pin the oracle (CPU tests) and the GPU path (GPU tests) to
the reference on machines without the reference tree.

    CEMC_REFERENCE=<reference tree> python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from cemc_gb300.lattice import (cubic_settings, fcc_settings, hcp_settings, l12_settings, seeded_ecis,  # noqa: E402
                                with_background)
from cemc_gb300.tables import CEModel  # noqa: E402

KB = 8.6173303e-5  # eV/K, the constant of cpp/src/linear_vib_correction.cpp:3

# name, L, pair shells, triplet shells, quad shells, species, move (0 flip, 1 swap), T, trials, seed,
# background symbol (None: every site active; else an inert second sublattice of that species,
# rocksalt-like, as in the reference's tests/test_sgc_mc.py:140-191), lattice ("fcc": one
# translation-symmetry group; "l12": FCC under L1_2 symmetry, four groups, like the four-group
# crystal of the reference's tests/helper_functions.py:8-27; "bcc", "sc": other cubic lattices;
# "hcp:<Lz>": L x L x Lz hexagonal close-packed cells)
CASES = [
    ("binary_flip", 4, 4, 2, 1, ["Al", "Mg"], 0, 800.0, 3000, 11, None),
    ("binary_swap", 4, 4, 2, 1, ["Al", "Mg"], 1, 800.0, 3000, 12, None),
    ("binary_swap_cold", 4, 4, 2, 1, ["Al", "Mg"], 1, 150.0, 3000, 13, None),
    ("ternary_flip", 4, 5, 3, 1, ["Al", "Mg", "Si"], 0, 800.0, 1500, 14, None),
    ("ternary_swap", 4, 5, 3, 1, ["Al", "Mg", "Si"], 1, 800.0, 1500, 15, None),
    ("rocksalt_flip", 4, 4, 2, 1, ["Li", "V"], 0, 800.0, 3000, 16, "O"),
    ("rocksalt_swap", 4, 4, 2, 1, ["Li", "V"], 1, 800.0, 3000, 17, "O"),
    ("l12_flip", 4, 4, 2, 1, ["Al", "Mg"], 0, 800.0, 3000, 18, None, "l12"),
    ("l12_swap", 4, 4, 2, 1, ["Al", "Mg"], 1, 800.0, 3000, 19, None, "l12"),
    ("l12_ternary_swap", 3, 3, 2, 0, ["Al", "Mg", "Si"], 1, 800.0, 1500, 20, None, "l12"),
    # corner sublattice + the three face sublattices merged into one group: groups of N/4 and 3N/4 sites
    ("l12_merged_flip", 4, 4, 2, 1, ["Al", "Mg"], 0, 800.0, 3000, 21, None, "l12:0111"),
    ("l12_merged_swap", 4, 4, 2, 1, ["Al", "Mg"], 1, 800.0, 3000, 22, None, "l12:0111"),
    # other cubic Bravais lattices (the reference's tests use BCC and SC cells, test_CE_updater.py:21,206-228)
    ("bcc_swap", 4, 4, 2, 1, ["Al", "Mg"], 1, 800.0, 3000, 23, None, "bcc"),
    ("sc_ternary_flip", 5, 3, 2, 1, ["Al", "Mg", "Si"], 0, 800.0, 1500, 24, None, "sc"),
    # HCP (space group P6_3/mmc): two translation groups related by a screw, 4 x 4 x 3 hexagonal cells
    ("hcp_swap", 4, 3, 2, 1, ["Mg", "Zn"], 1, 800.0, 3000, 25, None, "hcp:3"),
    ("hcp_ternary_flip", 4, 3, 2, 0, ["Al", "Mg", "Zn"], 0, 800.0, 1500, 26, None, "hcp:3"),
    # four translation groups on the active sublattice plus an inert one
    ("l12_background_swap", 4, 4, 2, 1, ["Li", "V"], 1, 800.0, 3000, 27, "O", "l12"),
]


def model_hash(m: CEModel) -> str:
    h = hashlib.sha256()
    for a in (m.table, m.term_eci, m.term_ref, m.term_size, m.term_nb, m.eci_weight, m.bf):
        h.update(np.ascontiguousarray(a).tobytes())
    h.update("|".join(m.eci_names).encode())
    return h.hexdigest()


def make_settings(lattice, L, ps, ts, qs, syms):
    """``fcc``, ``l12`` or ``l12:<group of each sublattice>`` (e.g. ``l12:0111``)."""
    if lattice.startswith("l12"):
        gob = tuple(int(ch) for ch in lattice.split(":")[1]) if ":" in lattice else (0, 1, 2, 3)
        return l12_settings(L, ps, ts, qs, syms, group_of_basis=gob)
    if lattice in ("bcc", "sc"):
        return cubic_settings(lattice, L, ps, ts, qs, syms)
    if lattice.startswith("hcp"):  # hcp:<cells along c>
        return hcp_settings(L, int(lattice.split(":")[1]), ps, ts, qs, syms)
    return fcc_settings(L, ps, ts, qs, syms)


def build_case(name, L, ps, ts, qs, syms, move, T, n, seed, background, lattice="fcc"):
    import oracle as O
    s = make_settings(lattice, L, ps, ts, qs, syms)
    if background:
        s = with_background(s, background)
    eci = seeded_ecis(s.cset, 0)
    m = CEModel(s, list(eci))
    orc = O.Oracle(m)
    rng = np.random.default_rng(seed)
    occ0 = rng.integers(0, len(syms), m.n_sites).astype(np.int8)
    occ0[m.background] = 0  # background sites keep a placeholder id; the reference sees the background symbol

    def ref_symbols(occ):
        out = m.symbols_of(occ)
        for i in m.background:
            out[int(i)] = background
        return out
    ev = m.eci_vector(eci)
    kT = KB * T
    st = orc.new_chain_state(occ0, ev, kT, move)
    cf0 = st.cf.copy()
    tr = orc.run(st, seed=seed, chain_id=0, t_begin=0, n_trials=n, trace=True)

    upd, _ = O.make_reference_updater(s, ref_symbols(occ0), dict(zip(m.eci_names, cf0)), eci)
    occ = occ0.copy()
    cur = upd.get_energy()
    acc = np.zeros(n, dtype=np.int8)
    de = np.zeros(n)
    for i in range(n):
        a, b = int(tr.site[2 * i]), int(tr.site[2 * i + 1])
        if move == 1:
            A, B = occ[a], occ[b]
            changes = [(a, m.symbols[A], m.symbols[B]), (b, m.symbols[B], m.symbols[A])]
        else:
            changes = [(a, m.symbols[occ[a]], m.symbols[b])]
        new = upd.calculate(changes)
        de[i] = new - cur
        ok = True if new < cur else (tr.u[i] <= math.exp(-(new - cur) / kT))
        acc[i] = ok
        if ok:
            upd.clear_history()
            cur = new
            for j, _, nw in changes:
                occ[j] = m.symbols.index(nw)
        else:
            upd.undo_changes()
    ref_cf = upd.get_cf()
    cf_final = np.array([ref_cf[k] for k in m.eci_names])

    # Known answers of explicit single-site updates (CEUpdater::update_cf).
    upd2, _ = O.make_reference_updater(s, ref_symbols(occ0), dict(zip(m.eci_names, cf0)), eci)
    occ_u = occ0.copy()
    n_upd = 12
    upd_sites = rng.choice(m.movable, n_upd, replace=False).astype(np.int32)
    upd_new = np.zeros(n_upd, dtype=np.int8)
    upd_cf = np.zeros((n_upd, m.n_eci))
    upd_e = np.zeros(n_upd)
    for i, site in enumerate(upd_sites):
        new = (occ_u[site] + 1 + rng.integers(len(syms) - 1)) % len(syms)
        upd_new[i] = new
        upd2.update_cf((int(site), m.symbols[occ_u[site]], m.symbols[new]))
        occ_u[site] = new
        c = upd2.get_cf()
        upd_cf[i] = [c[k] for k in m.eci_names]
        upd_e[i] = upd2.get_energy()

    return dict(
        L=L, shells=np.array([ps, ts, qs]), species=np.array(syms), move=move, T=T, kT=kT, seed=seed,
        background=np.array(background or ""), lattice=np.array(lattice),
        n_trials=n, model_hash=model_hash(m), eci=ev, eci_names=np.array(m.eci_names),
        occ0=occ0, cf0=cf0, sites=tr.site.reshape(n, 2), u=tr.u, ref_acc=acc, ref_de=de,
        occ_final=occ, cf_final=cf_final, energy_final=cur,
        upd_sites=upd_sites, upd_new=upd_new, upd_cf=upd_cf, upd_energy=upd_e,
    )


def build_constraint_verdicts():
    """Verdicts of the reference's own constraint classes (mc_constraints.py) on random moves.

    Loads cemc/mcmc/mc_constraints.py and cemc/tools/geometry.py from the reference tree
    by path (they import only numpy) and asks FixedElement, ConstrainElementByTag and
    FixEdgeLayers about random single-site changes and swaps of a ternary FCC 4x4x4 cell.
    """
    import importlib.util
    import types
    ref = os.environ.get("CEMC_REFERENCE", "")
    if not os.path.isdir(os.path.join(ref, "cemc")):
        raise SystemExit("set CEMC_REFERENCE to the reference source tree (it holds cemc/ and cpp/)")

    def load(name, rel):
        spec = importlib.util.spec_from_file_location(name, os.path.join(ref, rel))
        mod = importlib.util.module_from_spec(spec)
        sys.modules[name] = mod
        spec.loader.exec_module(mod)
        return mod

    for pkg in ("cemc", "cemc.tools"):
        sys.modules.setdefault(pkg, types.ModuleType(pkg))
    geom = load("cemc.tools.geometry", "cemc/tools/geometry.py")
    sys.modules["cemc.tools"].geometry = geom
    mc_cons = load("ref_mc_constraints", "cemc/mcmc/mc_constraints.py")

    syms = ["Al", "Mg", "Si"]
    s = fcc_settings(4, 3, 2, 0, syms)
    n = s.n_sites
    a = s.cell.a
    pos = s.cell.positions.astype(np.float64) * (a / 2.0)
    cell = np.eye(3) * (a * s.cell.L)

    class Atom:
        def __init__(self, index, tag):
            self.index, self.tag = index, tag

    class Atoms(list):
        def get_cell(self):
            return cell

        def get_positions(self):
            return pos

    tags = np.arange(n) % 4
    element_by_tag = [["Al", "Mg"], ["Mg"], ["Al", "Si"], ["Al", "Mg", "Si"]]
    atoms = Atoms(Atom(i, int(tags[i])) for i in range(n))
    thickness = 3.0
    cons = [mc_cons.FixedElement(element="Mg"), mc_cons.ConstrainElementByTag(atoms, element_by_tag),
            mc_cons.FixEdgeLayers(thickness=thickness, atoms=atoms)]
    rng = np.random.default_rng(33)
    occ = rng.integers(0, 3, n)
    n_moves = 600
    moves = np.full((n_moves, 2, 3), -1, dtype=np.int32)  # up to two changes (site, old id, new id)
    verdict = np.zeros((n_moves, len(cons)), dtype=np.int8)
    for k in range(n_moves):
        if k % 2 == 0:
            i = int(rng.integers(n))
            new = int((occ[i] + 1 + rng.integers(2)) % 3)
            ch = [(i, int(occ[i]), new)]
        else:
            i, j = (int(x) for x in rng.choice(n, 2, replace=False))
            while occ[i] == occ[j]:
                j = int(rng.integers(n))
            ch = [(i, int(occ[i]), int(occ[j])), (j, int(occ[j]), int(occ[i]))]
        for q, c in enumerate(ch):
            moves[k, q] = c
        changes = [(c[0], syms[c[1]], syms[c[2]]) for c in ch]
        verdict[k] = [bool(con(changes)) for con in cons]
    return dict(symbols=np.array(syms), positions=pos, cell=cell, tags=tags,
                element_by_tag=np.array(["|".join(e) for e in element_by_tag]), fixed_element=np.array("Mg"),
                thickness=np.array(thickness), moves=moves, verdict=verdict,
                constraint_names=np.array(["FixedElement", "ConstrainElementByTag", "FixEdgeLayers"]))


def main():
    import contextlib
    out_dir = HERE
    only = set(sys.argv[1:])  # case names to (re)generate; default all
    if not only or "constraints" in only:
        data = build_constraint_verdicts()
        np.savez_compressed(os.path.join(out_dir, "constraints_verdicts.npz"), **data)
        print("constraints_verdicts: %d moves, legal fractions %s" % (len(data["verdict"]),
                                                                     data["verdict"].mean(axis=0).round(3)))
    for case in CASES:
        if only and case[0] not in only:
            continue
        # the reference's init logs to the C++ streams; silence them at the fd level
        with open(os.devnull, "w") as devnull, contextlib.ExitStack():
            saved = os.dup(1), os.dup(2)
            os.dup2(devnull.fileno(), 1)
            os.dup2(devnull.fileno(), 2)
            try:
                data = build_case(*case)
            finally:
                os.dup2(saved[0], 1)
                os.dup2(saved[1], 2)
        path = os.path.join(out_dir, case[0] + ".npz")
        np.savez_compressed(path, **data)
        print("%s: %d trials, acceptance %.3f, final energy %.6f -> %s" % (
            case[0], data["n_trials"], data["ref_acc"].mean(), data["energy_final"], os.path.basename(path)))


if __name__ == "__main__":
    main()
