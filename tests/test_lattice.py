"""Geometry and cluster generator: shells, cluster multiplicities, symmetry, names."""
import itertools

import numpy as np
import pytest

from cemc_gb300.lattice import (FCCSupercell, enumerate_cluster_types, equivalent_decorations, fcc_settings,
                                fcc_shell_vectors, seeded_ecis)
from cemc_gb300.tables import CEModel


def test_fcc_shell_multiplicities():
    shells = fcc_shell_vectors(6)
    assert [len(s) for s in shells] == [12, 6, 24, 12, 24, 8]
    assert [int((s[0] ** 2).sum()) for s in shells] == [2, 4, 6, 8, 10, 12]


def test_supercell_indexing_roundtrip():
    cell = FCCSupercell(3)
    assert cell.n_sites == 4 * 27
    idx = cell.index_of(cell.positions)
    assert np.array_equal(idx, np.arange(cell.n_sites))
    # periodic images map to the same site
    assert np.array_equal(cell.index_of(cell.positions + 2 * cell.L), idx)


def test_cluster_counts_binary_recipe():
    types = enumerate_cluster_types(4, 2, 1)
    got = [(t.size, t.dia2, len(t.offsets)) for t in types]
    assert got == [(2, 2, 12), (2, 4, 6), (2, 6, 24), (2, 8, 12), (3, 2, 24), (3, 4, 36), (4, 2, 8)]
    terms = sum(len(t.offsets) for t in types)
    assert terms == 122  # sub-cluster products per flip of the binary recipe


def test_cluster_orbits_cover_every_occurrence():
    """Each cluster containing the origin appears once per (type, ordering) and every order maps onto the prototype."""
    for t in enumerate_cluster_types(5, 3, 1):
        seen = set()
        for off, order in zip(t.offsets, t.order):
            pts = np.vstack([np.zeros((1, 3), dtype=np.int64), off])
            key = tuple(sorted(map(tuple, pts.tolist())))
            assert key not in seen
            seen.add(key)
            # the canonical ordering reproduces the prototype's pairwise distances
            ordered = pts[order]
            d1 = ((ordered[:, None] - ordered[None]) ** 2).sum(-1)
            p = t.prototype
            d2 = ((p[:, None] - p[None]) ** 2).sum(-1)
            assert np.array_equal(d1, d2)
        # each cluster of size s is counted once per member: multiplicity divisible by size over the orbit
        assert len(t.offsets) % 1 == 0


@pytest.mark.parametrize("L", [4, 6])
def test_neighbour_relation_is_symmetric(L):
    s = fcc_settings(L, 4, 2, 1, ["Al", "Mg"])
    tab = s.table
    n = s.n_sites
    for i in range(0, n, max(1, n // 37)):
        for j in tab[i]:
            assert i in set(tab[j].tolist())


def test_no_self_interaction_and_distinct_members():
    s = fcc_settings(4, 5, 3, 1, ["Al", "Mg", "Si"])
    for name, info in s.cluster_info[0].items():
        for sub in info["indices"]:
            assert info["ref_indx"] not in sub
            assert len(set(sub)) == len(sub)


def test_supercell_too_small_is_rejected():
    with pytest.raises(ValueError):
        fcc_settings(1, 4, 2, 1, ["Al", "Mg"])


def test_equivalent_decorations():
    assert equivalent_decorations([0, 1], [[0, 1]]) == [[0, 1], [1, 0]]
    assert equivalent_decorations([0, 0, 1], [[0, 1, 2]]) == [[0, 0, 1], [0, 1, 0], [1, 0, 0]]
    assert equivalent_decorations([0, 1, 1], [[1, 2]]) == [[0, 1, 1]]
    assert equivalent_decorations([1, 0, 1], []) == [[1, 0, 1]]
    # every decoration's class contains it and classes partition the decorations
    eq = [[0, 1, 2, 3]]
    for deco in itertools.product(range(2), repeat=4):
        cls = equivalent_decorations(list(deco), eq)
        assert list(deco) in cls
        assert all(sorted(c) == sorted(deco) for c in cls)


def test_eci_names_sorted_and_parseable():
    s = fcc_settings(4, 5, 3, 1, ["Al", "Mg", "Si"])
    names = s.cset.names
    assert names == sorted(names)
    assert names[0] == "c0" and names[1] == "c1_0" and names[2] == "c1_1"
    assert len(names) == 63
    for n in names[3:]:
        prefix, deco = n.rsplit("_", 1)
        assert prefix in s.cluster_info[0]
        assert len(deco) == s.cluster_info[0][prefix]["size"]


def test_seeded_ecis_recipe():
    s = fcc_settings(4, 4, 2, 1, ["Al", "Mg"])
    e1 = seeded_ecis(s.cset, 0)
    e2 = seeded_ecis(s.cset, 0)
    assert e1 == e2 and e1["c0"] == -3.0
    assert seeded_ecis(s.cset, 1) != e1


def test_model_terms_and_weights():
    s = fcc_settings(4, 4, 2, 1, ["Al", "Mg"])
    eci = seeded_ecis(s.cset, 0)
    m = CEModel(s, list(eci))
    assert m.n_terms == 122 and m.n_cols == 54
    assert np.all(np.diff(m.term_eci) >= 0)
    n = m.n_sites
    for k, name in enumerate(m.eci_names):
        if m.eci_kind[k] == 2:
            t = m.eci_type[k]
            size = m.type_size[t]
            assert m.eci_weight[k] == pytest.approx(size / (m.type_M[t] * n))
            assert m.eci_full_weight[k] == pytest.approx(1.0 / (m.type_M[t] * n))


def test_model_from_sparse_translation_matrix_matches_dense():
    """The list-of-dicts translation matrix (the reference's sparse form) gives the same table."""
    s = fcc_settings(4, 4, 2, 1, ["Al", "Mg"])
    eci = seeded_ecis(s.cset, 0)
    m1 = CEModel(s, list(eci))

    class Plain:
        pass

    p = Plain()
    for attr in ("unique_elements", "num_unique_elements", "index_by_trans_symm", "background_indices",
                 "cluster_info", "basis_functions", "trans_matrix"):
        setattr(p, attr, getattr(s, attr))
    m2 = CEModel(p, list(eci))
    assert np.array_equal(m1.table, m2.table)
    assert np.array_equal(m1.term_nb, m2.term_nb)
    dense = np.zeros((s.n_sites, int(s.column_sites.max()) + 1), dtype=np.int32)
    dense[:, s.column_sites] = s.table
    p.trans_matrix = dense
    m3 = CEModel(p, list(eci))
    assert np.array_equal(m1.table, m3.table)


def test_model_rejects_unknown_eci():
    s = fcc_settings(4, 4, 2, 1, ["Al", "Mg"])
    with pytest.raises(ValueError):
        CEModel(s, ["c0", "c1_0", "c7_d9999_0_0000000"])


def test_cubic_lattice_shells_and_neighbour_symmetry():
    """BCC / SC shells (8, 6, 12, 24 and 6, 12, 8, 6 neighbours) and a symmetric neighbour relation."""
    from cemc_gb300.lattice import cubic_settings, shell_vectors
    assert [len(v) for v in shell_vectors("bcc", 4)] == [8, 6, 12, 24]
    assert [len(v) for v in shell_vectors("sc", 4)] == [6, 12, 8, 6]
    for kind, L in (("bcc", 4), ("sc", 5)):
        s = cubic_settings(kind, L, 3, 2, 0, ["Al", "Mg"])
        tab = s.table
        rows = [set(r.tolist()) for r in tab]
        for i in range(s.n_sites):
            for j in rows[i]:
                assert i in rows[j]
        m = CEModel(s, list(seeded_ecis(s.cset, 0)))
        assert m.n_groups == 1 and np.array_equal(m.gpu_table, m.table)


def test_l12_groups_share_names_and_pack_columns():
    """Four translation groups of equal size; the three face groups see the same cluster names; each
    group's table row lists only its own neighbours (self-padded), and the relation stays symmetric."""
    from cemc_gb300.lattice import l12_settings
    s = l12_settings(4, 4, 2, 1, ["Al", "Mg"])
    assert [len(g) for g in s.index_by_trans_symm] == [64, 64, 64, 64]
    names = [set(d) for d in s.cluster_info]
    assert names[1] == names[2] == names[3] and names[0] != names[1]
    m = CEModel(s, list(seeded_ecis(s.cset, 0)))
    assert m.n_groups == 4 and m.gpu_n_cols == 54 and m.n_cols > 54
    assert np.allclose(m.group_scale, 1.0)
    rows = [set(r.tolist()) for r in m.gpu_table]
    for i in range(m.n_sites):
        for j in rows[i]:
            assert i in rows[j]
    merged = CEModel(l12_settings(4, 4, 2, 1, ["Al", "Mg"], group_of_basis=(0, 1, 1, 1)),
                     list(seeded_ecis(s.cset, 0)))
    assert merged.n_groups == 2 and np.allclose(merged.group_scale, [1.0, 1.0 / 3.0])


def test_hcp_space_group_shells_and_groups():
    """HCP (P6_3/mmc): 24 space-group operations, shells of 12, 6, 2, 18 neighbours, two translation groups
    sharing every cluster name, in-plane and out-of-plane nearest-neighbour pairs as distinct types."""
    from cemc_gb300.lattice import _HCP_BASIS, _hcp_ops, _hex_metric, hcp_settings, hcp_shell_radii
    import itertools
    assert len(_hcp_ops()) == 24
    radii = hcp_shell_radii(4)
    rng = np.arange(-3, 4)
    cells = np.array(list(itertools.product(rng, rng, rng))) * 6
    pts = (cells[:, None, :] + _HCP_BASIS[None]).reshape(-1, 3)
    q = _hex_metric(pts)
    assert [int((q == r).sum()) for r in radii] == [12, 6, 2, 18]
    s = hcp_settings(4, 3, 3, 2, 1, ["Mg", "Zn"])
    assert len(s.index_by_trans_symm) == 2 and set(s.cluster_info[0]) == set(s.cluster_info[1])
    pairs = [t for t in s.cset.types if t.size == 2 and t.dia2 == 108]
    assert sorted(len(t.members[0]) for t in pairs) == [6, 6]
    m = CEModel(s, list(seeded_ecis(s.cset, 0)))
    rows = [set(r.tolist()) for r in m.gpu_table]
    for i in range(m.n_sites):
        for j in rows[i]:
            assert i in rows[j]


@pytest.mark.parametrize("case", __import__("conftest").golden_cases())
def test_gpu_packing_invariants(case):
    """Per-group packing the kernels rely on, for every golden model: each group's terms are one
    ECI-sorted range, name only its own columns, and the packed row of a site lists its group's
    columns of the reference-shaped table; the row relation is symmetric."""
    from conftest import golden_model, load_golden
    g = load_golden(case)
    s, m, eci = golden_model(g)
    gt = m.group_terms
    assert gt[0] == 0 and gt[-1] == m.n_terms and np.all(np.diff(gt) >= 0) and len(gt) == m.n_groups + 1
    for q in range(m.n_groups):
        lo, hi = int(gt[q]), int(gt[q + 1])
        assert np.all(np.diff(m.term_eci[lo:hi]) >= 0)
        ncol = len(m.group_cols[q])
        for t in range(lo, hi):
            for j in range(int(m.term_size[t]) - 1):
                assert int(m.term_nb[t, j]) // m.n_bf < ncol
        sites = np.nonzero(m.site_group == q)[0]
        assert np.array_equal(m.gpu_table[np.ix_(sites, np.arange(ncol))],
                              m.table[np.ix_(sites, np.array(m.group_cols[q]))])
        assert np.all(m.gpu_table[sites, ncol:] == sites[:, None])
    rows = [set(r.tolist()) for r in m.gpu_table]
    for i in m.movable.tolist():
        for j in rows[i]:
            assert i in rows[j]
    assert np.allclose(m.group_scale, m.group_count[0] / np.maximum(m.group_count, 1))


def test_generator_argument_checks():
    """Group assignments must number the groups 0..n-1; cells too small for the cluster recipe alias
    members onto one site and are refused."""
    from cemc_gb300.lattice import hcp_settings, l12_settings
    with pytest.raises(ValueError):
        l12_settings(4, 3, 2, 0, ["Al", "Mg"], group_of_basis=(0, 2, 2, 2))
    with pytest.raises(ValueError):
        l12_settings(4, 3, 2, 0, ["Al", "Mg"], group_of_basis=(0, 1, 1))
    with pytest.raises(ValueError):
        hcp_settings(1, 1, 3, 2, 0, ["Mg", "Zn"])
    s = l12_settings(4, 3, 2, 0, ["Al", "Mg"], group_of_basis=(0, 0, 1, 1))
    assert [len(g) for g in s.index_by_trans_symm] == [128, 128]
