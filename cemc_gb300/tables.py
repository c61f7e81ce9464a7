"""Packed cluster-expansion tables built from a settings object.

``CEModel`` parses the same settings attributes the reference's native updater
reads in ``CEUpdater::init`` (``cpp/src/ce_updater.cpp:32-234``):
``unique_elements``, ``index_by_trans_symm``, ``background_indices``,
``cluster_info``, ``basis_functions`` and ``trans_matrix`` plus an ECI dict, and
produces

* the reference-shaped model (per-cluster member columns, canonical order,
  equivalent decorations, normalisation counts), and
* the flattened "terms" the GPU kernels walk: one term per (translation
  group, cluster ECI, equivalent decoration, sub-cluster), carrying the
  decoration index of the changed site and (column, decoration) of every
  other member, with the columns in the group's own order (``gpu_table``).

Semantics kept from the reference (``ce_updater.cpp``):
* ECI names are kept in sorted order (``named_array.cpp:7-23``);
* ``c0`` never changes, ``c1_<d>`` changes by ``(bf[d][new]-bf[d][old])/N_total``
  with ``N_total`` counting background sites (366-371);
* a cluster ECI ``<prefix>_<deco>`` sums over the equivalent decorations and
  the sub-clusters of the changed site's translation group and is scaled by
  ``size / |eq| / (M_prefix * N_group)`` (391-402), where ``M_prefix`` sums the
  sub-cluster counts over all groups (137-144) and ``N_group`` counts the
  group's sites (769-775);
* decoration digit ``q`` applies to the site at position ``order[q]`` of
  ``[ref] + members`` (``sort_indices``, 981-994).
"""
from __future__ import annotations

from typing import Dict, List, Sequence

import numpy as np

from .lattice import equivalent_decorations


def _split_name(name: str):
    pos = name.rfind("_")
    return name[:pos], name[pos + 1:]


class CEModel:
    def __init__(self, settings, eci_names: Sequence[str]):
        self.symbols: List[str] = sorted(set(settings.unique_elements))
        self.n_sym = len(self.symbols)
        self.n_bf = int(settings.num_unique_elements) - 1
        if self.n_bf < 1:
            raise ValueError("need at least two species")
        sym_id = {s: i for i, s in enumerate(self.symbols)}

        # Translation-symmetry groups and background sites (ce_updater.cpp:733-776, 1017-1026).
        groups = [list(map(int, g)) for g in settings.index_by_trans_symm]
        background = set(int(i) for i in settings.background_indices)
        n_sites = getattr(settings, "n_sites", None)
        if n_sites is None:
            tm = settings.trans_matrix
            n_sites = len(tm) if isinstance(tm, list) else int(np.asarray(tm).shape[0])
        self.n_sites = int(n_sites)
        site_group = np.full(self.n_sites, -1, dtype=np.int32)
        for gi, g in enumerate(groups):
            for i in g:
                if site_group[i] != -1:
                    raise RuntimeError("One site appears to be present in more than one translation symmetry group!")
                site_group[i] = gi
        for i in range(self.n_sites):
            if site_group[i] == -1 and i not in background:
                raise RuntimeError("Site %d has not been assigned to any translational symmetry group!" % i)
        self.site_group = site_group
        self.n_groups = len(groups)
        self.group_count = np.array([int((site_group == gi).sum()) for gi in range(self.n_groups)], dtype=np.int32)
        self.movable = np.nonzero(site_group >= 0)[0].astype(np.int32)
        self.background = np.array(sorted(background), dtype=np.int32)
        self.background_symbol = getattr(settings, "background_symbol", None)

        # Basis functions bf[dec, id] (basis_function.cpp:5-19).
        bf = np.zeros((self.n_bf, self.n_sym))
        for d, entry in enumerate(settings.basis_functions):
            for s, v in entry.items():
                bf[d, sym_id[s]] = float(v)
        self.bf = bf

        # Clusters per group (cluster.cpp:185-232) and their counts (ce_updater.cpp:115-148).
        info = settings.cluster_info
        type_names: List[str] = []
        for g in info:
            for name in g.keys():
                if name not in type_names:
                    type_names.append(name)
        type_names.sort()
        self.type_names = type_names
        tindex = {n: i for i, n in enumerate(type_names)}
        n_types = len(type_names)
        self.type_size = np.zeros(n_types, dtype=np.int32)
        self.type_m = np.zeros((n_types, self.n_groups), dtype=np.int32)
        self.type_off = np.zeros((n_types, self.n_groups), dtype=np.int32)
        self.type_equiv: List[List[List[int]]] = [[] for _ in range(n_types)]
        member_sites: List[List[int]] = []
        orders: List[List[int]] = []
        for gi, g in enumerate(info):
            for name in sorted(g.keys()):
                c = g[name]
                t = tindex[name]
                size = int(c["size"])
                if size > 4:
                    raise ValueError("Only cluster sizes 2, 3 and 4 are supported!")
                self.type_size[t] = size
                self.type_equiv[t] = [list(map(int, e)) for e in c.get("equiv_sites", [])]
                self.type_off[t, gi] = len(member_sites)
                self.type_m[t, gi] = len(c["indices"])
                for sub, order in zip(c["indices"], c["order"]):
                    member_sites.append([int(x) for x in sub])
                    orders.append([int(x) for x in order])
        self.type_M = self.type_m.sum(axis=1).astype(np.int32)

        # Neighbour columns: the sorted distinct member indices (ce_updater.cpp:899-979).
        cols = sorted({x for sub in member_sites for x in sub})
        self.column_sites = np.array(cols, dtype=np.int64)
        col_of = {c: i for i, c in enumerate(cols)}
        self.n_cols = len(cols)
        rows = len(member_sites)
        self.members = np.full((max(rows, 1), 3), -1, dtype=np.int32)
        self.order = np.full((max(rows, 1), 4), -1, dtype=np.int32)
        for r, (sub, order) in enumerate(zip(member_sites, orders)):
            self.members[r, :len(sub)] = [col_of[x] for x in sub]
            self.order[r, :len(order)] = order
        self.table = self._read_table(settings, cols)
        if len(self.background):  # background rows are never read; they point at the site itself
            self.table[self.background] = self.background[:, None]

        # ECIs in sorted-name order.
        names = sorted(eci_names)
        self.eci_names = names
        self.n_eci = len(names)
        self.eci_kind = np.zeros(self.n_eci, dtype=np.int32)
        self.eci_type = np.full(self.n_eci, -1, dtype=np.int32)
        self.eci_dec = np.full(self.n_eci, -1, dtype=np.int32)
        eq_off = [0]
        eq_decos: List[List[int]] = []
        self.singlet_eci = np.full(self.n_bf, -1, dtype=np.int32)
        for k, name in enumerate(names):
            if name.startswith("c0"):
                self.eci_kind[k] = 0
            elif name.startswith("c1"):
                dec = int(_split_name(name)[1])
                self.eci_kind[k] = 1
                self.eci_type[k] = dec
                self.eci_dec[k] = dec
                self.singlet_eci[dec] = k
            else:
                prefix, deco = _split_name(name)
                if prefix not in tindex:
                    raise ValueError("All ECIs does not correspond to a correlation function!")
                t = tindex[prefix]
                self.eci_kind[k] = 2
                self.eci_type[k] = t
                d = [int(ch) for ch in deco]
                if len(d) != self.type_size[t]:
                    raise ValueError("decoration of %s does not match the cluster size" % name)
                for e in equivalent_decorations(d, self.type_equiv[t]):
                    eq_decos.append(e + [0] * (4 - len(e)))
            eq_off.append(len(eq_decos))
        self.eq_off = np.array(eq_off, dtype=np.int32)
        self.eq_decos = np.array(eq_decos if eq_decos else [[0, 0, 0, 0]], dtype=np.int32)
        if np.any(self.singlet_eci < 0):
            missing = [b for b in range(self.n_bf) if self.singlet_eci[b] < 0]
            self.singlet_eci = np.where(self.singlet_eci < 0, 0, self.singlet_eci).astype(np.int32)
            self.missing_singlets = missing
        else:
            self.missing_singlets = []
        self._build_terms()

    @staticmethod
    def _read_table(settings, cols: List[int]) -> np.ndarray:
        """Neighbour table T[site, column] from the settings' translation matrix."""
        if hasattr(settings, "table") and hasattr(settings, "column_sites"):
            pos = {int(c): i for i, c in enumerate(settings.column_sites.tolist())}
            perm = np.array([pos[c] for c in cols], dtype=np.int64)
            return np.ascontiguousarray(settings.table[:, perm]).astype(np.int32)
        tm = settings.trans_matrix
        if isinstance(tm, list):
            out = np.zeros((len(tm), len(cols)), dtype=np.int32)
            for i, row in enumerate(tm):
                if not row:
                    out[i] = i  # background rows are never read; they point at the site itself
                    continue
                out[i] = [int(row[c]) for c in cols]
            return out
        tm = np.asarray(tm, dtype=np.int32)
        if max(cols) + 1 > tm.shape[1]:
            raise ValueError("Something is wrong with the translation matrix passed.")
        return np.ascontiguousarray(tm[:, cols])

    def _build_terms(self):
        """Flatten (group, ECI, equivalent decoration, sub-cluster) into GPU terms.

        Terms are sorted by translation group, then ECI.  Each group gets its
        own column order (the columns its sub-clusters name, ascending), and
        ``gpu_table`` lists a site's neighbours in its group's order; unused
        trailing entries point at the site itself, so every row is exactly
        the site's neighbourhood.  With one group this is the reference's
        column order and ``gpu_table == table``.
        """
        G = self.n_groups
        self.gpu_supported = self.n_bf <= 4 and 1 <= G <= 8
        group_cols: List[List[int]] = []
        for g in range(G):
            used = set()
            for t in range(len(self.type_names)):
                off, m, size = int(self.type_off[t, g]), int(self.type_m[t, g]), int(self.type_size[t])
                for r in range(off, off + m):
                    used.update(int(c) for c in self.members[r, :size - 1])
            group_cols.append(sorted(used))
        self.group_cols = group_cols
        n_pack = max([len(c) for c in group_cols] + [1])
        gpu_table = np.repeat(np.arange(self.n_sites, dtype=np.int32)[:, None], n_pack, axis=1)
        for g in range(G):
            sites = np.nonzero(self.site_group == g)[0]
            cols = group_cols[g]
            if len(cols):
                gpu_table[np.ix_(sites, np.arange(len(cols)))] = self.table[np.ix_(sites, np.array(cols))]
        self.gpu_table = np.ascontiguousarray(gpu_table, dtype=np.int32)
        self.gpu_n_cols = int(n_pack)
        n_ref = int(self.group_count[0]) if G else 1
        self.group_scale = np.array([float(n_ref) / float(max(int(c), 1)) for c in self.group_count]
                                    if G else [1.0])

        term_eci, term_ref, term_size, term_nb, group_terms = [], [], [], [], [0]
        weight = np.zeros(self.n_eci)
        full_weight = np.zeros(self.n_eci)
        for k in range(self.n_eci):
            if self.eci_kind[k] != 2:
                continue
            t = self.eci_type[k]
            n_eq = int(self.eq_off[k + 1] - self.eq_off[k])
            if int(self.type_M[t]) > 0 and G >= 1:
                weight[k] = (float(self.type_size[t]) / float(n_eq)) / float(int(self.type_M[t]) * n_ref)
            norm = sum(int(self.type_m[t, s]) * int(self.group_count[s]) for s in range(G))
            full_weight[k] = 1.0 / (float(n_eq) * float(norm)) if norm else 0.0
        for g in range(G):
            pos = {c: j for j, c in enumerate(group_cols[g])}
            for k in range(self.n_eci):
                if self.eci_kind[k] != 2:
                    continue
                t = self.eci_type[k]
                size = int(self.type_size[t])
                decos = self.eq_decos[self.eq_off[k]:self.eq_off[k + 1]]
                off, m = int(self.type_off[t, g]), int(self.type_m[t, g])
                for deco in decos:
                    for r in range(off, off + m):
                        order = self.order[r, :size]
                        inv = np.empty(size, dtype=np.int64)
                        inv[order] = np.arange(size)
                        d = [int(deco[inv[p]]) for p in range(size)]
                        term_eci.append(k)
                        term_ref.append(d[0])
                        term_size.append(size)
                        nb = [pos[int(self.members[r, j])] * self.n_bf + d[j + 1] for j in range(size - 1)]
                        term_nb.append(nb + [0] * (3 - len(nb)))
            group_terms.append(len(term_eci))
        self.term_eci = np.array(term_eci, dtype=np.int32)
        self.term_ref = np.array(term_ref, dtype=np.int32)
        self.term_size = np.array(term_size, dtype=np.int32)
        self.term_nb = np.array(term_nb if term_nb else np.zeros((0, 3)), dtype=np.int32).reshape(-1, 3)
        self.n_terms = len(term_eci)
        self.group_terms = np.array(group_terms if G else [0, 0], dtype=np.int32)
        self.eci_weight = weight
        self.eci_full_weight = full_weight

    def eci_vector(self, eci: Dict[str, float]) -> np.ndarray:
        return np.array([float(eci.get(n, 0.0)) for n in self.eci_names])

    def occupation(self, symbols: Sequence[str]) -> np.ndarray:
        """Species ids of atom symbols; background sites get the placeholder id 0."""
        lut = {s: i for i, s in enumerate(self.symbols)}
        bg = set(self.background.tolist())
        return np.array([0 if i in bg else lut[s] for i, s in enumerate(symbols)], dtype=np.int8)

    def symbols_of(self, occ: np.ndarray) -> List[str]:
        """Atom symbols of species ids; background sites read the settings' background symbol."""
        out = [self.symbols[int(i)] for i in occ]
        if self.background_symbol is not None:
            for i in self.background.tolist():
                out[i] = self.background_symbol
        return out
