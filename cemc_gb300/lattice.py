"""Cubic supercells, cluster enumeration and the settings object a CE updater reads.

The reference takes its lattice, clusters, translation matrix and basis
functions from a CLEASE settings object (``BC``) and parses it in
``cpp/src/ce_updater.cpp:43-212`` and ``cpp/src/cluster.cpp:185-232``.  CLEASE is
not part of this project, so this module generates the same information for
cubic supercells (FCC, BCC, SC; and FCC with the four sublattices of its L1_2
ordering as separate translation-symmetry groups) from the geometry alone:

* sites of an ``L x L x L`` conventional cubic supercell (4, 2 or 1 sites per
  cube), ordered like ``bulk(..., cubic=True).repeat((L, L, L))``;
* neighbour shells and all pair / triplet / quadruplet clusters that contain
  the reference site 0, classified into symmetry-distinct types with the 48
  operations of the cubic point group plus lattice translations;
* for every sub-cluster the ``order`` permutation onto a canonical labelling
  and, per type, the ``equiv_sites`` groups (orbits of the cluster's own
  symmetry), which fix the equivalent-decoration averaging of
  ``cpp/src/cluster.cpp:41-128``;
* the translation table ``T[i, c]`` = site reached from site ``i`` by the
  offset of neighbour column ``c`` (the reference's
  ``RowSparseStructMatrix``, ``cpp/src/row_sparse_struct_matrix.cpp:114-122``);
* basis functions: binary spins (+1, -1) and the ternary basis
  phi1 = sqrt(3/2) s, phi2 = sqrt(2) (1 - 3/2 s^2) over spins (+1, 0, -1).

Cluster names follow the reference's naming contract: ``c0``, ``c1_<d>`` and
``c<size>_d<dia>_<variant>_<decostring>``; the decoration string is the part
after the last underscore (``ce_updater.cpp:701-710``).
"""
from __future__ import annotations

import itertools
import math
from dataclasses import dataclass, field
from typing import Dict, List, Sequence, Tuple

import numpy as np

# Conventional cubic bases in half-lattice-constant units (site order inside a cube).
_FCC_BASIS = np.array([(0, 0, 0), (0, 1, 1), (1, 0, 1), (1, 1, 0)], dtype=np.int64)
_CUBIC_BASES = {
    "fcc": _FCC_BASIS,
    "bcc": np.array([(0, 0, 0), (1, 1, 1)], dtype=np.int64),
    "sc": np.array([(0, 0, 0)], dtype=np.int64),
}


def _is_lattice_vector(kind: str, g: np.ndarray) -> np.ndarray:
    """Rows of ``g`` (half-lattice units) that are vectors of the cubic Bravais lattice ``kind``."""
    if kind == "fcc":
        return g.sum(axis=1) % 2 == 0
    if kind == "bcc":
        par = np.mod(g, 2)
        return (par == par[:, :1]).all(axis=1)
    if kind == "sc":
        return (np.mod(g, 2) == 0).all(axis=1)
    raise ValueError("unknown lattice %r (fcc, bcc or sc)" % kind)


def _cubic_point_group() -> np.ndarray:
    """The 48 signed permutation matrices of the cubic group O_h."""
    ops = []
    for perm in itertools.permutations(range(3)):
        for signs in itertools.product((1, -1), repeat=3):
            m = np.zeros((3, 3), dtype=np.int64)
            for r, (c, s) in enumerate(zip(perm, signs)):
                m[r, c] = s
            ops.append(m)
    return np.array(ops)


_OH = _cubic_point_group()


def shell_vectors(kind: str, max_shell: int) -> List[np.ndarray]:
    """Neighbour vectors of a cubic Bravais lattice (half-lattice units), one array per shell.

    Shell k (1-based) holds every lattice vector with the k-th smallest
    non-zero length.  FCC lattice vectors are the integer vectors whose
    coordinate sum is even; BCC ones have coordinates of one parity; SC ones
    are even.
    """
    r = 2
    while True:
        rng = np.arange(-r, r + 1)
        g = np.array(np.meshgrid(rng, rng, rng, indexing="ij")).reshape(3, -1).T
        g = g[_is_lattice_vector(kind, g) & (np.abs(g).sum(axis=1) > 0)]
        d2 = (g * g).sum(axis=1)
        radii = np.unique(d2)
        # Every shell up to max_shell is complete if its radius is below r^2.
        if len(radii) >= max_shell and radii[max_shell - 1] < r * r:
            shells = []
            for k in range(max_shell):
                v = g[d2 == radii[k]]
                order = np.lexsort(v.T[::-1])
                shells.append(v[order])
            return shells
        r += 1


def fcc_shell_vectors(max_shell: int) -> List[np.ndarray]:
    return shell_vectors("fcc", max_shell)


def shell_radius2(max_shell: int, kind: str = "fcc") -> List[int]:
    return [int((s[0] * s[0]).sum()) for s in shell_vectors(kind, max_shell)]


@dataclass
class ClusterType:
    """One symmetry-distinct cluster (the reference's ``Cluster``, ``cluster.hpp:14-54``)."""

    name: str  # prefix, e.g. c2_d0000_0
    size: int
    dia2: int  # squared max distance, half-lattice units
    prototype: np.ndarray  # (size, 3) canonical labelling of the sites
    equiv_sites: List[List[int]]
    # Sub-clusters containing the reference site (site at the origin):
    offsets: List[np.ndarray] = field(default_factory=list)  # (size-1, 3) member vectors
    order: List[List[int]] = field(default_factory=list)  # canonical position -> index in [ref]+members


def _canonical_key(points: np.ndarray) -> Tuple:
    """Symmetry-invariant key of a finite point set (translations + O_h)."""
    best = None
    for v in points:
        shifted = points - v
        for g in _OH:
            img = shifted @ g.T
            key = tuple(sorted(map(tuple, img.tolist())))
            if best is None or key < best:
                best = key
    return best


def _map_onto(points: np.ndarray, proto: np.ndarray) -> List[int]:
    """Find a lattice symmetry carrying ``proto`` onto ``points``.

    Returns ``order`` with ``order[q]`` = index into ``points`` of the site that
    canonical position ``q`` lands on.
    """
    proto_set = {tuple(p): q for q, p in enumerate(proto.tolist())}
    for v in points:
        shifted = points - v
        for g in _OH:
            img = shifted @ g.T
            mapping = [proto_set.get(tuple(p)) for p in img.tolist()]
            if None in mapping or len(set(mapping)) != len(mapping):
                continue
            order = [0] * len(points)
            for idx, q in enumerate(mapping):
                order[q] = idx
            return order
    raise RuntimeError("sub-cluster is not equivalent to its prototype")


def _equiv_sites(proto: np.ndarray) -> List[List[int]]:
    """Orbits (size >= 2) of the prototype's own symmetry on its positions."""
    n = len(proto)
    parent = list(range(n))

    def find(a):
        while parent[a] != a:
            parent[a] = parent[parent[a]]
            a = parent[a]
        return a

    proto_set = {tuple(p): q for q, p in enumerate(proto.tolist())}
    for v in proto:
        shifted = proto - v
        for g in _OH:
            img = shifted @ g.T
            # translate so that the image coincides with the prototype as a set
            for w in proto:
                cand = img + w
                mapping = [proto_set.get(tuple(p)) for p in cand.tolist()]
                if None in mapping or len(set(mapping)) != n:
                    continue
                for q in range(n):
                    a, b = find(q), find(mapping[q])
                    if a != b:
                        parent[a] = b
    groups: Dict[int, List[int]] = {}
    for q in range(n):
        groups.setdefault(find(q), []).append(q)
    return [sorted(gq) for gq in sorted(groups.values()) if len(gq) >= 2]


def enumerate_cluster_types(pair_shells: int, triplet_shells: int, quad_shells: int,
                            kind: str = "fcc") -> List[ClusterType]:
    """All pair/triplet/quad types of a cubic Bravais lattice with max distance in the given shells.

    A cluster of size >= 3 belongs to the set if every pairwise distance is at
    most the radius of shell ``triplet_shells`` (resp. ``quad_shells``); size 0
    means "no clusters of that size".  Symmetry: lattice translations and O_h.
    """
    max_shell = max(pair_shells, triplet_shells, quad_shells, 1)
    shells = shell_vectors(kind, max_shell)
    radii = [int((s[0] * s[0]).sum()) for s in shells]
    types: List[ClusterType] = []

    def add_size(size: int, n_shells: int):
        if n_shells <= 0:
            return
        cutoff = radii[n_shells - 1]
        nbrs = np.concatenate(shells[:n_shells])
        found: Dict[Tuple, ClusterType] = {}
        for combo in itertools.combinations(range(len(nbrs)), size - 1):
            pts = np.vstack([np.zeros((1, 3), dtype=np.int64), nbrs[list(combo)]])
            diff = pts[:, None, :] - pts[None, :, :]
            d2 = (diff * diff).sum(axis=2)
            if d2.max() > cutoff:
                continue
            key = _canonical_key(pts)
            ct = found.get(key)
            if ct is None:
                proto = np.array(key, dtype=np.int64)
                ct = ClusterType(name="", size=size, dia2=int(d2.max()), prototype=proto,
                                 equiv_sites=_equiv_sites(proto))
                found[key] = ct
            ct.offsets.append(pts[1:].copy())
            ct.order.append(_map_onto(pts, ct.prototype))
        # Name: c<size>_d<dia index>_<variant>, diameters ranked within this size.
        cts = sorted(found.values(), key=lambda c: (c.dia2, len(c.offsets), c.prototype.tolist()))
        dias = sorted({c.dia2 for c in cts})
        variant: Dict[int, int] = {}
        for c in cts:
            di = dias.index(c.dia2)
            v = variant.get(di, 0)
            variant[di] = v + 1
            c.name = "c%d_d%04d_%d" % (size, di, v)
            types.append(c)

    add_size(2, pair_shells)
    add_size(3, triplet_shells)
    add_size(4, quad_shells)
    return types


def equivalent_decorations(deco: Sequence[int], equiv_sites: Sequence[Sequence[int]]) -> List[List[int]]:
    """Distinct decorations reachable by permuting positions inside each equivalent-site group.

    This is the averaging set the reference obtains from
    ``equivalent_deco`` (called at ``cpp/src/cluster.cpp:78-110``): the product of
    the permutation groups of every group of equivalent positions, applied to
    the decoration, with duplicates removed (first occurrence kept).
    """
    deco = list(deco)
    if not equiv_sites:
        return [deco]
    per_group = [list(itertools.permutations(g)) for g in equiv_sites]
    out: List[List[int]] = []
    seen = set()
    for choice in itertools.product(*per_group):
        new = list(deco)
        for group, perm in zip(equiv_sites, choice):
            for src, dst in zip(group, perm):
                new[dst] = deco[src]
        t = tuple(new)
        if t not in seen:
            seen.add(t)
            out.append(new)
    return out


def binary_basis(symbols: Sequence[str]) -> List[Dict[str, float]]:
    """Spin basis for two species: +1 for the first (sorted) symbol, -1 for the second."""
    s = sorted(symbols)
    return [{s[0]: 1.0, s[1]: -1.0}]


def ternary_basis(symbols: Sequence[str]) -> List[Dict[str, float]]:
    """phi1 = sqrt(3/2) s, phi2 = sqrt(2) (1 - 1.5 s^2), spins +1, 0, -1 in sorted symbol order."""
    s = sorted(symbols)
    spins = {s[0]: 1.0, s[1]: 0.0, s[2]: -1.0}
    phi1 = {k: math.sqrt(1.5) * v for k, v in spins.items()}
    phi2 = {k: math.sqrt(2.0) * (1.0 - 1.5 * v * v) for k, v in spins.items()}
    return [phi1, phi2]


class CubicSupercell:
    """Sites and periodic translation of an ``L x L x L`` supercell of conventional cubes.

    ``kind`` is ``fcc`` (4 sites per cube), ``bcc`` (2) or ``sc`` (1); sites
    are ordered cube by cube, basis order inside a cube, like
    ``bulk(..., cubic=True).repeat((L, L, L))``.
    """

    def __init__(self, L: int, a: float = 4.05, kind: str = "fcc"):
        if L < 1:
            raise ValueError("supercell size must be positive")
        if kind not in _CUBIC_BASES:
            raise ValueError("unknown lattice %r (fcc, bcc or sc)" % kind)
        self.kind = kind
        self.basis = _CUBIC_BASES[kind]
        self.L = int(L)
        self.a = float(a)
        self.period = 2 * self.L
        cells = np.array(list(itertools.product(range(L), repeat=3)), dtype=np.int64)
        pos = (2 * cells)[:, None, :] + self.basis[None, :, :]
        self.positions = pos.reshape(-1, 3)  # half-lattice units
        self.n_sites = len(self.positions)
        self._parity_code = {tuple(b.tolist()): i for i, b in enumerate(self.basis)}

    def index_of(self, pos: np.ndarray) -> np.ndarray:
        """Site index of (possibly unwrapped) positions, shape (..., 3)."""
        p = np.mod(pos, self.period)
        cell = p // 2
        parity = p % 2
        code = (parity[..., 0] * 4 + parity[..., 1] * 2 + parity[..., 2]).astype(np.int64)
        lut = np.full(8, -1, dtype=np.int64)
        for par, i in self._parity_code.items():
            lut[par[0] * 4 + par[1] * 2 + par[2]] = i
        b = lut[code]
        if np.any(b < 0):
            raise ValueError("position is not a %s lattice site" % self.kind.upper())
        L = self.L
        return ((cell[..., 0] * L + cell[..., 1]) * L + cell[..., 2]) * len(self.basis) + b


class FCCSupercell(CubicSupercell):
    """``L x L x L`` conventional FCC supercell (4 sites per cube)."""

    def __init__(self, L: int, a: float = 4.05):
        super().__init__(L, a, "fcc")


@dataclass
class ECIName:
    name: str
    kind: str  # "c0", "c1" or "cluster"
    decoration: List[int]
    cluster: int = -1  # index into ClusterSet.types for kind == "cluster"


class ClusterSet:
    """Cluster types, decorations and ECI names of one lattice/cluster recipe."""

    def __init__(self, types: List[ClusterType], n_bf: int):
        self.types = types
        self.n_bf = n_bf
        self.type_index = {t.name: i for i, t in enumerate(types)}
        names: List[ECIName] = [ECIName("c0", "c0", [])]
        for b in range(n_bf):
            names.append(ECIName("c1_%d" % b, "c1", [b]))
        for ti, t in enumerate(types):
            reps = set()
            for deco in itertools.product(range(n_bf), repeat=t.size):
                eq = equivalent_decorations(deco, t.equiv_sites)
                rep = min(tuple(d) for d in eq)
                reps.add(rep)
            for rep in sorted(reps):
                s = "".join(str(d) for d in rep)
                names.append(ECIName("%s_%s" % (t.name, s), "cluster", list(rep), ti))
        # NamedArray keeps its names sorted (cpp/src/named_array.cpp:7-23).
        names.sort(key=lambda e: e.name)
        self.eci_names = names

    @property
    def names(self) -> List[str]:
        return [e.name for e in self.eci_names]

    def neighbour_offsets(self) -> np.ndarray:
        """Distinct member offsets over all sub-clusters (the table columns), sorted."""
        offs = set()
        for t in self.types:
            for o in t.offsets:
                for v in o.tolist():
                    offs.add(tuple(v))
        return np.array(sorted(offs), dtype=np.int64).reshape(-1, 3)


def fcc_cluster_set(pair_shells: int, triplet_shells: int, quad_shells: int, n_species: int,
                    kind: str = "fcc") -> ClusterSet:
    return ClusterSet(enumerate_cluster_types(pair_shells, triplet_shells, quad_shells, kind), n_species - 1)


class Settings:
    """Duck-typed stand-in for the settings object ``CEUpdater::init`` reads.

    Attribute formats follow ``cpp/src/ce_updater.cpp:43-212`` and
    ``cpp/src/cluster.cpp:185-232``: ``unique_elements``, ``num_unique_elements``,
    ``index_by_trans_symm``, ``background_indices``, ``cluster_info``,
    ``basis_functions`` and ``trans_matrix`` (here a list of dicts, the
    reference's sparse form, since the dense form is ``N x max_column``).
    It also carries the packed arrays the GPU path uses.
    """

    def __init__(self, cell: CubicSupercell, cset: ClusterSet, symbols: Sequence[str]):
        self.cell = cell
        self.cset = cset
        self.unique_elements = sorted(symbols)
        self.num_unique_elements = len(self.unique_elements)
        if self.num_unique_elements - 1 != cset.n_bf:
            raise ValueError("cluster set decorations do not match the species count")
        if self.num_unique_elements == 2:
            self.basis_functions = binary_basis(self.unique_elements)
        elif self.num_unique_elements == 3:
            self.basis_functions = ternary_basis(self.unique_elements)
        else:
            raise ValueError("only binary and ternary alloys are generated")
        n = cell.n_sites
        self.n_sites = n
        self.index_by_trans_symm = [list(range(n))]
        self.background_indices: List[int] = []
        offs = cset.neighbour_offsets()
        self.column_offsets = offs
        col_sites = cell.index_of(offs)  # site index of each column = neighbour of site 0
        if len(set(col_sites.tolist())) != len(col_sites) or 0 in set(col_sites.tolist()):
            raise ValueError("supercell too small: neighbour offsets alias onto the same site")
        self.column_sites = col_sites
        # table[i, c] = site reached from site i by column offset c
        self.table = cell.index_of(cell.positions[:, None, :] + offs[None, :, :]).astype(np.int32)
        off_to_col = {tuple(v): c for c, v in enumerate(offs.tolist())}
        self.member_cols: List[np.ndarray] = []
        info: Dict[str, dict] = {}
        for t in cset.types:
            cols = np.array([[off_to_col[tuple(v)] for v in o.tolist()] for o in t.offsets], dtype=np.int32)
            self.member_cols.append(cols)
            indices = [[int(col_sites[c]) for c in row] for row in cols]
            info[t.name] = {
                "ref_indx": 0,
                "size": t.size,
                "max_cluster_dia": 0.5 * cell.a * math.sqrt(t.dia2),
                "symm_group": 0,
                "name": t.name,
                "descriptor": "%s_%d_body_d2_%d" % (cell.kind, t.size, t.dia2),
                "indices": indices,
                "order": [list(o) for o in t.order],
                "equiv_sites": [list(g) for g in t.equiv_sites],
            }
        self.cluster_info = [info]
        self._trans_list = None

    @property
    def trans_matrix(self):
        """Sparse translation matrix: one dict ``{column site: site}`` per row."""
        if self._trans_list is None:
            cols = self.column_sites.tolist()
            self._trans_list = [dict(zip(cols, row)) for row in self.table.tolist()]
        return self._trans_list

    def symbol_ids(self, symbols: Sequence[str]) -> np.ndarray:
        lut = {s: i for i, s in enumerate(self.unique_elements)}
        return np.array([lut[s] for s in symbols], dtype=np.int8)

    def bf_table(self) -> np.ndarray:
        """bf[b, id] as in ``cpp/src/basis_function.cpp:5-19``."""
        out = np.zeros((len(self.basis_functions), self.num_unique_elements))
        for b, d in enumerate(self.basis_functions):
            for s, v in d.items():
                out[b, self.unique_elements.index(s)] = v
        return out


class BackgroundSettings:
    """Settings of a supercell with an inert second sublattice (background sites).

    Rocksalt-like: the active sublattice is ``base`` (an FCC supercell of N sites,
    indices 0..N-1, all clusters among them) and N background sites N..2N-1
    hold ``background_symbol`` (e.g. O) that never moves and belongs to no
    cluster (``ignore_background_atoms``; tests/test_sgc_mc.py:140-191 of the
    reference runs that case with a ``FixedElement`` constraint).  Background
    sites count in N (the singlet increment and the energy scale use the total,
    ce_updater.cpp:366-371, 236-242) and have no translation-symmetry group.
    Their rows of the translation matrix are empty dicts (the reference skips
    background rows, ce_updater.cpp:925-927); the packed table maps them onto
    themselves.
    """

    def __init__(self, base, background_symbol: str = "O"):
        n = base.n_sites
        self.base = base
        self.cell = base.cell
        self.cset = base.cset
        self.unique_elements = list(base.unique_elements)
        self.num_unique_elements = base.num_unique_elements
        self.basis_functions = base.basis_functions
        self.cluster_info = base.cluster_info
        self.background_symbol = background_symbol
        self.n_sites = 2 * n
        self.index_by_trans_symm = [list(grp) for grp in base.index_by_trans_symm]  # the active sites' groups
        self.background_indices = list(range(n, 2 * n))
        self.column_sites = base.column_sites
        bg = np.arange(n, 2 * n, dtype=np.int32)
        self.table = np.vstack([base.table, np.repeat(bg[:, None], base.table.shape[1], axis=1)]).astype(np.int32)
        self._trans_list = None

    @property
    def trans_matrix(self):
        if self._trans_list is None:
            self._trans_list = list(self.base.trans_matrix) + [{} for _ in range(self.n_sites // 2)]
        return self._trans_list

    def symbols_with_background(self, active_symbols: Sequence[str]) -> List[str]:
        """Atom symbols of the whole cell: the active sites' symbols, then the background symbol."""
        return list(active_symbols) + [self.background_symbol] * (self.n_sites // 2)


def with_background(settings, background_symbol: str = "O") -> BackgroundSettings:
    return BackgroundSettings(settings, background_symbol)


def fcc_settings(L: int, pair_shells: int, triplet_shells: int, quad_shells: int,
                 symbols: Sequence[str], a: float = 4.05) -> Settings:
    cset = fcc_cluster_set(pair_shells, triplet_shells, quad_shells, len(symbols))
    return Settings(FCCSupercell(L, a), cset, symbols)


def cubic_settings(kind: str, L: int, pair_shells: int, triplet_shells: int, quad_shells: int,
                   symbols: Sequence[str], a: float = 4.05) -> Settings:
    """Settings of an ``L^3``-cube supercell of the cubic Bravais lattice ``kind`` (fcc, bcc, sc).

    The reference's tests build BCC and SC cells through CLEASE
    (tests/test_CE_updater.py:21, 206-228); one translation-symmetry group.
    """
    cset = fcc_cluster_set(pair_shells, triplet_shells, quad_shells, len(symbols), kind)
    return Settings(CubicSupercell(L, a, kind), cset, symbols)


def seeded_ecis(cset: ClusterSet, seed: int, c0: float = -3.0, singlet_sigma: float = 0.05,
                pair_sigma: float = 0.02, triplet_sigma: float = 0.005, quad_sigma: float = 0.002) -> Dict[str, float]:
    """ECIs drawn as in the benchmark recipes.

    c0 fixed; singlets N(0, singlet_sigma); pairs N(0, pair_sigma / shell) where
    shell is the 1-based neighbour shell of the pair; triplets and quadruplets
    N(0, sigma).  Drawn in sorted-name order from ``numpy.random.default_rng(seed)``.
    """
    rng = np.random.default_rng(seed)
    eci: Dict[str, float] = {}
    for e in cset.eci_names:
        if e.kind == "c0":
            eci[e.name] = float(c0)
        elif e.kind == "c1":
            eci[e.name] = float(rng.normal(0.0, singlet_sigma))
        else:
            t = cset.types[e.cluster]
            if t.size == 2:
                shell = int(t.name.split("_")[1][1:]) + 1
                eci[e.name] = float(rng.normal(0.0, pair_sigma / shell))
            elif t.size == 3:
                eci[e.name] = float(rng.normal(0.0, triplet_sigma))
            else:
                eci[e.name] = float(rng.normal(0.0, quad_sigma))
    return eci


# ---------------------------------------------------------------------------
# Several translation-symmetry groups: the FCC lattice under the symmetry of
# its L1_2 (Cu3Au-type) ordering, space group Pm-3m.  Its translations are the
# cubic lattice vectors (even vectors in half-lattice units) and its point
# group is O_h about a cube corner, so the four sites of the conventional cube
# fall into four translation classes: the corner sublattice and three face
# sublattices.  The reference takes such settings from CLEASE (one
# ``cluster_info`` dict and one ``ref_indx`` per group; its tests build a
# four-group crystal in tests/helper_functions.py:8-27) and keeps one cluster
# list per group (cpp/src/ce_updater.cpp:115-148): a cluster type seen from
# several groups keeps one name, and ``M_prefix`` sums its sub-cluster counts
# over the groups.


def _canonical_key_sg(points: np.ndarray, tmod: int) -> Tuple:
    """Key of a point set's orbit under translations by ``tmod * Z^3`` and O_h about the origin."""
    best = None
    for g in _OH:
        img = points @ g.T
        for q in img:
            t = q - np.mod(q, tmod)
            key = tuple(sorted(map(tuple, (img - t).tolist())))
            if best is None or key < best:
                best = key
    return best


def _space_group_maps(src: np.ndarray, dst: np.ndarray, tmod: int):
    """Yield ``mapping`` (index of src point -> index of dst point) of every space-group element src -> dst."""
    dst_set = {tuple(p): q for q, p in enumerate(dst.tolist())}
    n = len(src)
    for g in _OH:
        img = src @ g.T
        for p0 in dst:
            t = p0 - img[0]
            if np.any(np.mod(t, tmod)):
                continue
            mapping = [dst_set.get(tuple(p)) for p in (img + t).tolist()]
            if None in mapping or len(set(mapping)) != n:
                continue
            yield mapping


def _map_onto_sg(points: np.ndarray, proto: np.ndarray, tmod: int) -> List[int]:
    """``order[q]`` = index into ``points`` of the site that prototype position ``q`` corresponds to."""
    for mapping in _space_group_maps(points, proto, tmod):
        order = [0] * len(points)
        for idx, q in enumerate(mapping):
            order[q] = idx
        return order
    raise RuntimeError("sub-cluster is not equivalent to its prototype")


def _equiv_sites_sg(proto: np.ndarray, tmod: int) -> List[List[int]]:
    """Orbits (size >= 2) of the prototype's stabiliser in the space group, on its positions."""
    n = len(proto)
    parent = list(range(n))

    def find(a):
        while parent[a] != a:
            parent[a] = parent[parent[a]]
            a = parent[a]
        return a

    for mapping in _space_group_maps(proto, proto, tmod):
        for q in range(n):
            a, b = find(q), find(mapping[q])
            if a != b:
                parent[a] = b
    groups: Dict[int, List[int]] = {}
    for q in range(n):
        groups.setdefault(find(q), []).append(q)
    return [sorted(gq) for gq in sorted(groups.values()) if len(gq) >= 2]


@dataclass
class SublatticeClusterType:
    """One cluster type (space-group orbit) with its sub-clusters per translation group."""

    name: str
    size: int
    dia2: int
    prototype: np.ndarray
    equiv_sites: List[List[int]]
    members: List[List[np.ndarray]]  # [group] -> list of (size-1, 3) member positions around the group's reference
    orders: List[List[List[int]]]   # [group] -> canonical order of [ref] + members


def enumerate_l12_cluster_types(pair_shells: int, triplet_shells: int,
                                quad_shells: int) -> List[SublatticeClusterType]:
    """Cluster types of the FCC lattice under Pm-3m, seen from the four sublattice references.

    The reference of group b is basis site b of the cube at the origin.  Size
    cut-offs follow ``enumerate_cluster_types`` (every pairwise distance of a
    cluster within the given shell radius).
    """
    max_shell = max(pair_shells, triplet_shells, quad_shells, 1)
    shells = fcc_shell_vectors(max_shell)
    radii = [int((s[0] * s[0]).sum()) for s in shells]
    n_groups = len(_FCC_BASIS)
    types: List[SublatticeClusterType] = []
    for size, n_shells in ((2, pair_shells), (3, triplet_shells), (4, quad_shells)):
        if n_shells <= 0:
            continue
        cutoff = radii[n_shells - 1]
        vecs = np.concatenate(shells[:n_shells])
        found: Dict[Tuple, SublatticeClusterType] = {}
        for b, ref in enumerate(_FCC_BASIS):
            for combo in itertools.combinations(range(len(vecs)), size - 1):
                pts = np.vstack([ref[None, :], ref[None, :] + vecs[list(combo)]])
                diff = pts[:, None, :] - pts[None, :, :]
                d2 = (diff * diff).sum(axis=2)
                if d2.max() > cutoff:
                    continue
                key = _canonical_key_sg(pts, 2)
                ct = found.get(key)
                if ct is None:
                    proto = np.array(key, dtype=np.int64)
                    ct = SublatticeClusterType("", size, int(d2.max()), proto, _equiv_sites_sg(proto, 2),
                                               [[] for _ in range(n_groups)], [[] for _ in range(n_groups)])
                    found[key] = ct
                ct.members[b].append(pts[1:].copy())
                ct.orders[b].append(_map_onto_sg(pts, ct.prototype, 2))
        cts = sorted(found.values(),
                     key=lambda c: (c.dia2, sum(len(m) for m in c.members), c.prototype.tolist()))
        dias = sorted({c.dia2 for c in cts})
        variant: Dict[int, int] = {}
        for c in cts:
            di = dias.index(c.dia2)
            v = variant.get(di, 0)
            variant[di] = v + 1
            c.name = "c%d_d%04d_%d" % (size, di, v)
            types.append(c)
    return types


class SublatticeSettings:
    """Settings object of an FCC supercell with several translation-symmetry groups (L1_2 symmetry).

    Same attribute formats as ``Settings``.  ``index_by_trans_symm`` lists the
    sites of each group; ``cluster_info`` holds one dict per group whose
    ``indices`` are the member sites of the sub-clusters around the group's
    reference site; the translation matrix maps a column site j of site i's
    group to j + (position of i - position of the group's reference).

    ``group_of_basis`` assigns the four sublattices to groups.  The default
    (0, 1, 2, 3) gives the four translation classes.  Merging sublattices,
    e.g. (0, 1, 1, 1), gives groups of unequal size whose members share the
    cluster list of the group's first sublattice (carried over by an FCC
    translation): settings the reference accepts, which exercise its
    per-group normalisation ``M_prefix * N_group`` (ce_updater.cpp:400-402)
    with N_group differing between groups.
    """

    def __init__(self, cell: FCCSupercell, types: List[SublatticeClusterType], symbols: Sequence[str],
                 group_of_basis: Sequence[int] = (0, 1, 2, 3)):
        self.cell = cell
        self.unique_elements = sorted(symbols)
        self.num_unique_elements = len(self.unique_elements)
        self.cset = ClusterSet(types, self.num_unique_elements - 1)
        if self.num_unique_elements == 2:
            self.basis_functions = binary_basis(self.unique_elements)
        elif self.num_unique_elements == 3:
            self.basis_functions = ternary_basis(self.unique_elements)
        else:
            raise ValueError("only binary and ternary alloys are generated")
        n = cell.n_sites
        gob = np.asarray(group_of_basis, dtype=np.int64)
        n_groups = int(gob.max()) + 1
        if sorted(set(gob.tolist())) != list(range(n_groups)) or len(gob) != len(_FCC_BASIS):
            raise ValueError("group_of_basis must map the four sublattices onto groups 0..n-1")
        ref_basis = [int(np.nonzero(gob == q)[0][0]) for q in range(n_groups)]  # a group's first sublattice
        self.n_sites = n
        basis_of = np.arange(n) % len(_FCC_BASIS)  # site order: 4 basis sites per cube
        self.site_basis = basis_of
        self.index_by_trans_symm = [np.nonzero(gob[basis_of] == q)[0].tolist() for q in range(n_groups)]
        self.background_indices: List[int] = []
        info: List[Dict[str, dict]] = []
        col_set = set()
        for b in ref_basis:
            d: Dict[str, dict] = {}
            for t in types:
                if not t.members[b]:
                    continue
                idx = [cell.index_of(m).astype(np.int64).tolist() for m in t.members[b]]
                for row, m in zip(idx, t.members[b]):
                    if len(set(row)) != len(row) or b in row:
                        raise ValueError("supercell too small: cluster members alias onto the same site")
                col_set.update(x for row in idx for x in row)
                d[t.name] = {
                    "ref_indx": b,
                    "size": t.size,
                    "max_cluster_dia": 0.5 * cell.a * math.sqrt(t.dia2),
                    "symm_group": b,
                    "name": t.name,
                    "descriptor": "l12_%d_body_d2_%d" % (t.size, t.dia2),
                    "indices": idx,
                    "order": [list(o) for o in t.orders[b]],
                    "equiv_sites": [list(g) for g in t.equiv_sites],
                }
            info.append(d)
        self.cluster_info = info
        cols = np.array(sorted(col_set), dtype=np.int64)
        self.column_sites = cols
        # every offset that a group's sub-clusters reach must land on a distinct site
        for b in ref_basis:
            offs = {tuple((m - _FCC_BASIS[b]).tolist()) for t in types for ms in t.members[b] for m in ms}
            sites = cell.index_of(np.array(sorted(offs), dtype=np.int64) + _FCC_BASIS[b])
            if len(set(sites.tolist())) != len(sites):
                raise ValueError("supercell too small: neighbour offsets alias onto the same site")
        ref_site = np.array(ref_basis, dtype=np.int64)[gob[basis_of]]  # reference site (cube 0) of i's group
        shift = cell.positions - cell.positions[ref_site]  # position of i - position of its group's reference
        self.table = cell.index_of(cell.positions[cols][None, :, :] + shift[:, None, :]).astype(np.int32)
        self._trans_list = None

    trans_matrix = Settings.trans_matrix
    symbol_ids = Settings.symbol_ids
    bf_table = Settings.bf_table


def l12_settings(L: int, pair_shells: int, triplet_shells: int, quad_shells: int,
                 symbols: Sequence[str], a: float = 4.05,
                 group_of_basis: Sequence[int] = (0, 1, 2, 3)) -> SublatticeSettings:
    """FCC supercell of ``L^3`` cubes with the sublattices as translation-symmetry groups."""
    return SublatticeSettings(FCCSupercell(L, a), enumerate_l12_cluster_types(pair_shells, triplet_shells,
                                                                              quad_shells), symbols, group_of_basis)


# ---------------------------------------------------------------------------
# Hexagonal close-packed crystals.  Positions are integer coordinates in sixths
# of the hexagonal cell vectors a1 = a (1, 0, 0), a2 = a (-1/2, sqrt(3)/2, 0),
# a3 = (0, 0, c) with the ideal c / a = sqrt(8/3); the two atoms of the cell sit
# at (0, 0, 0) and (2, 4, 3).  Squared distances are Q(u, v, w) = 3 (u^2 - uv +
# v^2) + 8 w^2 = 108 |r|^2 / a^2 (nearest neighbours: Q = 108).  The space group
# P6_3/mmc is non-symmorphic: its operations pair the 24 hexagonal point
# operations with fractional translations, and the two atoms of the cell are
# related by a screw, not by a lattice translation, so an HCP supercell has two
# translation-symmetry groups that share cluster names (CLEASE's convention for
# HCP, which the reference takes as given).

_HCP_BASIS = np.array([(0, 0, 0), (2, 4, 3)], dtype=np.int64)
_HEX_PERIOD = 6


def _hex_metric(v: np.ndarray) -> np.ndarray:
    v = np.asarray(v, dtype=np.int64)
    return 3 * (v[..., 0] ** 2 - v[..., 0] * v[..., 1] + v[..., 1] ** 2) + 8 * v[..., 2] ** 2


def _hex_point_group() -> List[np.ndarray]:
    """The 24 operations of 6/mmm as integer matrices on lattice coordinates (closure of 6, m, m_z)."""
    rot = np.array([[1, -1, 0], [1, 0, 0], [0, 0, 1]], dtype=np.int64)  # a1 -> a1 + a2, a2 -> -a1
    swap = np.array([[0, 1, 0], [1, 0, 0], [0, 0, 1]], dtype=np.int64)
    zflip = np.diag([1, 1, -1]).astype(np.int64)
    group = {tuple(np.eye(3, dtype=np.int64).ravel())}
    frontier = list(group)
    while frontier:
        nxt = []
        for g in frontier:
            G = np.array(g).reshape(3, 3)
            for h in (rot, swap, zflip):
                key = tuple((h @ G).ravel())
                if key not in group:
                    group.add(key)
                    nxt.append(key)
        frontier = nxt
    return [np.array(g).reshape(3, 3) for g in sorted(group)]


def _hcp_space_group() -> List[Tuple[np.ndarray, np.ndarray]]:
    """(R, t) with R a point operation and t a translation (sixths) mapping the atom set onto itself."""
    basis = {tuple(b) for b in _HCP_BASIS.tolist()}
    ops = []
    for R in _hex_point_group():
        img = _HCP_BASIS @ R.T
        for t in itertools.product(range(_HEX_PERIOD), repeat=3):
            moved = {tuple(np.mod(p + np.array(t), _HEX_PERIOD).tolist()) for p in img}
            if moved == basis:
                ops.append((R, np.array(t, dtype=np.int64)))
    return ops


_HCP_OPS = None


def _hcp_ops():
    global _HCP_OPS
    if _HCP_OPS is None:
        _HCP_OPS = _hcp_space_group()
    return _HCP_OPS


def _hcp_canonical_key(points: np.ndarray) -> Tuple:
    best = None
    for R, t in _hcp_ops():
        img = points @ R.T + t
        for q in img:
            shift = q - np.mod(q, _HEX_PERIOD)
            key = tuple(sorted(map(tuple, (img - shift).tolist())))
            if best is None or key < best:
                best = key
    return best


def _hcp_maps(src: np.ndarray, dst: np.ndarray):
    dst_set = {tuple(p): q for q, p in enumerate(dst.tolist())}
    n = len(src)
    for R, t in _hcp_ops():
        img = src @ R.T + t
        for p0 in dst:
            shift = p0 - img[0]
            if np.any(np.mod(shift, _HEX_PERIOD)):
                continue
            mapping = [dst_set.get(tuple(p)) for p in (img + shift).tolist()]
            if None in mapping or len(set(mapping)) != n:
                continue
            yield mapping


def _hcp_order(points: np.ndarray, proto: np.ndarray) -> List[int]:
    for mapping in _hcp_maps(points, proto):
        order = [0] * len(points)
        for idx, q in enumerate(mapping):
            order[q] = idx
        return order
    raise RuntimeError("sub-cluster is not equivalent to its prototype")


def _hcp_equiv_sites(proto: np.ndarray) -> List[List[int]]:
    n = len(proto)
    parent = list(range(n))

    def find(a):
        while parent[a] != a:
            parent[a] = parent[parent[a]]
            a = parent[a]
        return a

    for mapping in _hcp_maps(proto, proto):
        for q in range(n):
            a, b = find(q), find(mapping[q])
            if a != b:
                parent[a] = b
    groups: Dict[int, List[int]] = {}
    for q in range(n):
        groups.setdefault(find(q), []).append(q)
    return [sorted(gq) for gq in sorted(groups.values()) if len(gq) >= 2]


def hcp_shell_radii(max_shell: int) -> List[int]:
    """Squared distances Q of the first neighbour shells of an HCP site (108 = nearest neighbours)."""
    rng = np.arange(-4, 5)
    cells = np.array(list(itertools.product(rng, rng, rng)), dtype=np.int64) * _HEX_PERIOD
    pts = (cells[:, None, :] + _HCP_BASIS[None, :, :]).reshape(-1, 3)
    q = np.unique(_hex_metric(pts))
    return [int(x) for x in q[q > 0][:max_shell]]


def enumerate_hcp_cluster_types(pair_shells: int, triplet_shells: int,
                                quad_shells: int) -> List[SublatticeClusterType]:
    """Cluster types of the HCP crystal (space group P6_3/mmc) seen from its two atoms."""
    max_shell = max(pair_shells, triplet_shells, quad_shells, 1)
    radii = hcp_shell_radii(max_shell)
    rng = np.arange(-4, 5)
    cells = np.array(list(itertools.product(rng, rng, rng)), dtype=np.int64) * _HEX_PERIOD
    all_pts = (cells[:, None, :] + _HCP_BASIS[None, :, :]).reshape(-1, 3)
    n_groups = len(_HCP_BASIS)
    types: List[SublatticeClusterType] = []
    for size, n_shells in ((2, pair_shells), (3, triplet_shells), (4, quad_shells)):
        if n_shells <= 0:
            continue
        cutoff = radii[n_shells - 1]
        found: Dict[Tuple, SublatticeClusterType] = {}
        for b, ref in enumerate(_HCP_BASIS):
            d = _hex_metric(all_pts - ref)
            nbrs = all_pts[(d > 0) & (d <= cutoff)]
            nbrs = nbrs[np.lexsort(nbrs.T[::-1])]
            for combo in itertools.combinations(range(len(nbrs)), size - 1):
                pts = np.vstack([ref[None, :], nbrs[list(combo)]])
                diff = pts[:, None, :] - pts[None, :, :]
                dia2 = int(_hex_metric(diff).max())
                if dia2 > cutoff:
                    continue
                key = _hcp_canonical_key(pts)
                ct = found.get(key)
                if ct is None:
                    proto = np.array(key, dtype=np.int64)
                    ct = SublatticeClusterType("", size, dia2, proto, _hcp_equiv_sites(proto),
                                               [[] for _ in range(n_groups)], [[] for _ in range(n_groups)])
                    found[key] = ct
                ct.members[b].append(pts[1:].copy())
                ct.orders[b].append(_hcp_order(pts, ct.prototype))
        cts = sorted(found.values(), key=lambda c: (c.dia2, sum(len(m) for m in c.members), c.prototype.tolist()))
        dias = sorted({c.dia2 for c in cts})
        variant: Dict[int, int] = {}
        for c in cts:
            di = dias.index(c.dia2)
            v = variant.get(di, 0)
            variant[di] = v + 1
            c.name = "c%d_d%04d_%d" % (size, di, v)
            types.append(c)
    return types


class HCPSupercell:
    """``L x L x Lz`` hexagonal cells of an HCP crystal (2 sites per cell), cell-major site order."""

    def __init__(self, L: int, Lz: int, a: float = 3.21):
        if L < 1 or Lz < 1:
            raise ValueError("supercell size must be positive")
        self.L, self.Lz, self.a = int(L), int(Lz), float(a)
        self.c = self.a * math.sqrt(8.0 / 3.0)
        self.period = np.array([L, L, Lz], dtype=np.int64) * _HEX_PERIOD
        cells = np.array(list(itertools.product(range(L), range(L), range(Lz))), dtype=np.int64)
        self.positions = ((_HEX_PERIOD * cells)[:, None, :] + _HCP_BASIS[None, :, :]).reshape(-1, 3)
        self.n_sites = len(self.positions)

    def index_of(self, pos: np.ndarray) -> np.ndarray:
        p = np.mod(pos, self.period)
        cell = p // _HEX_PERIOD
        rem = p % _HEX_PERIOD
        b = np.full(p.shape[:-1], -1, dtype=np.int64)
        for i, base in enumerate(_HCP_BASIS.tolist()):
            b[(rem == base).all(-1)] = i
        if np.any(b < 0):
            raise ValueError("position is not an HCP site")
        return ((cell[..., 0] * self.L + cell[..., 1]) * self.Lz + cell[..., 2]) * len(_HCP_BASIS) + b

    def cartesian(self) -> np.ndarray:
        """Site positions in angstrom."""
        f = self.positions.astype(np.float64) / _HEX_PERIOD
        a1 = np.array([self.a, 0.0, 0.0])
        a2 = np.array([-0.5 * self.a, 0.5 * math.sqrt(3.0) * self.a, 0.0])
        a3 = np.array([0.0, 0.0, self.c])
        return f[:, :1] * a1 + f[:, 1:2] * a2 + f[:, 2:3] * a3


class HCPSettings:
    """Settings object of an HCP supercell: two translation-symmetry groups (the two atoms of the
    hexagonal cell), one ``cluster_info`` dict per group; same attribute formats as ``Settings``."""

    def __init__(self, cell: HCPSupercell, types: List[SublatticeClusterType], symbols: Sequence[str]):
        self.cell = cell
        self.unique_elements = sorted(symbols)
        self.num_unique_elements = len(self.unique_elements)
        self.cset = ClusterSet(types, self.num_unique_elements - 1)
        if self.num_unique_elements == 2:
            self.basis_functions = binary_basis(self.unique_elements)
        elif self.num_unique_elements == 3:
            self.basis_functions = ternary_basis(self.unique_elements)
        else:
            raise ValueError("only binary and ternary alloys are generated")
        n = cell.n_sites
        self.n_sites = n
        nb = len(_HCP_BASIS)
        basis_of = np.arange(n) % nb
        self.index_by_trans_symm = [np.nonzero(basis_of == b)[0].tolist() for b in range(nb)]
        self.background_indices: List[int] = []
        info: List[Dict[str, dict]] = []
        col_set = set()
        for b in range(nb):
            d: Dict[str, dict] = {}
            offs = set()
            for t in types:
                if not t.members[b]:
                    continue
                idx = [cell.index_of(mm).astype(np.int64).tolist() for mm in t.members[b]]
                for row in idx:
                    if len(set(row)) != len(row) or b in row:
                        raise ValueError("supercell too small: cluster members alias onto the same site")
                for mm in t.members[b]:
                    offs.update(tuple(x) for x in (mm - _HCP_BASIS[b]).tolist())
                col_set.update(x for row in idx for x in row)
                d[t.name] = {
                    "ref_indx": b,
                    "size": t.size,
                    "max_cluster_dia": cell.a * math.sqrt(t.dia2 / 108.0),
                    "symm_group": b,
                    "name": t.name,
                    "descriptor": "hcp_%d_body_q_%d" % (t.size, t.dia2),
                    "indices": idx,
                    "order": [list(o) for o in t.orders[b]],
                    "equiv_sites": [list(g) for g in t.equiv_sites],
                }
            sites = cell.index_of(np.array(sorted(offs), dtype=np.int64) + _HCP_BASIS[b])
            if len(set(sites.tolist())) != len(sites):
                raise ValueError("supercell too small: neighbour offsets alias onto the same site")
            info.append(d)
        self.cluster_info = info
        cols = np.array(sorted(col_set), dtype=np.int64)
        self.column_sites = cols
        shift = cell.positions - cell.positions[basis_of]  # a lattice translation (same atom of the cell)
        self.table = cell.index_of(cell.positions[cols][None, :, :] + shift[:, None, :]).astype(np.int32)
        self._trans_list = None

    trans_matrix = Settings.trans_matrix
    symbol_ids = Settings.symbol_ids
    bf_table = Settings.bf_table


def hcp_settings(L: int, Lz: int, pair_shells: int, triplet_shells: int, quad_shells: int,
                 symbols: Sequence[str], a: float = 3.21) -> HCPSettings:
    """HCP supercell of ``L x L x Lz`` hexagonal cells (ideal c / a) with the given cluster recipe."""
    return HCPSettings(HCPSupercell(L, Lz, a), enumerate_hcp_cluster_types(pair_shells, triplet_shells, quad_shells),
                       symbols)
