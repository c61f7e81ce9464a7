"""Move constraints of the Monte Carlo drivers (cemc/mcmc/mc_constraints.py), checked on the device.

The reference asks every constraint object whether a proposed move is legal
and redraws the move until all agree (montecarlo.py:976-988).  The constraint
classes it ships decide from each change ``(site, old symbol, new symbol)``
alone (``PairConstraint``, as shipped, accepts every move), so the device holds
them as two masks per chain and runs the same redraw loop inside the fused kernel:

* ``frozen``: species whose sites may not change.  ``FixedElement`` compares
  the change's old symbol with its element (mc_constraints.py:95-107; the other
  comparison it makes is against the site index and never matches), so a move
  that would change a site holding the element is illegal, a move that puts the
  element on a site is not;
* ``allow[site]``: species that may be placed on the site.
  ``ConstrainElementByTag`` allows the elements listed for the site's tag
  (175-190); ``FixEdgeLayers`` allows nothing on the sites near the cell's
  faces (110-172).

A change is legal when its old species is not frozen and its new species is
allowed at its site; a move is legal when all its changes are.  The classes
below keep the reference's constructors and ``__call__`` (host-side check of a
list of changes, used by ``insert_symbol``); ``device_masks`` also accepts the
reference's own objects of these classes.
"""
from __future__ import annotations

from typing import Optional, Sequence, Tuple

import numpy as np


class MCConstraint:
    """Base class: a callable returning True when the proposed changes are legal."""

    def __init__(self):
        self.name = "GenericConstraint"

    def __call__(self, system_changes) -> bool:
        return True


class FixedElement(MCConstraint):
    """Sites holding ``element`` never change (mc_constraints.py:83-107)."""

    def __init__(self, element=None):
        super().__init__()
        self.name = "FixedElement"
        self.element = element

    def __call__(self, system_changes) -> bool:
        for change in system_changes:
            if change[0] == self.element or change[1] == self.element:
                return False
        return True


class ConstrainElementByTag(MCConstraint):
    """Only the elements listed for a site's tag may be placed on it (mc_constraints.py:175-190).

    ``atoms`` items need ``index`` and ``tag``; ``element_by_tag[tag]`` lists the allowed symbols.
    """

    def __init__(self, atoms=None, element_by_tag=()):
        super().__init__()
        self.name = "ConstrainElementByTag"
        self.element_by_tag = list(element_by_tag)
        self.allowed_elements = self._get_allowed_elements(atoms)

    def _get_allowed_elements(self, atoms):
        elems = [[] for _ in range(len(atoms))]
        for atom in atoms:
            elems[atom.index] = self.element_by_tag[atom.tag]
        return elems

    def __call__(self, system_changes) -> bool:
        for change in system_changes:
            if change[2] not in self.allowed_elements[change[0]]:
                return False
        return True


class FixEdgeLayers(MCConstraint):
    """Sites within ``thickness`` of a face of the cell never change (mc_constraints.py:110-172).

    ``atoms`` needs ``get_cell()`` (3 x 3 rows = cell vectors) and ``get_positions()``.  For each
    pair of cell vectors the layer is the slab between the planes (through the origin side and
    through the opposite face) shifted inward by ``thickness`` and outward by a tenth of it.
    """

    def __init__(self, thickness=4.0, atoms=None):
        super().__init__()
        self.name = "FixEdgeLayers"
        self.cell = np.asarray(atoms.get_cell(), dtype=np.float64)
        self.thickness = float(thickness)
        self.pos = np.asarray(atoms.get_positions(), dtype=np.float64)
        self.planes = self._init_planes()

    def _init_planes(self):
        planes = []
        for t, (i, j) in zip((2, 1, 0), ((0, 1), (0, 2), (1, 2))):
            normal = np.cross(self.cell[i], self.cell[j])
            normal = normal / np.linalg.norm(normal)
            unit = self.cell[t] / np.linalg.norm(self.cell[t])
            planes.append(((normal, -0.1 * self.thickness * unit), (normal, unit * self.thickness)))
            planes.append(((normal, self.cell[t] + 0.1 * self.thickness * unit),
                           (normal, self.cell[t] - self.thickness * unit)))
        return planes

    @staticmethod
    def _signed(plane, x):
        normal, point = plane
        return float(np.dot(normal, x - point))

    def _is_between_any(self, x) -> bool:
        for p1, p2 in self.planes:
            if np.sign(self._signed(p1, x) * self._signed(p2, x)) < 0:
                return True
        return False

    def fixed_sites(self) -> np.ndarray:
        return np.array([i for i in range(len(self.pos)) if self._is_between_any(self.pos[i])], dtype=np.int64)

    def __call__(self, system_changes) -> bool:
        for change in system_changes:
            if self._is_between_any(self.pos[change[0]]):
                return False
        return True


class PairConstraint(MCConstraint):
    """"Two elements may not share a pair cluster" (mc_constraints.py:24-80), as the reference ships it.

    The reference validates its arguments, then overwrites ``cluster_name`` with the element list
    and hands ``str(elements)`` (e.g. "['Al', 'Mg']") to the C++ check as the cluster name
    (mc_constraints.py:55-63); ``CEUpdater::get_clusters`` finds no cluster of that name
    (ce_updater.cpp:879-889), so ``PairConstraint::elems_in_pair`` scans nothing and returns false
    (pair_constraint.cpp:14-44) and every move is legal.  This class keeps the argument checks and
    that verdict; on the device it adds no mask.
    """

    def __init__(self, calc=None, cluster_name=None, elements=None):
        super().__init__()
        self.name = "PairConstraint"
        if calc is None:
            raise ValueError("No calculator object given!")
        if cluster_name is None:
            raise ValueError("No cluster name given!")
        if elements is None:
            raise ValueError("No element list given!")
        size = int(cluster_name[1])
        if size != 2:
            raise ValueError("Only pair clusters given.Given cluster has {} elements".format(size))
        if len(elements) != 2:
            raise ValueError("The elements list has to consist of exactly two elements")
        self.calc = calc
        self.cluster_name = elements  # as the reference does (mc_constraints.py:59)
        self.elements = elements

    def __call__(self, system_changes) -> bool:
        return True


def device_masks(constraint, symbols: Sequence[str], n_sites: int) -> Tuple[Optional[np.ndarray], int]:
    """(allow, frozen) of one constraint: allow uint8 [n_sites] (bit s = species s may be placed on
    the site) or None for no restriction; frozen bit s = a site holding species s may not change.

    ``symbols``: the model's species in id order.  Accepts these classes and the reference's
    objects of the same names; anything else raises ``NotImplementedError``.
    """
    sym_id = {s: i for i, s in enumerate(symbols)}
    kind = type(constraint).__name__
    if kind == "FixedElement" and hasattr(constraint, "element"):
        # an element the model does not know (a background species) never appears in a change
        return None, (1 << sym_id[constraint.element]) if constraint.element in sym_id else 0
    if kind == "ConstrainElementByTag" and hasattr(constraint, "allowed_elements"):
        allowed = constraint.allowed_elements
        if len(allowed) != n_sites:
            raise ValueError("ConstrainElementByTag lists %d sites, the cell has %d" % (len(allowed), n_sites))
        allow = np.zeros(n_sites, dtype=np.uint8)
        for i, elems in enumerate(allowed):
            for e in elems:
                if e in sym_id:
                    allow[i] |= np.uint8(1 << sym_id[e])
        return allow, 0
    if kind == "PairConstraint":
        return None, 0  # accepts every move as shipped (see PairConstraint)
    if kind == "FixEdgeLayers" and hasattr(constraint, "_is_between_any") and hasattr(constraint, "pos"):
        allow = np.full(n_sites, 0xFF, dtype=np.uint8)
        pos = np.asarray(constraint.pos)
        for i in range(n_sites):
            if constraint._is_between_any(pos[i]):
                allow[i] = 0
        return allow, 0
    raise NotImplementedError(
        "constraint %s has no device form: the GPU drivers run FixedElement, ConstrainElementByTag, "
        "FixEdgeLayers and PairConstraint" % kind)


def combined_masks(constraints, symbols: Sequence[str], n_sites: int) -> Tuple[Optional[np.ndarray], int]:
    """AND of the allow masks and OR of the frozen masks of several constraints."""
    allow, frozen = None, 0
    for c in constraints:
        a, f = device_masks(c, symbols, n_sites)
        if a is not None:
            allow = a.copy() if allow is None else (allow & a)
        frozen |= int(f)
    return allow, frozen
