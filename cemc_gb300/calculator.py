"""Drop-in cluster-expansion calculator backed by the GPU library.

``CE`` keeps the reference calculator's interface (cemc/ce_calculator.py:136-617):
``calculate(atoms, ["energy"], system_changes)``, ``get_energy``, ``get_cf``,
``update_cf``, ``undo_changes``, ``clear_history``, ``update_ecis``,
``get_singlets``, ``set_symbols``, ``set_composition``, ``singlet2comp``,
``copy``, ``save``/``load``.  Each call is one kernel launch on the
configuration resident on the GPU (``DeviceUpdater``), which replaces the
reference's ``PyCEUpdater`` / ``CEUpdater`` (cemc/cpp_ext/pyce_updater.pyx:5-60).

The undo buffer mirrors the reference's ``CFHistoryTracker`` semantics
(cpp/src/cf_history_tracker.cpp:46-149): changes since the last
``clear_history`` can be undone; the correlation functions return to their
values at that point.  Like the reference, symbol changes are mirrored into
the ``atoms`` object (ce_updater.cpp:338-347, 435-446).
"""
from __future__ import annotations

import ctypes as C
import json
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np
import torch

from . import _lib
from .engine import Geometry, _ptr, _stream_ptr
from .tables import CEModel


class SelfInteractionError(Exception):
    """Same sites appear twice in one cluster (cemc/ce_calculator.py:20-21, 153-157)."""


_GEOMETRY_CACHE: Dict[Tuple[int, Tuple[str, ...], str], Tuple[CEModel, Geometry]] = {}


def model_and_geometry(settings, eci_names: Sequence[str], device="cuda") -> Tuple[CEModel, Geometry]:
    """Device tables for (settings, ECI names), built once and shared by every calculator/chain."""
    key = (id(settings), tuple(sorted(eci_names)), str(device))
    hit = _GEOMETRY_CACHE.get(key)
    if hit is not None and hit[0] is not None and getattr(hit[0], "_settings_ref", None) is settings:
        return hit
    model = CEModel(settings, list(eci_names))
    model._settings_ref = settings
    geo = Geometry(model, device)
    _GEOMETRY_CACHE[key] = (model, geo)
    return model, geo


class DeviceUpdater:
    """One configuration resident on the GPU: occupation, correlation functions, energy, undo buffer."""

    def __init__(self, geo: Geometry, occ, eci, cf=None, stream=None):
        self.geo = geo
        self.model = geo.model
        dev = geo.device
        self.stream = stream
        self.occ_d = torch.as_tensor(np.asarray(occ, dtype=np.int8)).to(dev).contiguous()
        self.eci_d = torch.as_tensor(np.asarray(eci, dtype=np.float64)).to(dev).contiguous()
        self.cf_d = torch.zeros(self.model.n_eci, dtype=torch.float64, device=dev)
        self.energy_d = torch.zeros(1, dtype=torch.float64, device=dev)
        self.status_d = torch.zeros(1, dtype=torch.int32, device=dev)
        self.de_d = torch.zeros(1, dtype=torch.float64, device=dev)
        self.dcf_d = torch.zeros(self.model.n_eci, dtype=torch.float64, device=dev)
        if cf is None:
            self.recompute()
        else:
            self.cf_d.copy_(torch.as_tensor(np.asarray(cf, dtype=np.float64)))
            self._energy_from_cf()
        self.history: List[Tuple[int, int, int]] = []
        self._snap_cf = self.cf_d.clone()
        self._snap_energy = self.energy_d.clone()

    # -- device calls ----------------------------------------------------------
    def recompute(self):
        scratch = torch.empty(max(self.geo.scratch_doubles(1), 1), dtype=torch.float64, device=self.occ_d.device)
        _lib.check(self.geo.L.cemc_recompute(self.geo.handle, 1, _ptr(self.occ_d), _ptr(self.eci_d), _ptr(self.cf_d),
                                             _ptr(self.energy_d), _ptr(scratch), _stream_ptr(self.stream)))

    def _energy_from_cf(self):
        _lib.check(self.geo.L.cemc_energy(self.geo.handle, 1, _ptr(self.eci_d), _ptr(self.cf_d), _ptr(self.energy_d),
                                          _stream_ptr(self.stream)))

    def apply(self, changes: Sequence[Tuple[int, int, int]], record: bool = True):
        """Apply (site, old id, new id) changes in order (``cemc_apply_changes``)."""
        if not changes:
            return
        arr = np.asarray(changes, dtype=np.int64).reshape(-1, 3)
        if arr[:, 0].min() < 0 or arr[:, 0].max() >= self.model.n_sites:
            raise IndexError("site index out of range")
        if len(self.model.background) and np.isin(arr[:, 0], self.model.background).any():
            raise RuntimeError("Attempting to move a background atom!")
        dev = self.occ_d.device
        sites = torch.as_tensor(arr[:, 0].astype(np.int32)).to(dev)
        old = torch.as_tensor(arr[:, 1].astype(np.int8)).to(dev)
        new = torch.as_tensor(arr[:, 2].astype(np.int8)).to(dev)
        _lib.check(self.geo.L.cemc_apply_changes(self.geo.handle, _ptr(self.occ_d), _ptr(self.cf_d),
                                                 _ptr(self.energy_d), _ptr(self.eci_d), len(arr), _ptr(sites),
                                                 _ptr(old), _ptr(new), _ptr(self.status_d), _stream_ptr(self.stream)))
        st = int(self.status_d.item())
        if st == _lib.ERR_STATE:
            raise RuntimeError("The atom position tracker does not match the current state")
        if st:
            raise _lib.CemcError(st, "apply_changes failed")
        if record:
            self.history.extend((int(s), int(o), int(n)) for s, o, n in arr)

    def delta_swap(self, a: int, b: int):
        _lib.check(self.geo.L.cemc_delta_e(self.geo.handle, _ptr(self.occ_d), _ptr(self.eci_d), _lib.MOVE_SWAP, a, b,
                                           0, _ptr(self.de_d), _ptr(self.dcf_d), _stream_ptr(self.stream)))
        return float(self.de_d.item()), self.dcf_d.cpu().numpy()

    def delta_flip(self, a: int, new: int):
        _lib.check(self.geo.L.cemc_delta_e(self.geo.handle, _ptr(self.occ_d), _ptr(self.eci_d), _lib.MOVE_FLIP, a, -1,
                                           new, _ptr(self.de_d), _ptr(self.dcf_d), _stream_ptr(self.stream)))
        return float(self.de_d.item()), self.dcf_d.cpu().numpy()

    def set_eci(self, eci_vec):
        self.eci_d.copy_(torch.as_tensor(np.asarray(eci_vec, dtype=np.float64)))
        self._energy_from_cf()
        self._snap_energy = self.energy_d.clone()

    def set_occupation(self, occ):
        """Replace the whole occupation; correlation functions follow from the full recompute."""
        self.occ_d.copy_(torch.as_tensor(np.asarray(occ, dtype=np.int8)))
        self.recompute()

    # -- undo buffer -------------------------------------------------------------
    def clear(self):
        self.history.clear()
        self._snap_cf.copy_(self.cf_d)
        self._snap_energy.copy_(self.energy_d)

    def undo(self) -> List[Tuple[int, int, int]]:
        """Revert every change since ``clear``; returns the reverted changes (latest first)."""
        undone = list(reversed(self.history))
        if undone:
            # each touched site returns to the species it had before its first change
            first_old = {}
            for s, o, _ in self.history:
                first_old.setdefault(s, o)
            dev = self.occ_d.device
            sites = torch.as_tensor(np.fromiter(first_old.keys(), dtype=np.int64)).to(dev)
            olds = torch.as_tensor(np.fromiter(first_old.values(), dtype=np.int8)).to(dev)
            self.occ_d.index_copy_(0, sites, olds)
        self.cf_d.copy_(self._snap_cf)
        self.energy_d.copy_(self._snap_energy)
        self.history.clear()
        return undone

    # -- host views --------------------------------------------------------------
    def cf(self) -> np.ndarray:
        return self.cf_d.cpu().numpy()

    def energy(self) -> float:
        return float(self.energy_d.item())

    def occupation(self) -> np.ndarray:
        return self.occ_d.cpu().numpy()


def _has_self_interaction(cluster_info) -> bool:
    """cemc/ce_calculator.py:596-608."""
    for info in cluster_info:
        for _, cluster in info.items():
            for sub in cluster["indices"]:
                if cluster["ref_indx"] in sub:
                    return True
                if len(set(sub)) != len(sub):
                    return True
    return False


class CE:
    """Cluster-expansion calculator on the GPU with the reference's interface.

    :param atoms: sequence of objects with a ``symbol`` attribute (an ASE
        ``Atoms`` works); changes are mirrored into it.
    :param BC: settings object (``cemc_gb300.lattice.Settings`` or any object
        with the attributes ``CEUpdater::init`` reads).
    :param eci: dict of ECIs; ``c0`` is added with 0.0 if missing.
    :param initial_cf: dict of correlation functions; if None they are
        computed from scratch by the GPU full recompute.
    """

    implemented_properties = ["energy"]

    def __init__(self, atoms, BC, eci=None, initial_cf=None, device="cuda"):
        self.BC = BC
        if _has_self_interaction(BC.cluster_info):
            raise SelfInteractionError("The simulation cell is so small that the same site is present multiple "
                                       "times within one cluster. Increase the size of the simulation cell.")
        if eci is None:
            raise ValueError("ECIs are required")
        if "c0" not in eci:
            eci["c0"] = 0.0
            if initial_cf is not None:
                initial_cf["c0"] = 1.0
        self.eci = eci
        self.atoms = atoms
        self.model, self.geometry = model_and_geometry(BC, list(eci.keys()), device)
        m = self.model
        self._sym_id = {s: i for i, s in enumerate(m.symbols)}
        symbols = [a.symbol for a in atoms]
        if len(symbols) != m.n_sites:
            raise ValueError("The number of atoms and the dimension of the translation matrix is inconsistent")
        occ = m.occupation(symbols)
        cf = None
        if initial_cf is not None:
            cf = np.array([float(initial_cf[n]) for n in m.eci_names])
        self.updater = DeviceUpdater(self.geometry, occ, m.eci_vector(eci), cf=cf)
        self.results = {}
        self._linear_vib_correction = None
        if hasattr(atoms, "set_calculator"):
            try:
                atoms.set_calculator(self)
            except Exception:
                pass
        self.cf = self.get_cf()

    # -- the reference's calculator interface ----------------------------------
    def get_energy(self) -> float:
        return self.updater.energy()

    def _to_ids(self, system_changes):
        out = []
        for change in system_changes:
            i, old, new = change[0], change[1], change[2]
            out.append((int(i), self._sym_id[old], self._sym_id[new]))
        return out

    def _mirror(self, changes, use_new=True):
        for i, o, n in changes:
            self.atoms[i].symbol = self.model.symbols[n if use_new else o]

    def calculate(self, atoms=None, properties=None, system_changes=()):
        """Apply the changes and return the new energy (cemc/ce_calculator.py:345-364)."""
        changes = self._to_ids(system_changes)
        self.updater.apply(changes)
        self._mirror(changes)
        self.results["energy"] = self.updater.energy()
        return self.results["energy"]

    def update_cf(self, single_change):
        changes = self._to_ids([single_change])
        self.updater.apply(changes)
        self._mirror(changes)

    def undo_changes(self):
        undone = self.updater.undo()
        for i, o, _ in undone:
            self.atoms[i].symbol = self.model.symbols[o]

    def clear_history(self):
        self.updater.clear()

    def get_cf(self) -> Dict[str, float]:
        return dict(zip(self.model.eci_names, self.updater.cf().tolist()))

    def update_ecis(self, new_ecis: Dict[str, float]):
        self.eci = new_ecis
        unknown = [k for k in new_ecis if k not in self.model.eci_names]
        if unknown:
            raise ValueError("All ECIs has to correspond to a correlation function!")
        self.updater.set_eci(self.model.eci_vector(new_ecis))

    def get_singlets(self) -> np.ndarray:
        cf = self.updater.cf()
        return np.array([cf[k] for k in self.model.singlet_eci])

    def set_symbols(self, symbs: Sequence[str]):
        if len(symbs) != self.model.n_sites:
            raise ValueError("Length of the symbols array has to match the length of the atoms object.!")
        occ = self.model.occupation(symbs)
        self.updater.set_occupation(occ)
        for i, s in enumerate(symbs):
            self.atoms[i].symbol = s
        self.clear_history()

    def set_composition(self, comp: Dict[str, float]):
        """cemc/ce_calculator.py:397-434: all sites to the majority element, then fill in order."""
        tot = sum(comp.values())
        if abs(tot - 1.0) > 1e-6:
            raise ValueError("The specified concentration does not sum to 1!")
        init_elm = max(comp.items(), key=lambda kv: kv[1])[0]
        n = self.model.n_sites
        symbs = [init_elm] * n
        start = 0
        for elm, conc in comp.items():
            if elm == init_elm:
                continue
            n_at = int(round(conc * n))
            for i in range(start, start + n_at):
                symbs[i] = elm
            start += n_at
        self.set_symbols(symbs)

    def singlet2comp(self, singlets: Dict[str, float]) -> Dict[str, float]:
        """Concentrations from singlet values (cemc/ce_calculator.py:450-519)."""
        bfs = self.BC.basis_functions
        if len(singlets) != len(bfs):
            raise ValueError("The number singlet terms specified is different from the number of basis functions")
        rhs = np.zeros(len(bfs))
        spec_element = list(bfs[0].keys())[0]
        for key, value in singlets.items():
            dec = int(key[-1])
            rhs[dec] = value - bfs[dec][spec_element]
        matrix = np.zeros((len(bfs), len(bfs)))
        for key in singlets.keys():
            row = int(key[-1])
            col = 0
            for element in bfs[0].keys():
                if element == spec_element:
                    continue
                matrix[row, col] = bfs[row][element] - bfs[row][spec_element]
                col += 1
        concs = np.linalg.solve(matrix, rhs)
        eps = 1e-6
        concs[(concs < 0.0) & (concs > -eps)] = 0.0
        spec = 1.0 - np.sum(concs)
        if -eps < spec < 0.0:
            spec = 0.0
        if spec > 1.0 or spec < 0.0 or np.any(concs > 1.0) or np.any(concs < 0.0):
            raise RuntimeError("Something strange happened when converting singlets to composition")
        out, counter = {}, 0
        for element in bfs[0].keys():
            if element == spec_element:
                out[element] = spec
            else:
                out[element] = concs[counter]
                counter += 1
        return out

    def set_singlets(self, singlets):
        self.set_composition(self.singlet2comp(singlets))

    # -- vibrational correction: not part of this implementation ----------------
    @property
    def linear_vib_correction(self):
        return self._linear_vib_correction

    def include_linvib_in_ecis(self, T):
        if self._linear_vib_correction is not None:
            raise NotImplementedError("linear vibrational corrections are not supported")

    def vib_energy(self, T) -> float:
        return 0.0

    # -- copies and persistence ----------------------------------------------------
    def copy(self):
        import copy as _copy
        atoms = _copy.deepcopy(self.atoms) if not hasattr(self.atoms, "copy") else self.atoms.copy()
        return CE(atoms, self.BC, eci=dict(self.eci), initial_cf=self.get_cf())

    def backup_dict(self):
        return {"cf": self.get_cf(), "symbols": [a.symbol for a in self.atoms], "eci": self.eci}

    def save(self, fname):
        with open(fname, "w") as f:
            json.dump(self.backup_dict(), f, indent=2, separators=(",", ": "))

    @staticmethod
    def load(fname, atoms, BC):
        """Rebuild from a saved file; the caller supplies the atoms container and settings."""
        with open(fname) as f:
            data = json.load(f)
        for a, s in zip(atoms, data["symbols"]):
            a.symbol = s
        return CE(atoms, BC, eci=data["eci"], initial_cf=data["cf"])

    def set_num_threads(self, num_threads):
        """Accepted for compatibility; the GPU path has no host threads to set."""
        return None


class SimpleAtom:
    __slots__ = ("symbol", "index", "tag")

    def __init__(self, symbol, index, tag=0):
        self.symbol = symbol
        self.index = index
        self.tag = tag


class SimpleAtoms(list):
    """Minimal atoms container (a list of objects with ``symbol`` and ``index``) with a calculator slot."""

    def __init__(self, symbols: Sequence[str]):
        super().__init__(SimpleAtom(s, i) for i, s in enumerate(symbols))
        self._calc = None

    def set_calculator(self, calc):
        self._calc = calc

    def get_calculator(self):
        return self._calc

    @property
    def calc(self):
        return self._calc

    def get_chemical_symbols(self):
        return [a.symbol for a in self]

    def copy(self):
        new = SimpleAtoms(self.get_chemical_symbols())
        return new
