"""Python side of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Loads the C restatement (``libce_oracle.so``, built from ``ce_oracle.c``) and,
when it has been built here, the reference's own compiled ``CEUpdater``
(``_ref/cemc_ref_updater*.so``, see ``build_ref.sh``).  Only tests,
``__graft_entry__.smoke()`` and the CPU-baseline legs of ``bench.py`` import
this module; the product path never does.
"""
from __future__ import annotations

import ctypes as C
import glob
import os
import subprocess
import sys
import types
from typing import Dict, List, Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libce_oracle.so")

MOVE_FLIP = 0
MOVE_SWAP = 1


class Accum(C.Structure):
    _fields_ = [("e_ref", C.c_double), ("sum_e", C.c_double), ("sum_e2", C.c_double),
                ("sum_s", C.c_double * 4), ("sum_s2", C.c_double * 4), ("sum_se", C.c_double * 4),
                ("n_samples", C.c_uint64), ("n_accept", C.c_uint64)]


ACCUM_DTYPE = np.dtype([("e_ref", "f8"), ("sum_e", "f8"), ("sum_e2", "f8"), ("sum_s", "f8", 4),
                        ("sum_s2", "f8", 4), ("sum_se", "f8", 4), ("n_samples", "u8"), ("n_accept", "u8")])
assert ACCUM_DTYPE.itemsize == C.sizeof(Accum)

_P = C.c_void_p


class OrcModel(C.Structure):
    _fields_ = [(n, C.c_int32) for n in ("n_sites", "n_cols", "n_sym", "n_bf", "n_eci", "n_types", "n_groups",
                                         "n_movable")] + \
               [(n, _P) for n in ("table", "site_group", "group_count", "movable", "bf", "type_size", "type_m",
                                  "type_M", "type_off", "members", "order", "eci_kind", "eci_type", "eq_off",
                                  "eq_decos", "singlet_eci")]


class OrcChain(C.Structure):
    _fields_ = [("occ", _P), ("cf", _P), ("eci", _P), ("kT", C.c_double), ("energy", _P), ("acc", _P),
                ("trk", _P), ("loc", _P), ("trk_start", _P), ("trk_count", _P),
                ("allow", _P), ("frozen", C.c_uint32), ("max_attempts", C.c_int32), ("accept_first", C.c_int32),
                ("recycle", C.c_int32)]


class NoLegalMove(RuntimeError):
    """The constraint redraws of a trial ran out (CanNotFindLegalMoveError); ``trace`` holds the run."""

    def __init__(self, trace):
        super().__init__("no trial move satisfying the constraints within the allowed redraws")
        self.trace = trace


class OrcTrace(C.Structure):
    _fields_ = [("site", _P), ("acc", _P), ("de", _P), ("u", _P)]


def build(force: bool = False) -> str:
    """Compile the C oracle (make, gcc) and return the library path."""
    src = os.path.join(HERE, "ce_oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        L.orc_energy.restype = C.c_double
        L.orc_energy.argtypes = [C.POINTER(OrcModel), _P, _P]
        L.orc_update_cf.restype = C.c_int
        L.orc_update_cf.argtypes = [C.POINTER(OrcModel), _P, C.c_int, C.c_int, _P, _P]
        L.orc_full_cf.restype = None
        L.orc_full_cf.argtypes = [C.POINTER(OrcModel), _P, _P]
        L.orc_tracker_init.restype = None
        L.orc_tracker_init.argtypes = [C.POINTER(OrcModel), _P, _P, _P, _P, _P]
        L.orc_run_chain.restype = C.c_int
        L.orc_run_chain.argtypes = [C.POINTER(OrcModel), C.POINTER(OrcChain), C.c_int, C.c_uint64, C.c_uint32,
                                    C.c_uint64, C.c_uint64, C.POINTER(OrcTrace)]
        L.orc_run_many.restype = C.c_int
        L.orc_run_many.argtypes = [C.POINTER(OrcModel), C.POINTER(OrcChain), C.c_int, _P, C.c_int, C.c_uint64,
                                   C.c_uint64, C.c_uint64, C.c_int]
        _lib = L
    return _lib


def _ptr(a: Optional[np.ndarray]) -> Optional[int]:
    return None if a is None else a.ctypes.data


class Oracle:
    """FP64 reference-order evaluation of one model (see ce_oracle.c)."""

    def __init__(self, model):
        self.model = model
        m = model
        self._keep = {
            "table": np.ascontiguousarray(m.table, dtype=np.int32),
            "site_group": np.ascontiguousarray(m.site_group, dtype=np.int32),
            "group_count": np.ascontiguousarray(m.group_count, dtype=np.int32),
            "movable": np.ascontiguousarray(m.movable, dtype=np.int32),
            "bf": np.ascontiguousarray(m.bf, dtype=np.float64),
            "type_size": np.ascontiguousarray(m.type_size, dtype=np.int32),
            "type_m": np.ascontiguousarray(m.type_m, dtype=np.int32),
            "type_M": np.ascontiguousarray(m.type_M, dtype=np.int32),
            "type_off": np.ascontiguousarray(m.type_off, dtype=np.int32),
            "members": np.ascontiguousarray(m.members, dtype=np.int32),
            "order": np.ascontiguousarray(m.order, dtype=np.int32),
            "eci_kind": np.ascontiguousarray(m.eci_kind, dtype=np.int32),
            "eci_type": np.ascontiguousarray(m.eci_type, dtype=np.int32),
            "eq_off": np.ascontiguousarray(m.eq_off, dtype=np.int32),
            "eq_decos": np.ascontiguousarray(m.eq_decos, dtype=np.int32),
            "singlet_eci": np.ascontiguousarray(m.singlet_eci, dtype=np.int32),
        }
        k = self._keep
        self.c = OrcModel(m.n_sites, m.n_cols, m.n_sym, m.n_bf, m.n_eci, len(m.type_names), m.n_groups,
                          len(m.movable), *[_ptr(k[n]) for n in ("table", "site_group", "group_count", "movable",
                                                                  "bf", "type_size", "type_m", "type_M",
                                                                  "type_off", "members", "order", "eci_kind",
                                                                  "eci_type", "eq_off", "eq_decos",
                                                                  "singlet_eci")])
        self.L = lib()

    def energy(self, eci: np.ndarray, cf: np.ndarray) -> float:
        eci = np.ascontiguousarray(eci, dtype=np.float64)
        cf = np.ascontiguousarray(cf, dtype=np.float64)
        return self.L.orc_energy(C.byref(self.c), _ptr(eci), _ptr(cf))

    def full_cf(self, occ: np.ndarray) -> np.ndarray:
        occ = np.ascontiguousarray(occ, dtype=np.int8)
        out = np.zeros(self.model.n_eci)
        self.L.orc_full_cf(C.byref(self.c), _ptr(occ), _ptr(out))
        return out

    def update_cf(self, occ: np.ndarray, site: int, new_id: int, cf: np.ndarray) -> np.ndarray:
        """cf after changing ``site`` to ``new_id`` (occ is not modified)."""
        occ = np.ascontiguousarray(occ, dtype=np.int8)
        cf = np.ascontiguousarray(cf, dtype=np.float64)
        out = np.zeros_like(cf)
        rc = self.L.orc_update_cf(C.byref(self.c), _ptr(occ), int(site), int(new_id), _ptr(cf), _ptr(out))
        if rc == 3:
            raise RuntimeError("Attempting to move a background atom!")
        return out

    def new_chain_state(self, occ: np.ndarray, eci: np.ndarray, kT: float, move: int, e_ref: Optional[float] = None,
                        allow: Optional[np.ndarray] = None, frozen: int = 0, max_attempts: int = 0,
                        accept_first: int = 0, recycle: int = 0):
        """Host-side chain (occ, cf from the full recompute, energy, tracker, sums).

        ``allow`` (uint8 per site, bit s = species s may be placed there), ``frozen`` (bit s = a site
        holding species s may not change) and ``max_attempts`` are the move constraints."""
        m = self.model
        st = types.SimpleNamespace()
        st.occ = np.ascontiguousarray(occ, dtype=np.int8).copy()
        st.eci = np.ascontiguousarray(eci, dtype=np.float64).copy()
        st.cf = self.full_cf(st.occ)
        st.energy = np.array([self.energy(st.eci, st.cf)])
        st.acc = np.zeros(1, dtype=ACCUM_DTYPE)
        st.acc["e_ref"] = st.energy[0] if e_ref is None else e_ref
        st.kT = float(kT)
        st.trk = np.zeros(m.n_sites, dtype=np.int32)
        st.loc = np.zeros(m.n_sites, dtype=np.int32)
        st.trk_start = np.zeros(m.n_sym, dtype=np.int32)
        st.trk_count = np.zeros(m.n_sym, dtype=np.int32)
        if move == MOVE_SWAP:
            self.L.orc_tracker_init(C.byref(self.c), _ptr(st.occ), _ptr(st.trk), _ptr(st.loc), _ptr(st.trk_start),
                                    _ptr(st.trk_count))
        st.move = move
        st.allow = None if allow is None else np.ascontiguousarray(allow, dtype=np.uint8).copy()
        st.frozen = int(frozen)
        st.max_attempts = int(max_attempts)
        st.accept_first = int(accept_first)
        st.recycle = int(recycle)
        return st

    def _cchain(self, st) -> OrcChain:
        return OrcChain(_ptr(st.occ), _ptr(st.cf), _ptr(st.eci), st.kT, _ptr(st.energy), _ptr(st.acc),
                        _ptr(st.trk), _ptr(st.loc), _ptr(st.trk_start), _ptr(st.trk_count),
                        _ptr(getattr(st, "allow", None)), int(getattr(st, "frozen", 0)),
                        int(getattr(st, "max_attempts", 0)), int(getattr(st, "accept_first", 0)),
                        int(getattr(st, "recycle", 0)))

    def run(self, st, seed: int, chain_id: int, t_begin: int, n_trials: int, trace: bool = False):
        """Run trials [t_begin, t_begin + n_trials) of one chain in place; optional per-trial trace."""
        ch = self._cchain(st)
        tr = None
        out = None
        if trace:
            out = types.SimpleNamespace(site=np.zeros(2 * n_trials, dtype=np.int32),
                                        acc=np.zeros(n_trials, dtype=np.int8),
                                        de=np.zeros(n_trials), u=np.zeros(n_trials))
            tr = OrcTrace(_ptr(out.site), _ptr(out.acc), _ptr(out.de), _ptr(out.u))
        rc = self.L.orc_run_chain(C.byref(self.c), C.byref(ch), st.move, seed, chain_id, t_begin, n_trials,
                                  C.byref(tr) if tr is not None else None)
        if rc == 8:
            raise NoLegalMove(out)
        if rc:
            raise RuntimeError("oracle run failed with status %d" % rc)
        return out

    def run_many(self, states: Sequence, seed: int, chain_ids: Sequence[int], t_begin: int, n_trials: int,
                 n_threads: int):
        """Run many chains on host threads (the CPU baseline)."""
        arr = (OrcChain * len(states))(*[self._cchain(s) for s in states])
        ids = np.ascontiguousarray(chain_ids, dtype=np.uint32)
        move = states[0].move
        rc = self.L.orc_run_many(C.byref(self.c), arr, len(states), _ptr(ids), move, seed, t_begin, n_trials,
                                 n_threads)
        if rc:
            raise RuntimeError("oracle run failed with status %d" % rc)


# ---------------------------------------------------------------------------
# The reference's own compiled CEUpdater (only where build_ref.sh has run).

def _install_equivalent_deco_module():
    """Provide ``ase.clease.tools.equivalent_deco`` for cluster.cpp:78-81.

    The reference imports that CLEASE helper to expand equivalent
    decorations.  CLEASE is not installed, so a module object carrying this
    project's implementation of the same rule is registered under that name.
    """
    from cemc_gb300.lattice import equivalent_decorations
    if "ase.clease.tools" in sys.modules:
        return
    ase = sys.modules.get("ase") or types.ModuleType("ase")
    clease = types.ModuleType("ase.clease")
    tools = types.ModuleType("ase.clease.tools")
    tools.equivalent_deco = lambda deco, equiv_sites: equivalent_decorations(list(deco),
                                                                              [list(g) for g in equiv_sites])
    ase.clease = clease
    clease.tools = tools
    sys.modules.setdefault("ase", ase)
    sys.modules["ase.clease"] = clease
    sys.modules["ase.clease.tools"] = tools


def reference_module():
    """The compiled reference binding, or None when it was not built here."""
    ref_dir = os.path.join(HERE, "_ref")
    if not glob.glob(os.path.join(ref_dir, "cemc_ref_updater*.so")):
        return None
    if ref_dir not in sys.path:
        sys.path.insert(0, ref_dir)
    import cemc_ref_updater  # noqa: E402
    _install_equivalent_deco_module()
    return cemc_ref_updater


class _Atom:
    __slots__ = ("symbol", "index")

    def __init__(self, symbol, index):
        self.symbol = symbol
        self.index = index


_KEEP_ALIVE: List[object] = []


def make_reference_updater(settings, symbols: Sequence[str], cf: Dict[str, float], eci: Dict[str, float]):
    """A reference ``PyCEUpdater`` over a plain list of atoms; returns (updater, atoms).

    ``CEUpdater`` stores the atoms object without taking a reference and
    releases one in its destructor (cpp/src/ce_updater.cpp:22, 33).  The
    harness therefore takes that reference on its behalf and keeps the list
    alive for the life of the process.
    """
    import ctypes
    mod = reference_module()
    if mod is None:
        raise RuntimeError("reference CEUpdater not built (oracle/build_ref.sh)")
    atoms = [_Atom(s, i) for i, s in enumerate(symbols)]
    ctypes.pythonapi.Py_IncRef(ctypes.py_object(atoms))
    _KEEP_ALIVE.append(atoms)
    upd = mod.PyCEUpdater(atoms, settings, dict(cf), dict(eci))
    return upd, atoms
