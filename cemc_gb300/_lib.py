"""ctypes binding of libcemc_gb300.so (declarations in include/cemc_gb300.h).

The library is the only compute path: if it cannot be loaded, every call
raises.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import build as _build

OK = 0
ERR_ARG = 1
ERR_CUDA = 2
ERR_BACKGROUND = 3
ERR_STATE = 4
ERR_LIMIT = 5
ERR_TIMEOUT = 6
ERR_INTERNAL = 7
ERR_NO_MOVE = 8

MOVE_FLIP = 0
MOVE_SWAP = 1
PREC_F64 = 0
PREC_F32 = 1
KERNEL_AUTO = 0
KERNEL_GENERIC = 1
KERNEL_SPIN = 2
KERNEL_SPIN_HALFWARP = 3
KERNEL_TABLE = 4
KERNEL_FIELD = 5
KERNEL_SPIN_QUARTER = 6
MAX_BF = 4
MAX_GROUPS = 8

_P = C.c_void_p


class Accum(C.Structure):
    _fields_ = [("e_ref", C.c_double), ("sum_e", C.c_double), ("sum_e2", C.c_double),
                ("sum_s", C.c_double * MAX_BF), ("sum_s2", C.c_double * MAX_BF), ("sum_se", C.c_double * MAX_BF),
                ("n_samples", C.c_uint64), ("n_accept", C.c_uint64)]


ACCUM_DOUBLES = C.sizeof(Accum) // 8  # 17 doubles: 15 sums + two uint64 counters


class GeometryDesc(C.Structure):
    _fields_ = [("n_sites", C.c_int32), ("n_cols", C.c_int32), ("n_sym", C.c_int32), ("n_bf", C.c_int32),
                ("n_eci", C.c_int32), ("n_terms", C.c_int32),
                ("table", _P), ("bf", _P), ("eci_kind", _P), ("eci_dec", _P), ("eci_weight", _P),
                ("eci_full_weight", _P), ("term_eci", _P), ("term_ref", _P), ("term_size", _P), ("term_nb", _P),
                ("movable", _P), ("n_movable", C.c_int32),
                ("n_groups", C.c_int32), ("site_group", _P), ("group_terms", _P), ("group_scale", _P)]


class RunDesc(C.Structure):
    _fields_ = [("n_chains", C.c_int32), ("move", C.c_int32), ("precision", C.c_int32), ("warps", C.c_int32),
                ("seed", C.c_uint64), ("n_trials", C.c_uint64),
                ("occ", _P), ("cf", _P), ("energy", _P), ("eci", _P), ("kT", _P), ("trial", _P), ("accum", _P),
                ("trk", _P), ("loc", _P), ("trk_start", _P), ("trk_count", _P),
                ("trace_site", _P), ("trace_acc", _P), ("trace_de", _P), ("status", _P), ("chain_key", _P),
                ("accum_slot", _P), ("chain_trials", _P), ("kernel", C.c_int32), ("cluster", C.c_int32),
                ("scratch", _P), ("scratch_doubles", C.c_uint64), ("stamps", _P), ("stamp_words", C.c_uint64),
                ("kernel_used", C.c_int32), ("site_allow", _P), ("frozen", _P), ("max_attempts", C.c_int32),
                ("accept_first", C.c_int32), ("recycle_waste", C.c_int32)]


class CemcError(RuntimeError):
    """A library call returned a non-zero status."""

    def __init__(self, code: int, msg: str):
        super().__init__("%s (status %d)" % (msg, code))
        self.code = code


_lock = threading.Lock()
_lib = None


def path() -> str:
    return _build.LIB


def load():
    """Load (building first if stale) the CUDA library; raises if that fails."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        lib_path = _build.LIB
        if not os.path.exists(lib_path) or _build._stale():
            try:
                _build.build()
            except Exception as exc:  # no silent fallback: the CUDA path is the product
                raise ImportError("libcemc_gb300.so could not be built: %s" % exc) from exc
        L = C.CDLL(lib_path)
        L.cemc_geometry_create.argtypes = [C.POINTER(GeometryDesc), C.POINTER(_P)]
        L.cemc_geometry_destroy.argtypes = [_P]
        L.cemc_run.argtypes = [_P, C.POINTER(RunDesc), _P]
        L.cemc_recompute_scratch_doubles.restype = C.c_size_t
        L.cemc_recompute_scratch_doubles.argtypes = [_P, C.c_int32]
        L.cemc_recompute.argtypes = [_P, C.c_int32, _P, _P, _P, _P, _P, _P]
        L.cemc_geometry_device_bytes.restype = C.c_size_t
        L.cemc_geometry_device_bytes.argtypes = [_P]
        L.cemc_stamp_words.restype = C.c_size_t
        L.cemc_stamp_words.argtypes = [_P, C.c_int32]
        L.cemc_energy.argtypes = [_P, C.c_int32, _P, _P, _P, _P]
        L.cemc_recompute_noalloc.argtypes = [_P, C.c_int32, _P, _P, _P, _P, _P]
        L.cemc_apply_changes.argtypes = [_P, _P, _P, _P, _P, C.c_int32, _P, _P, _P, _P, _P]
        L.cemc_delta_e.argtypes = [_P, _P, _P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, _P, _P, _P]
        L.cemc_pt_exchange.argtypes = [C.c_int32, C.c_int32, C.c_uint64, C.c_uint64, _P, _P, _P, _P, _P, _P]
        L.cemc_last_error.argtypes = [C.c_char_p, C.c_size_t]
        L.cemc_version.argtypes = [C.POINTER(C.c_int32)] * 3
        for name in ("cemc_geometry_create", "cemc_geometry_destroy", "cemc_run", "cemc_recompute", "cemc_energy",
                     "cemc_recompute_noalloc",
                     "cemc_apply_changes", "cemc_delta_e", "cemc_pt_exchange", "cemc_last_error", "cemc_version"):
            getattr(L, name).restype = C.c_int
        _lib = L
        return L


def check(rc: int):
    if rc != OK:
        buf = C.create_string_buffer(512)
        _lib.cemc_last_error(buf, 512)
        raise CemcError(rc, buf.value.decode(errors="replace"))


def exported_symbols():
    """Names declared in include/cemc_gb300.h that the loaded library exports."""
    L = load()
    names = []
    for n in ("cemc_geometry_create", "cemc_geometry_destroy", "cemc_geometry_device_bytes", "cemc_run",
              "cemc_recompute_scratch_doubles", "cemc_stamp_words", "cemc_recompute", "cemc_recompute_noalloc", "cemc_energy", "cemc_apply_changes", "cemc_delta_e", "cemc_pt_exchange", "cemc_last_error",
              "cemc_version"):
        if hasattr(L, n):
            names.append(n)
    return names
