"""Device-resident chains and the calls that drive the CUDA library.

``Geometry`` owns the device copy of one supercell + cluster expansion.
``ChainBatch`` owns the state of many chains of one geometry as PyTorch
tensors on the GPU (occupation int8, correlation functions / energy FP64,
per-species site lists for swap moves, RNG counters, running sums) and runs
them through ``cemc_run`` in one launch.  PyTorch provides device memory and
streams only; all arithmetic runs in the library's kernels.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Sequence

import numpy as np
import torch

from . import _lib
from .tables import CEModel

MOVE_FLIP = _lib.MOVE_FLIP
MOVE_SWAP = _lib.MOVE_SWAP
PREC_F64 = _lib.PREC_F64
PREC_F32 = _lib.PREC_F32
KERNEL_AUTO = _lib.KERNEL_AUTO
KERNEL_GENERIC = _lib.KERNEL_GENERIC
KERNEL_SPIN = _lib.KERNEL_SPIN
KERNEL_SPIN_HALFWARP = _lib.KERNEL_SPIN_HALFWARP
KERNEL_TABLE = _lib.KERNEL_TABLE
KERNEL_FIELD = _lib.KERNEL_FIELD
KERNEL_SPIN_QUARTER = _lib.KERNEL_SPIN_QUARTER
STAMP_GLOBAL_SITES = 16384  # larger supercells get exact conflict tables in device memory
ACCUM_DOUBLES = _lib.ACCUM_DOUBLES
# Field offsets (in doubles) of cemc_accum.
A_EREF, A_SUM_E, A_SUM_E2, A_SUM_S, A_SUM_S2, A_SUM_SE, A_NSAMP, A_NACC = 0, 1, 2, 3, 7, 11, 15, 16


def _ptr(t: Optional[torch.Tensor]) -> Optional[int]:
    return None if t is None else t.data_ptr()


def _stream_ptr(stream) -> Optional[int]:
    if stream is None:
        stream = torch.cuda.current_stream()
    return stream.cuda_stream


def require_cuda(device) -> torch.device:
    device = torch.device(device)
    if device.type != "cuda":
        raise RuntimeError("the cluster-expansion kernels run on CUDA devices only (got %s)" % device)
    if not torch.cuda.is_available():
        raise RuntimeError("no CUDA device is available: the GPU library has no CPU fallback")
    return device


class Geometry:
    """Device tables of one supercell and cluster expansion (``cemc_geometry_create``)."""

    def __init__(self, model: CEModel, device="cuda"):
        self.device = require_cuda(device)
        if not model.gpu_supported:
            raise NotImplementedError("the GPU path handles at most %d translation-symmetry groups and 4 decorations"
                                      % _lib.MAX_GROUPS)
        self.model = model
        self.L = _lib.load()
        m = model
        self._host = {
            "table": np.ascontiguousarray(m.gpu_table, dtype=np.int32),
            "bf": np.ascontiguousarray(m.bf, dtype=np.float64),
            "eci_kind": np.ascontiguousarray(m.eci_kind, dtype=np.int32),
            "eci_dec": np.ascontiguousarray(m.eci_dec, dtype=np.int32),
            "eci_weight": np.ascontiguousarray(m.eci_weight, dtype=np.float64),
            "eci_full_weight": np.ascontiguousarray(m.eci_full_weight, dtype=np.float64),
            "term_eci": np.ascontiguousarray(m.term_eci, dtype=np.int32),
            "term_ref": np.ascontiguousarray(m.term_ref, dtype=np.int32),
            "term_size": np.ascontiguousarray(m.term_size, dtype=np.int32),
            "term_nb": np.ascontiguousarray(m.term_nb, dtype=np.int32),
            "movable": np.ascontiguousarray(m.movable, dtype=np.int32),
            "site_group": np.ascontiguousarray(m.site_group, dtype=np.int32),
            "group_terms": np.ascontiguousarray(m.group_terms, dtype=np.int32),
            "group_scale": np.ascontiguousarray(m.group_scale, dtype=np.float64),
        }
        h = self._host
        desc = _lib.GeometryDesc(m.n_sites, m.gpu_n_cols, m.n_sym, m.n_bf, m.n_eci, m.n_terms,
                                 *[h[n].ctypes.data for n in ("table", "bf", "eci_kind", "eci_dec", "eci_weight",
                                                              "eci_full_weight", "term_eci", "term_ref",
                                                              "term_size", "term_nb")],
                                 h["movable"].ctypes.data, int(len(m.movable)), int(m.n_groups),
                                 h["site_group"].ctypes.data, h["group_terms"].ctypes.data,
                                 h["group_scale"].ctypes.data)
        handle = C.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(self.L.cemc_geometry_create(C.byref(desc), C.byref(handle)))
        self.handle = handle

    @property
    def n_sites(self):
        return self.model.n_sites

    @property
    def n_eci(self):
        return self.model.n_eci

    def close(self):
        if getattr(self, "handle", None) is not None and self.handle.value:
            with torch.cuda.device(self.device):
                self.L.cemc_geometry_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def scratch_doubles(self, n_chains: int) -> int:
        return int(self.L.cemc_recompute_scratch_doubles(self.handle, n_chains))

    def device_bytes(self) -> int:
        """Device memory of the geometry's tables (``cemc_geometry_device_bytes``)."""
        return int(self.L.cemc_geometry_device_bytes(self.handle))

    def stamp_words(self, n_chains: int) -> int:
        return int(self.L.cemc_stamp_words(self.handle, n_chains))


def build_tracker(occ: np.ndarray, n_sym: int, background=None):
    """Per-species site lists of swap moves: sites of each species in site order.

    Same layout as ``SwapMoveIndexTracker.init_tracker``
    (cemc/mcmc/swap_move_index_tracker.py:22-33), flattened: species s owns
    trk[start[s] : start[s] + count[s]] and loc[site] is the site's slot.
    Background sites are in no list (loc = -1); they sit after the last list.
    """
    occ = np.asarray(occ)
    n_chains, n = occ.shape
    bg = np.zeros(n, dtype=bool)
    if background is not None and len(background):
        bg[np.asarray(background, dtype=np.int64)] = True
    trk = np.empty((n_chains, n), dtype=np.int32)
    loc = np.empty((n_chains, n), dtype=np.int32)
    start = np.zeros((n_chains, n_sym), dtype=np.int32)
    count = np.zeros((n_chains, n_sym), dtype=np.int32)
    for c in range(n_chains):
        key = np.where(bg, n_sym, occ[c].astype(np.int64))
        order = np.argsort(key, kind="stable").astype(np.int32)
        cnt = np.bincount(key, minlength=n_sym + 1).astype(np.int32)
        st = np.concatenate([[0], np.cumsum(cnt)[:-1]]).astype(np.int32)
        trk[c] = order
        loc[c, order] = np.arange(n, dtype=np.int32) - np.repeat(st, cnt)
        loc[c, bg] = -1
        start[c] = st[:n_sym]
        count[c] = cnt[:n_sym]
    return trk, loc, start, count


class ChainBatch:
    """State of ``n_chains`` Markov chains of one geometry, resident on the GPU."""

    def __init__(self, geo: Geometry, occ, eci, kT, move: int, seed: int = 0, chain_keys=None,
                 stream: Optional[torch.cuda.Stream] = None):
        self.geo = geo
        dev = geo.device
        m = geo.model
        occ = np.ascontiguousarray(np.asarray(occ, dtype=np.int8).reshape(-1, m.n_sites))
        n_chains = occ.shape[0]
        eci = np.asarray(eci, dtype=np.float64).reshape(-1, m.n_eci)
        if eci.shape[0] == 1 and n_chains > 1:
            eci = np.repeat(eci, n_chains, axis=0)
        kT = np.broadcast_to(np.asarray(kT, dtype=np.float64), (n_chains,)).copy()
        if np.any(kT <= 0):
            raise ValueError("temperatures must be positive")
        if occ.min() < 0 or occ.max() >= m.n_sym:
            raise ValueError("occupation holds an unknown species id")
        self.n_chains = n_chains
        self.move = int(move)
        self.seed = int(seed)
        self.stream = stream
        t = lambda a, dt: torch.as_tensor(np.ascontiguousarray(a)).to(device=dev, dtype=dt)
        self.occ = t(occ, torch.int8)
        self.eci = t(eci, torch.float64)
        self.kT = t(kT, torch.float64)
        self.cf = torch.zeros((n_chains, m.n_eci), dtype=torch.float64, device=dev)
        self.energy = torch.zeros(n_chains, dtype=torch.float64, device=dev)
        self.trial = torch.zeros(n_chains, dtype=torch.int64, device=dev)
        self.accum = torch.zeros((n_chains, ACCUM_DOUBLES), dtype=torch.float64, device=dev)
        self.status = torch.zeros(n_chains, dtype=torch.int32, device=dev)
        keys = np.arange(n_chains, dtype=np.int64) if chain_keys is None else np.asarray(chain_keys, dtype=np.int64)
        self.chain_key = t(keys.astype(np.int32), torch.int32)
        self.trk = self.loc = self.trk_start = self.trk_count = None
        if self.move == MOVE_SWAP:
            trk, loc, start, count = build_tracker(occ, m.n_sym, m.background)
            present = (count > 0).sum(axis=1)
            if np.any(present < 2):
                raise ValueError("swap moves need at least two species present in every chain")
            self.trk, self.loc = t(trk, torch.int32), t(loc, torch.int32)
            self.trk_start, self.trk_count = t(start, torch.int32), t(count, torch.int32)
        self.scratch = torch.empty(max(geo.scratch_doubles(n_chains), 1), dtype=torch.float64, device=dev)
        self.recompute()
        self.reset_accumulators()

    @classmethod
    def wrap(cls, geo: Geometry, occ: torch.Tensor, cf: torch.Tensor, energy: torch.Tensor, eci: torch.Tensor,
             kT, move: int, seed: int = 0, chain_key: int = 0, stream=None) -> "ChainBatch":
        """One chain over EXISTING device tensors (no copies): occ (N,), cf (n_eci,), energy (1,), eci (n_eci,).

        Used by the drop-in drivers, whose calculator already holds the state on the device.
        """
        self = cls.__new__(cls)
        m = geo.model
        dev = occ.device
        self.geo = geo
        self.n_chains = 1
        self.move = int(move)
        self.seed = int(seed)
        self.stream = stream
        self.occ = occ.view(1, m.n_sites)
        self.cf = cf.view(1, m.n_eci)
        self.energy = energy.view(1)
        self.eci = eci.view(1, m.n_eci)
        self.kT = torch.tensor([float(kT)], dtype=torch.float64, device=dev)
        self.trial = torch.zeros(1, dtype=torch.int64, device=dev)
        self.accum = torch.zeros((1, ACCUM_DOUBLES), dtype=torch.float64, device=dev)
        self.status = torch.zeros(1, dtype=torch.int32, device=dev)
        self.chain_key = torch.tensor([int(chain_key)], dtype=torch.int32, device=dev)
        self.trk = self.loc = self.trk_start = self.trk_count = None
        if self.move == MOVE_SWAP:
            self.rebuild_tracker()
        self.scratch = torch.empty(max(geo.scratch_doubles(1), 1), dtype=torch.float64, device=dev)
        self.reset_accumulators()
        return self

    def rebuild_tracker(self):
        """Per-species site lists from the current occupation (after external changes)."""
        m = self.geo.model
        occ = self.occ.cpu().numpy()
        trk, loc, start, count = build_tracker(occ, m.n_sym, m.background)
        if np.any((count > 0).sum(axis=1) < 2):
            raise ValueError("swap moves need at least two species present in every chain")
        dev = self.occ.device
        self.trk = torch.as_tensor(trk).to(dev)
        self.loc = torch.as_tensor(loc).to(dev)
        self.trk_start = torch.as_tensor(start).to(dev)
        self.trk_count = torch.as_tensor(count).to(dev)

    def set_temperature(self, kT):
        self.kT.copy_(torch.as_tensor(np.broadcast_to(np.asarray(kT, dtype=np.float64), (self.n_chains,)).copy()))

    # -- checkpoint ------------------------------------------------------------
    _STATE = ("occ", "cf", "energy", "eci", "kT", "trial", "accum", "chain_key", "trk", "loc", "trk_start",
              "trk_count")

    def state_dict(self) -> dict:
        """Host copy of everything a continued run reads, bit for bit.

        Occupations, correlation functions, energies, ECIs, temperatures, the
        trial counter of each chain's counter-based stream, the running sums
        (their two uint64 counters kept as raw bits) and, for swaps, the
        per-species site lists, whose order decides which site a later trial
        draws.  A batch restored from it continues exactly as this one would.
        """
        torch.cuda.synchronize(self.occ.device)
        out = {"move": np.array(self.move), "seed": np.array(self.seed, dtype=np.uint64),
               "n_sites": np.array(self.geo.model.n_sites), "n_eci": np.array(self.geo.model.n_eci)}
        for name in self._STATE:
            t = getattr(self, name, None)
            if t is not None:
                out[name] = t.cpu().numpy().copy()
        return out

    def load_state_dict(self, st: dict):
        """Restore ``state_dict`` output into this batch (same geometry, chain count and move)."""
        m = self.geo.model
        if int(st["move"]) != self.move or int(st["n_sites"]) != m.n_sites or int(st["n_eci"]) != m.n_eci:
            raise ValueError("checkpoint is of another move type or geometry")
        if np.asarray(st["occ"]).reshape(-1, m.n_sites).shape[0] != self.n_chains:
            raise ValueError("checkpoint holds %d chains, this batch %d"
                             % (np.asarray(st["occ"]).reshape(-1, m.n_sites).shape[0], self.n_chains))
        self.seed = int(np.asarray(st["seed"]).astype(np.uint64))
        dev = self.occ.device
        for name in self._STATE:
            t = getattr(self, name, None)
            if name not in st:
                continue
            src = torch.as_tensor(np.ascontiguousarray(st[name]))
            if t is None:
                setattr(self, name, src.to(dev))
            else:
                t.copy_(src.view(t.shape).to(dev, dtype=t.dtype))
        torch.cuda.synchronize(dev)

    def save(self, fname):
        """``state_dict`` as a NumPy ``.npz`` file (no pickled objects)."""
        np.savez(fname, **self.state_dict())

    def load(self, fname):
        with np.load(fname, allow_pickle=False) as d:
            self.load_state_dict({k: d[k] for k in d.files})

    # -- library calls -----------------------------------------------------
    def run(self, n_trials: int, precision: int = PREC_F64, warps: int = 0, trace: bool = False,
            chain_trials: Optional[torch.Tensor] = None, kernel: int = 0, cluster: int = 0,
            site_allow: Optional[torch.Tensor] = None, frozen: Optional[torch.Tensor] = None,
            max_attempts: int = 0, accept_first: bool = False, recycle_waste: bool = False):
        """Run ``n_trials`` trials on every chain in one launch (``cemc_run``).

        ``chain_trials`` (device int64, one per chain, each <= n_trials) gives chains their own counts.
        ``warps`` evaluating warps per CTA; ``cluster`` CTAs per chain (1, 2, or 0 = chosen by the library).
        Move constraints: ``site_allow`` (device uint8 [n_chains, n_sites], bit s = species s may be
        placed on the site), ``frozen`` (device int32 [n_chains], bit s = a site holding species s may
        not change), ``max_attempts`` redraws per trial (0 = 10000); see ``mc_constraints``.
        ``accept_first``: the first trial of the call is accepted outright (every chain).
        ``recycle_waste``: waste-recycled acceptance and running sums (generic form, one CTA).
        """
        if site_allow is not None:
            if site_allow.dtype != torch.uint8 or site_allow.numel() != self.n_chains * self.geo.model.n_sites:
                raise ValueError("site_allow must be uint8 [n_chains, n_sites]")
        if frozen is not None and (frozen.dtype != torch.int32 or frozen.numel() != self.n_chains):
            raise ValueError("frozen must be int32 [n_chains]")
        tr = None
        if trace:
            tr = (torch.zeros(self.n_chains * n_trials * 2, dtype=torch.int32, device=self.occ.device),
                  torch.zeros(self.n_chains * n_trials, dtype=torch.int8, device=self.occ.device),
                  torch.zeros(self.n_chains * n_trials, dtype=torch.float64, device=self.occ.device))
        d = _lib.RunDesc(self.n_chains, self.move, int(precision), int(warps), self.seed & (2 ** 64 - 1),
                         int(n_trials), _ptr(self.occ), _ptr(self.cf), _ptr(self.energy), _ptr(self.eci),
                         _ptr(self.kT), _ptr(self.trial), _ptr(self.accum), _ptr(self.trk), _ptr(self.loc),
                         _ptr(self.trk_start), _ptr(self.trk_count),
                         _ptr(tr[0]) if tr else None, _ptr(tr[1]) if tr else None, _ptr(tr[2]) if tr else None,
                         _ptr(self.status), _ptr(self.chain_key), _ptr(getattr(self, "accum_slot", None)),
                         _ptr(chain_trials), int(kernel), int(cluster), _ptr(self.scratch),
                         self.scratch.numel() if self.scratch is not None else 0,
                         _ptr(self._stamps()), self._stamp_buf.numel() if self._stamp_buf is not None else 0,
                         0, _ptr(site_allow), _ptr(frozen), int(max_attempts), int(bool(accept_first)),
                         int(bool(recycle_waste)))
        with torch.cuda.device(self.occ.device):
            _lib.check(self.geo.L.cemc_run(self.geo.handle, C.byref(d), _stream_ptr(self.stream)))
        # the table form ends the call with a full recompute (cf and energy exact already)
        self.last_kernel = int(d.kernel_used)
        if trace:
            return (tr[0].view(self.n_chains, n_trials, 2), tr[1].view(self.n_chains, n_trials),
                    tr[2].view(self.n_chains, n_trials))
        return None

    def _stamps(self):
        """Exact conflict tables in device memory for supercells whose shared-memory table would be hashed."""
        if getattr(self, "_stamp_buf", None) is None:
            self._stamp_buf = None
            if self.geo.n_sites > STAMP_GLOBAL_SITES:
                words = int(self.geo.L.cemc_stamp_words(self.geo.handle, self.n_chains))
                self._stamp_buf = torch.empty(words, dtype=torch.int32, device=self.occ.device)
        return self._stamp_buf

    @property
    def recomputed(self) -> bool:
        """True when the last run already ended with a full recompute (table form)."""
        return getattr(self, "last_kernel", 0) == KERNEL_TABLE

    def recompute(self):
        """Full FP64 correlation-function recompute of every chain; resets energy (``cemc_recompute``)."""
        with torch.cuda.device(self.occ.device):
            _lib.check(self.geo.L.cemc_recompute(self.geo.handle, self.n_chains, _ptr(self.occ), _ptr(self.eci),
                                                 _ptr(self.cf), _ptr(self.energy), _ptr(self.scratch),
                                                 _stream_ptr(self.stream)))

    def check_status(self):
        st = self.status.cpu().numpy()
        if np.any(st != 0):
            bad = int(np.nonzero(st)[0][0])
            raise _lib.CemcError(int(st[bad]), "chain %d reported a device status" % bad)

    # -- accumulators --------------------------------------------------------
    def reset_accumulators(self, e_ref=None):
        self.accum.zero_()
        ref = self.energy if e_ref is None else torch.as_tensor(e_ref, dtype=torch.float64,
                                                                  device=self.energy.device)
        self.accum[:, A_EREF] = ref

    def accum_host(self) -> np.ndarray:
        """Running sums as float64 columns (the two uint64 counters converted to float values)."""
        raw = self.accum.cpu().numpy()
        out = raw.copy()
        counters = np.ascontiguousarray(raw[:, A_NSAMP:A_NACC + 1]).view(np.uint64)
        out[:, A_NSAMP:A_NACC + 1] = counters.astype(np.float64)
        return out

    def set_eci(self, eci):
        """Replace the ECIs of every chain (``CEUpdater::set_ecis``, ce_updater.cpp:615-629); energy follows."""
        m = self.geo.model
        eci = torch.as_tensor(np.asarray(eci, dtype=np.float64).reshape(-1, m.n_eci), device=self.eci.device)
        self.eci.copy_(eci.expand_as(self.eci))
        self.update_energy()

    def update_energy(self):
        """energy = N * eci . cf per chain, in the reference's summation order (``cemc_energy``)."""
        with torch.cuda.device(self.occ.device):
            _lib.check(self.geo.L.cemc_energy(self.geo.handle, self.n_chains, _ptr(self.eci), _ptr(self.cf),
                                              _ptr(self.energy), _stream_ptr(self.stream)))


def pt_exchange(energy: torch.Tensor, kT: torch.Tensor, replica_of: torch.Tensor, direction: int, seed: int,
                round_index: int, n_accept: Optional[torch.Tensor] = None, stream=None,
                position_of: Optional[torch.Tensor] = None):
    """One replica-exchange sweep over a ladder on the device (``cemc_pt_exchange``).

    ``replica_of[pos]`` is the chain at ladder position ``pos``; accepted pairs
    exchange temperatures (``kT`` is indexed by chain) and positions.
    """
    L = _lib.load()
    with torch.cuda.device(energy.device):
        _lib.check(L.cemc_pt_exchange(int(replica_of.numel()), int(direction), int(seed) & (2 ** 64 - 1),
                                      int(round_index), _ptr(energy), _ptr(kT), _ptr(replica_of),
                                      _ptr(position_of), _ptr(n_accept),
                                      _stream_ptr(stream)))
