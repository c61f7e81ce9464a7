"""Autotuner for the launch shape of the Monte Carlo kernel.

A launch shape is (warps, cluster, kernel): evaluating warps per CTA, CTAs per
chain (1, or a cluster pair of 2 on two SMs) and the kernel form (the
library's automatic choice, or the local-field form for single-site flips of a
geometry that has it).  The best shape depends on the supercell size (conflict
probability between trials of one round), the cluster set (work per trial),
the move type, the number of chains sharing the GPU (pairs only pay while SMs
are idle) and the acceptance rate of the chains (the local-field form spends
its time on accepted flips, the spin forms on every trial).
``best_config`` times short runs of the candidate shapes on the caller's batch
(state restored afterwards) or on a synthetic one and caches the winner in a
JSON file keyed by those features and the device name.
"""
from __future__ import annotations

import json
import os
import threading
from typing import Dict, Optional, Sequence, Tuple

import numpy as np
import torch

from . import engine as E

CANDIDATES = (4, 8, 12, 16)              # warps per CTA, one CTA per chain
PAIR_CANDIDATES = (8, 12, 16)            # warps per CTA, cluster pairs
FIELD_CANDIDATES = (16, 28)              # worker warps of the local-field form
QUARTER_CANDIDATES = (8, 12, 16)         # warps of the quarter-warp spin form (four flips per warp)
_CACHE_PATH = os.environ.get("CEMC_AUTOTUNE_CACHE",
                             os.path.join(os.path.expanduser("~"), ".cache", "cemc_gb300", "autotune.json"))
_lock = threading.Lock()
_mem: Dict[str, int] = {}


def _key(geo, move, precision, n_chains) -> str:
    name = torch.cuda.get_device_name(geo.device)
    m = geo.model
    # chains only matter up to one per SM
    sms = torch.cuda.get_device_properties(geo.device).multi_processor_count
    return "|".join(map(str, ("shape3", name, m.n_sites, m.gpu_n_cols, m.n_groups, m.n_terms, m.n_eci, move, precision,
                              min(int(n_chains), sms))))


def candidates(geo, n_chains: int, move: int = E.MOVE_SWAP):
    """(warps, cluster, kernel) shapes worth timing for ``n_chains`` chains on this device."""
    sms = torch.cuda.get_device_properties(geo.device).multi_processor_count
    out = [(w, 1, E.KERNEL_AUTO) for w in CANDIDATES]
    if 2 * int(n_chains) <= sms:
        out += [(w, 2, E.KERNEL_AUTO) for w in PAIR_CANDIDATES]
    if move == E.MOVE_FLIP:
        out += [(w, 1, E.KERNEL_FIELD) for w in FIELD_CANDIDATES]  # skipped where the geometry lacks it
        out += [(w, 1, E.KERNEL_SPIN_QUARTER) for w in QUARTER_CANDIDATES]
    return out


def _load():
    try:
        with open(_CACHE_PATH) as f:
            return json.load(f)
    except Exception:
        return {}


def _save(d):
    try:
        os.makedirs(os.path.dirname(_CACHE_PATH), exist_ok=True)
        tmp = _CACHE_PATH + ".tmp"
        with open(tmp, "w") as f:
            json.dump(d, f, indent=1, sort_keys=True)
        os.replace(tmp, _CACHE_PATH)
    except Exception:
        pass


def tune(geo, move: int, precision: int, n_chains: int, shapes=None, sweeps: float = 0.5,
         seed: int = 12345) -> Dict[tuple, float]:
    """Trials/s of each candidate shape on a random batch at a mid-range temperature."""
    m = geo.model
    n = min(int(n_chains), torch.cuda.get_device_properties(geo.device).multi_processor_count)
    rng = np.random.default_rng(seed)
    occ = rng.integers(0, m.n_sym, (n, m.n_sites)).astype(np.int8)
    eci = np.zeros(m.n_eci)
    eci[m.eci_kind == 2] = rng.normal(0.0, 0.01, int((m.eci_kind == 2).sum()))
    cb = E.ChainBatch(geo, occ, eci, 8.6173303e-5 * 800.0, move, seed=seed)
    return tune_on(cb, precision, shapes, sweeps)


def tune_on(cb, precision: int, shapes=None, sweeps: float = 0.25) -> Dict[tuple, float]:
    """Trials/s of each shape on the caller's own batch; its state is restored afterwards."""
    shapes = list(shapes) if shapes is not None else candidates(cb.geo, cb.n_chains, cb.move)
    names = ["occ", "cf", "energy", "trial", "accum"] + (["trk", "loc"] if cb.trk is not None else [])
    torch.cuda.synchronize()  # the batch's own stream may still be writing its state
    snap = {n: getattr(cb, n).clone() for n in names}
    trials = max(256, int(sweeps * cb.geo.n_sites))
    stream = cb.stream if cb.stream is not None else torch.cuda.current_stream()
    out = {}
    from ._lib import CemcError
    for shape in shapes:
        w, cl, kern = (tuple(shape) + (E.KERNEL_AUTO,))[:3]
        try:
            cb.run(trials // 4, precision=precision, warps=w, cluster=cl, kernel=kern)
        except CemcError as exc:
            # this shape does not fit in shared memory (5), or the form does not apply here (1)
            if exc.code == 5 or (exc.code == 1 and kern != E.KERNEL_AUTO):
                for n, t in snap.items():
                    getattr(cb, n).copy_(t)
                continue
            raise
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)  # the kernel runs on the batch's stream
        cb.run(trials, precision=precision, warps=w, cluster=cl, kernel=kern)
        e1.record(stream)
        torch.cuda.synchronize()
        out[(int(w), int(cl), int(kern))] = cb.n_chains * trials / (e0.elapsed_time(e1) * 1e-3)
        for n, t in snap.items():
            getattr(cb, n).copy_(t)
    torch.cuda.synchronize()
    return out


def best_config(geo, move: int, precision: int, n_chains: int, batch=None) -> Tuple[int, int, int]:
    """Cached best (warps, cluster, kernel) for this geometry/move/precision/chain count; tuned on ``batch``
    when given."""
    key = _key(geo, move, precision, n_chains)
    with _lock:
        if key in _mem:
            return _mem[key]
        disk = _load()
        if key in disk and len(disk[key]) == 3:
            _mem[key] = tuple(int(x) for x in disk[key])
            return _mem[key]
    rates = tune_on(batch, precision) if batch is not None else tune(geo, move, precision, n_chains)
    best = max(rates, key=rates.get)
    with _lock:
        _mem[key] = best
        disk = _load()
        disk[key] = list(best)
        _save(disk)
    return best


def best_warps(geo, move: int, precision: int, n_chains: int, batch=None) -> int:
    """Warps per CTA of the best shape among the library's automatic forms (``best_config``)."""
    w, _, kern = best_config(geo, move, precision, n_chains, batch)
    return w if kern == E.KERNEL_AUTO else 16
