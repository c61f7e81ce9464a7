"""Autotuner for the speculation width (warps per chain) of the Monte Carlo kernel.

The best width depends on the supercell size (conflict probability between
trials of one round), the cluster set (work per trial), the move type and the
number of chains sharing the GPU.  ``best_warps`` times short runs of the
candidate widths on scratch copies of a synthetic batch and caches the winner
in a JSON file keyed by those features and the device name.
"""
from __future__ import annotations

import json
import os
import threading
from typing import Dict, Optional, Sequence

import numpy as np
import torch

from . import engine as E

CANDIDATES = (1, 2, 4, 8, 12, 16, 24, 31)
_CACHE_PATH = os.environ.get("CEMC_AUTOTUNE_CACHE",
                             os.path.join(os.path.expanduser("~"), ".cache", "cemc_gb300", "autotune.json"))
_lock = threading.Lock()
_mem: Dict[str, int] = {}


def _key(geo, move, precision, n_chains) -> str:
    name = torch.cuda.get_device_name(geo.device)
    m = geo.model
    # chains only matter up to one per SM
    sms = torch.cuda.get_device_properties(geo.device).multi_processor_count
    return "|".join(map(str, (name, m.n_sites, m.n_cols, m.n_terms, m.n_eci, move, precision,
                              min(int(n_chains), sms))))


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


def tune(geo, move: int, precision: int, n_chains: int, candidates: Sequence[int] = CANDIDATES,
         sweeps: float = 0.5, seed: int = 12345) -> Dict[int, float]:
    """Trials/s of each candidate width on a random 50/50 batch at a mid-range temperature."""
    m = geo.model
    n = min(int(n_chains), torch.cuda.get_device_properties(geo.device).multi_processor_count)
    rng = np.random.default_rng(seed)
    occ = rng.integers(0, m.n_sym, (n, m.n_sites)).astype(np.int8)
    eci = np.zeros(m.n_eci)
    eci[m.eci_kind == 2] = rng.normal(0.0, 0.01, int((m.eci_kind == 2).sum()))
    cb = E.ChainBatch(geo, occ, eci, 8.6173303e-5 * 800.0, move, seed=seed)
    trials = max(256, int(sweeps * m.n_sites))
    out = {}
    for w in candidates:
        cb.run(trials // 4, precision=precision, warps=w)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        cb.run(trials, precision=precision, warps=w)
        e1.record()
        torch.cuda.synchronize()
        out[int(w)] = n * trials / (e0.elapsed_time(e1) * 1e-3)
    return out


def tune_on(cb, precision: int, candidates: Sequence[int] = CANDIDATES, sweeps: float = 0.25) -> Dict[int, float]:
    """Trials/s of each width on the caller's own batch; its state is restored afterwards."""
    names = ["occ", "cf", "energy", "trial", "accum"] + (["trk", "loc"] if cb.trk is not None else [])
    snap = {n: getattr(cb, n).clone() for n in names}
    trials = max(256, int(sweeps * cb.geo.n_sites))
    stream = cb.stream if cb.stream is not None else torch.cuda.current_stream()
    out = {}
    for w in candidates:
        cb.run(trials // 4, precision=precision, warps=w)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)  # the kernel runs on the batch's stream
        cb.run(trials, precision=precision, warps=w)
        e1.record(stream)
        torch.cuda.synchronize()
        out[int(w)] = cb.n_chains * trials / (e0.elapsed_time(e1) * 1e-3)
        for n, t in snap.items():
            getattr(cb, n).copy_(t)
    torch.cuda.synchronize()
    return out


def best_warps(geo, move: int, precision: int, n_chains: int, batch=None) -> int:
    """Cached best width for this geometry/move/precision/chain count; tuned on ``batch`` when given."""
    key = _key(geo, move, precision, n_chains)
    with _lock:
        if key in _mem:
            return _mem[key]
        disk = _load()
        if key in disk:
            _mem[key] = int(disk[key])
            return _mem[key]
    rates = tune_on(batch, precision) if batch is not None else tune(geo, move, precision, n_chains)
    best = max(rates, key=rates.get)
    with _lock:
        _mem[key] = best
        disk = _load()
        disk[key] = best
        _save(disk)
    return best
