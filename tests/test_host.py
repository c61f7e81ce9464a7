"""Host-side pieces that need no GPU: RNG, C-ABI exports, tracker layout, multi-rank timing."""
import ctypes
import os
import re
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT, golden_model, load_golden


def test_philox_known_answers():
    """Published Philox4x32-10 known-answer vectors (Random123, kat_vectors)."""
    from cemc_gb300.rng import philox4x32_10
    assert philox4x32_10(0, 0, 0, 0, 0, 0) == (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)
    f = 0xFFFFFFFF
    assert philox4x32_10(f, f, f, f, f, f) == (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)
    assert philox4x32_10(0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344, 0xa4093822, 0x299f31d0) == \
        (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1)


def test_oracle_proposals_follow_the_shared_stream(oracle_mod):
    """The oracle's flip proposals equal the host restatement of the device stream."""
    from cemc_gb300.rng import flip_proposal
    g = load_golden("binary_flip")
    s, m, eci = golden_model(g)
    occ = g["occ0"].copy()
    for i in range(200):
        site, new, u = flip_proposal(int(g["seed"]), 0, i, m.n_sites, lambda x: int(occ[x]), m.n_sym)
        assert (site, new) == tuple(g["sites"][i])
        assert u == g["u"][i]
        if g["ref_acc"][i]:
            occ[site] = new


def _declared_functions():
    text = open(os.path.join(ROOT, "include", "cemc_gb300.h")).read()
    return sorted(set(re.findall(r"^(?:int|size_t)\s+(cemc_\w+)\s*\(", text, flags=re.M)))


def test_header_declares_the_abi():
    names = _declared_functions()
    for n in ("cemc_geometry_create", "cemc_run", "cemc_recompute", "cemc_apply_changes", "cemc_delta_e",
              "cemc_pt_exchange", "cemc_energy", "cemc_last_error"):
        assert n in names


def test_library_loads_and_exports_every_declared_symbol():
    from cemc_gb300 import _lib
    try:
        L = _lib.load()
    except OSError as exc:  # pragma: no cover - needs libcudart at load time
        pytest.skip("CUDA runtime not loadable here: %s" % exc)
    for n in _declared_functions():
        assert hasattr(L, n), n
    maj, mino, sm = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
    assert L.cemc_version(ctypes.byref(maj), ctypes.byref(mino), ctypes.byref(sm)) == 0
    assert sm.value == 103
    buf = ctypes.create_string_buffer(64)
    assert L.cemc_last_error(buf, 64) == 0


def test_library_rejects_bad_descriptors_without_a_gpu():
    """Argument validation happens on the host before any device call."""
    from cemc_gb300 import _lib
    try:
        L = _lib.load()
    except OSError as exc:  # pragma: no cover
        pytest.skip("CUDA runtime not loadable here: %s" % exc)
    handle = ctypes.c_void_p()
    assert L.cemc_geometry_create(None, ctypes.byref(handle)) == _lib.ERR_ARG
    d = _lib.GeometryDesc()
    d.n_sites = 0
    assert L.cemc_geometry_create(ctypes.byref(d), ctypes.byref(handle)) == _lib.ERR_ARG
    assert L.cemc_run(None, None, None) == _lib.ERR_ARG
    assert L.cemc_pt_exchange(0, 0, 0, 0, None, None, None, None, None, None) == _lib.ERR_ARG


def test_asymmetric_neighbour_table_is_rejected():
    from cemc_gb300 import _lib
    try:
        L = _lib.load()
    except OSError as exc:  # pragma: no cover
        pytest.skip("CUDA runtime not loadable here: %s" % exc)
    table = np.array([[1], [2], [0]], dtype=np.int32)  # 0->1->2->0: not symmetric
    bf = np.array([1.0, -1.0])
    kind = np.array([0, 1], dtype=np.int32)
    dec = np.array([-1, 0], dtype=np.int32)
    w = np.zeros(2)
    d = _lib.GeometryDesc(3, 1, 2, 1, 2, 0, table.ctypes.data, bf.ctypes.data, kind.ctypes.data, dec.ctypes.data,
                          w.ctypes.data, w.ctypes.data, None, None, None, None)
    handle = ctypes.c_void_p()
    assert L.cemc_geometry_create(ctypes.byref(d), ctypes.byref(handle)) == _lib.ERR_ARG
    buf = ctypes.create_string_buffer(256)
    L.cemc_last_error(buf, 256)
    assert b"symmetric" in buf.value


def test_tracker_layout_matches_oracle(oracle_mod):
    from cemc_gb300.engine import build_tracker
    g = load_golden("ternary_swap")
    s, m, eci = golden_model(g)
    orc = oracle_mod.Oracle(m)
    st = orc.new_chain_state(g["occ0"], g["eci"], 0.07, 1)
    trk, loc, start, count = build_tracker(g["occ0"][None], m.n_sym)
    assert np.array_equal(trk[0], st.trk) and np.array_equal(loc[0], st.loc)
    assert np.array_equal(start[0], st.trk_start) and np.array_equal(count[0], st.trk_count)


_DIST_SCRIPT = r"""
import os, sys
sys.path.insert(0, {root!r})
import torch.distributed as dist
import bench
dist.init_process_group("gloo")
r = dist.get_rank()
t = bench.max_over_ranks(1.0 + r, dist)
n = bench.sum_over_ranks(10.0 * (r + 1), dist)
print("RESULT", r, t, n, flush=True)
dist.destroy_process_group()
"""


def test_bench_rank_aggregation_gloo_world2(tmp_path):
    """Two CPU ranks: the timing is the max over ranks, the work the sum (replicas, no data-path collective)."""
    script = tmp_path / "agg.py"
    script.write_text(_DIST_SCRIPT.format(root=ROOT))
    env = dict(os.environ, MASTER_ADDR="127.0.0.1", MASTER_PORT="29517", WORLD_SIZE="2")
    procs = []
    for r in range(2):
        e = dict(env, RANK=str(r), LOCAL_RANK=str(r))
        procs.append(subprocess.Popen([sys.executable, str(script)], env=e, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=120) for p in procs]
    for p, (o, err) in zip(procs, outs):
        assert p.returncode == 0, err
    res = sorted(l.split()[1:] for o, _ in outs for l in o.splitlines() if l.startswith("RESULT"))
    assert [float(x[1]) for x in res] == [2.0, 2.0]
    assert [float(x[2]) for x in res] == [30.0, 30.0]


def test_self_interaction_detection():
    from cemc_gb300.calculator import _has_self_interaction
    info = [{"c2": {"ref_indx": 0, "indices": [[1], [2]]}}]
    assert not _has_self_interaction(info)
    info = [{"c2": {"ref_indx": 0, "indices": [[0]]}}]
    assert _has_self_interaction(info)
    info = [{"c3": {"ref_indx": 0, "indices": [[1, 1]]}}]
    assert _has_self_interaction(info)


def test_translation_group_descriptors_are_validated_on_the_host():
    """cemc_geometry_create checks the group fields before any device call: term ranges that do not
    cover the terms or descend, a movable site without a group, a non-positive scale, too many groups
    and terms out of ECI order inside a group are refused with a message."""
    from cemc_gb300 import _lib
    from cemc_gb300.lattice import l12_settings, seeded_ecis
    from cemc_gb300.tables import CEModel
    try:
        L = _lib.load()
    except OSError as exc:  # pragma: no cover
        pytest.skip("CUDA runtime not loadable here: %s" % exc)
    s = l12_settings(4, 3, 2, 0, ["Al", "Mg"])
    m = CEModel(s, list(seeded_ecis(s.cset, 0)))

    def arrays():
        return {
            "table": np.array(m.gpu_table, dtype=np.int32, copy=True), "bf": np.array(m.bf, copy=True),
            "kind": np.array(m.eci_kind, dtype=np.int32, copy=True),
            "dec": np.array(m.eci_dec, dtype=np.int32, copy=True),
            "w": np.array(m.eci_weight, copy=True), "fw": np.array(m.eci_full_weight, copy=True),
            "te": np.array(m.term_eci, dtype=np.int32, copy=True),
            "tr": np.array(m.term_ref, dtype=np.int32, copy=True),
            "ts": np.array(m.term_size, dtype=np.int32, copy=True),
            "tn": np.array(m.term_nb, dtype=np.int32, copy=True),
            "mov": np.array(m.movable, dtype=np.int32, copy=True),
            "sg": np.array(m.site_group, dtype=np.int32, copy=True),
            "gt": np.array(m.group_terms, dtype=np.int32, copy=True),
            "gs": np.array(m.group_scale, dtype=np.float64, copy=True)}

    def create(h, n_groups=m.n_groups, site_group=True):
        d = _lib.GeometryDesc(m.n_sites, m.gpu_n_cols, m.n_sym, m.n_bf, m.n_eci, m.n_terms,
                              *[h[k].ctypes.data for k in ("table", "bf", "kind", "dec", "w", "fw", "te", "tr",
                                                           "ts", "tn")],
                              h["mov"].ctypes.data, len(m.movable), n_groups,
                              h["sg"].ctypes.data if site_group else None, h["gt"].ctypes.data, h["gs"].ctypes.data)
        handle = ctypes.c_void_p()
        rc = L.cemc_geometry_create(ctypes.byref(d), ctypes.byref(handle))
        buf = ctypes.create_string_buffer(256)
        L.cemc_last_error(buf, 256)
        if rc == _lib.OK:
            L.cemc_geometry_destroy(handle)
        return rc, buf.value.decode()

    rc, _ = create(arrays())  # the valid descriptor passes the host checks (no GPU here: the allocation fails)
    assert rc in (_lib.OK, _lib.ERR_CUDA)
    h = arrays()
    h["gt"][-1] -= 1
    assert create(h) == (_lib.ERR_ARG, "group term ranges must cover the terms")
    h = arrays()
    h["gt"][1], h["gt"][2] = h["gt"][2], h["gt"][1]
    assert create(h)[0] == _lib.ERR_ARG
    h = arrays()
    h["sg"][5] = m.n_groups
    assert create(h) == (_lib.ERR_ARG, "site 5 has no translation group")
    h = arrays()
    h["gs"][2] = 0.0
    assert create(h) == (_lib.ERR_ARG, "bad group scale")
    assert create(arrays(), site_group=False) == (_lib.ERR_ARG, "null group table")
    assert create(arrays(), n_groups=9)[0] == _lib.ERR_LIMIT
    h = arrays()
    lo = int(h["gt"][1])
    h["te"][lo], h["te"][lo + 1] = h["te"][lo + 1] + 1, h["te"][lo]
    if h["te"][lo] != h["te"][lo + 1]:
        assert create(h)[0] == _lib.ERR_ARG
