import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

KB = 8.6173303e-5


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the library's kernels)")


def golden_cases():
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.endswith(".npz") and not f.startswith("constraints"))


def load_golden(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False)
    return {k: d[k] for k in d.files}


def settings_for(lattice, L, ps, ts, qs, syms):
    """``fcc``, ``l12`` or ``l12:<group of each sublattice>`` settings (the lattice key of a golden case)."""
    from cemc_gb300.lattice import cubic_settings, fcc_settings, hcp_settings, l12_settings
    if lattice.startswith("l12"):
        gob = tuple(int(ch) for ch in lattice.split(":")[1]) if ":" in lattice else (0, 1, 2, 3)
        return l12_settings(L, ps, ts, qs, syms, group_of_basis=gob)
    if lattice in ("bcc", "sc"):
        return cubic_settings(lattice, L, ps, ts, qs, syms)
    if lattice.startswith("hcp"):  # hcp:<cells along c>
        return hcp_settings(L, int(lattice.split(":")[1]), ps, ts, qs, syms)
    return fcc_settings(L, ps, ts, qs, syms)


def golden_model(g):
    """Rebuild the settings/model of a golden case and check it is the generated one."""
    from cemc_gb300.lattice import seeded_ecis, with_background
    from cemc_gb300.tables import CEModel
    ps, ts, qs = (int(x) for x in g["shells"])
    syms = [str(s) for s in g["species"]]
    lattice = str(g["lattice"]) if "lattice" in g else "fcc"
    s = settings_for(lattice, int(g["L"]), ps, ts, qs, syms)
    bg = str(g["background"]) if "background" in g else ""
    if bg:
        s = with_background(s, bg)
    eci = seeded_ecis(s.cset, 0)
    m = CEModel(s, list(eci))
    return s, m, eci


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle
