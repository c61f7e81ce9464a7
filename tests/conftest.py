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
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.endswith(".npz"))


def load_golden(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False)
    return {k: d[k] for k in d.files}


def golden_model(g):
    """Rebuild the settings/model of a golden case and check it is the generated one."""
    from cemc_gb300.lattice import fcc_settings, seeded_ecis, with_background
    from cemc_gb300.tables import CEModel
    ps, ts, qs = (int(x) for x in g["shells"])
    syms = [str(s) for s in g["species"]]
    s = fcc_settings(int(g["L"]), ps, ts, qs, syms)
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
