"""Time the reference's own Metropolis drivers over its compiled CEUpdater (TEST / MEASUREMENT ONLY).

Loads the UNMODIFIED cemc/mcmc/montecarlo.py and sgc_montecarlo.py from the
reference tree by path and runs ``runMC(mode="fixed", steps=S, equil=False)``
on the compiled reference updater (oracle/_ref, built by build_ref.sh).  ASE,
CLEASE and the package __init__ (which imports every sampler of the package)
are not available, so these stand-ins are registered: ``ase.units`` (kB, kJ,
mol), ``ase.io.trajectory.TrajectoryWriter`` and ``cemc_cpp_code.PyClusterTracker``
(imported, never used by the two drivers), a bare ``cemc.mcmc`` package, and a
small calculator exposing the methods the drivers call on the reference's
``CE`` (cemc/ce_calculator.py:319-395).  Runs only where the reference tree is
present.

    CEMC_REFERENCE=<reference tree> python oracle/time_reference_runmc.py [--steps 20000]
"""
from __future__ import annotations

import argparse
import importlib.util
import json
import os
import sys
import time
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
REF = os.environ.get("CEMC_REFERENCE", "")
if not os.path.isdir(os.path.join(REF, "cemc")):
    sys.exit("set CEMC_REFERENCE to the reference source tree (it holds cemc/ and cpp/)")
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

KB_ASE = 8.617330337217213e-05  # ase.units.kB (CODATA 2014)


def _stub(name, **attrs):
    m = types.ModuleType(name)
    m.__dict__.update(attrs)
    sys.modules[name] = m
    return m


def load_reference_drivers():
    import oracle as O
    O.reference_module()  # registers ase.clease.tools for the updater
    ase = sys.modules.get("ase") or _stub("ase")
    ase.units = _stub("ase.units", kB=KB_ASE, kJ=1.0 / 96.48533212331002, mol=6.022140857e23)
    ase.io = _stub("ase.io")
    ase.io.trajectory = _stub("ase.io.trajectory", TrajectoryWriter=object)
    _stub("cemc_cpp_code", PyClusterTracker=object)
    cemc = _stub("cemc")
    cemc.__path__ = []
    mcmc = _stub("cemc.mcmc")
    mcmc.__path__ = []
    cemc.mcmc = mcmc

    def load(mod):
        spec = importlib.util.spec_from_file_location("cemc.mcmc." + mod, os.path.join(REF, "cemc", "mcmc", mod + ".py"))
        m = importlib.util.module_from_spec(spec)
        sys.modules["cemc.mcmc." + mod] = m
        spec.loader.exec_module(m)
        setattr(mcmc, mod, m)
        return m

    for mod in ("averager", "util", "exponential_filter", "swap_move_index_tracker", "bias_potential"):
        load(mod)
    mcmc.BiasPotential = mcmc.bias_potential.BiasPotential
    load("mc_observers")
    mc = load("montecarlo")
    sgc = load("sgc_montecarlo")
    return mc.Montecarlo, sgc.SGCMonteCarlo


class RefCalc:
    """The calculator methods the reference drivers call, over the compiled PyCEUpdater."""

    def __init__(self, settings, model, occ, eci):
        import oracle as O
        self.BC = settings
        self.eci = dict(eci)
        orc = O.Oracle(model)
        cf = orc.full_cf(occ)
        self.updater, self.atoms = O.make_reference_updater(settings, model.symbols_of(occ),
                                                            dict(zip(model.eci_names, cf)), self.eci)
        self.atoms_list = self.atoms
        self.results = {}

    def get_energy(self):
        return self.updater.get_energy()

    def calculate(self, atoms, properties, system_changes):
        e = self.updater.calculate(system_changes)
        self.cf = self.updater.get_cf()  # the reference builds the dict every trial (ce_calculator.py:362)
        return e

    def clear_history(self):
        self.updater.clear_history()

    def undo_changes(self):
        self.updater.undo_changes()

    def update_cf(self, change):
        self.updater.update_cf(change)

    def get_cf(self):
        return self.updater.get_cf()

    def update_ecis(self, eci):
        self.eci = eci
        self.updater.set_ecis(eci)

    def get_singlets(self):
        return self.updater.get_singlets()

    def vib_energy(self, T):
        return 0.0

    def include_linvib_in_ecis(self, T):
        pass


class RefAtoms(list):
    def __init__(self, atoms, calc):
        super().__init__(atoms)
        self._calc = calc

    def get_calculator(self):
        return self._calc


def main(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--steps", type=int, default=20000)
    args = p.parse_args(argv)
    if not os.path.isdir(os.path.join(REF, "cemc", "mcmc")):
        print(json.dumps({"unavailable": "reference tree not present"}))
        return 0
    import logging
    logging.getLogger("MonteCarlo").setLevel(logging.WARNING)
    Montecarlo, SGCMonteCarlo = load_reference_drivers()
    from cemc_gb300.lattice import fcc_settings, seeded_ecis
    from cemc_gb300.tables import CEModel
    out = []
    for L, label in ((8, "canonical swap, 2048 sites (binary FCC 8^3)"),
                     (16, "semi-grand-canonical flip, 16384 sites (binary FCC 16^3)")):
        s = fcc_settings(L, 4, 2, 1, ["Al", "Mg"])
        eci = seeded_ecis(s.cset, 0)
        m = CEModel(s, list(eci))
        rng = np.random.default_rng(0)
        occ = np.zeros(m.n_sites, dtype=np.int8)
        occ[rng.permutation(m.n_sites)[: m.n_sites // 2]] = 1
        devnull = os.open(os.devnull, os.O_WRONLY)
        saved = os.dup(1), os.dup(2)
        os.dup2(devnull, 1)
        os.dup2(devnull, 2)
        try:
            calc = RefCalc(s, m, occ, eci)
        finally:
            os.dup2(saved[0], 1)
            os.dup2(saved[1], 2)
        atoms = RefAtoms(calc.atoms, calc)
        np.random.seed(0)
        if L == 8:
            mc = Montecarlo(atoms, 800.0)
            t0 = time.perf_counter()
            mc.runMC(mode="fixed", steps=args.steps, equil=False)
        else:
            mc = SGCMonteCarlo(atoms, 800.0, symbols=["Al", "Mg"])
            t0 = time.perf_counter()
            mc.runMC(mode="fixed", steps=args.steps, chem_potential={"c1_0": 0.0}, equil=False)
        dt = time.perf_counter() - t0
        trials = args.steps + 1001  # runMC adds one step and the 1000-step bias probe (montecarlo.py:765,799)
        out.append({"workload": label, "trials": trials, "seconds": dt, "trials_per_s": trials / dt,
                    "threads": 1, "cpu": os.uname().machine})
    print(json.dumps(out))
    return 0


if __name__ == "__main__":
    sys.exit(main())
