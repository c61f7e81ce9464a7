"""Compile libcemc_gb300.so for sm_103a with nvcc (translation units in parallel)."""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libcemc_gb300.so")
UNITS = ["cemc_mc.cu", "cemc_field.cu", "cemc_cf.cu", "cemc_abi.cu"]
HEADERS = ["cemc_device.cuh", "cemc_launch.h", "cemc_kernels.h", "cemc_spin.h", "cemc_field.h", "philox.h"]
NVCC_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-lineinfo", "-O3", "-std=c++17",
              "-Xcompiler", "-fPIC", "-Xcompiler", "-O2"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(SRC, f) for f in UNITS + HEADERS]
    deps.append(os.path.join(HERE, "..", "include", "cemc_gb300.h"))
    return any(os.path.getmtime(p) > t for p in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()

    def compile_unit(unit: str) -> str:
        obj = os.path.join(OUT, unit.replace(".cu", ".o"))
        cmd = [nvcc, *NVCC_FLAGS, "-c", os.path.join(SRC, unit), "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        subprocess.run(cmd, check=True)
        return obj

    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(compile_unit, UNITS))
    tmp = LIB + ".tmp"
    subprocess.run([nvcc, "-shared", "-gencode", "arch=compute_103a,code=sm_103a", *objs, "-o", tmp,
                    "-lcudart"], check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
