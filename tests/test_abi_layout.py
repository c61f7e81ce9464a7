"""The ctypes mirrors of the C ABI structs (cemc_gb300/_lib.py) against include/cemc_gb300.h.

A small C program compiled with the host compiler prints sizeof / offsetof of every field of
cemc_accum, cemc_geometry_desc and cemc_run_desc; the ctypes structures must agree field by
field, so a descriptor passed from Python lands in the library unchanged.  No GPU needed.
"""
import ctypes as C
import os
import shutil
import subprocess

import pytest

from conftest import ROOT


def _c_layout(tmp_path, structs, header="cemc_gb300.h", include=os.path.join(ROOT, "include")):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no host C compiler")
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "%s"' % header, "int main(void) {"]
    for name, fields in structs.items():
        lines.append('  printf("%s size %%zu\\n", sizeof(%s));' % (name, name))
        for f in fields:
            lines.append('  printf("%s %s %%zu\\n", offsetof(%s, %s));' % (name, f, name, f))
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", include, str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    res = {}
    for line in out.splitlines():
        name, field, value = line.split()
        res[(name, field)] = int(value)
    return res


def test_ctypes_structs_match_the_c_header(tmp_path):
    from cemc_gb300 import _lib
    pairs = {"cemc_accum": _lib.Accum, "cemc_geometry_desc": _lib.GeometryDesc, "cemc_run_desc": _lib.RunDesc}
    structs = {name: [f[0] for f in cls._fields_] for name, cls in pairs.items()}
    c = _c_layout(tmp_path, structs)
    for name, cls in pairs.items():
        assert C.sizeof(cls) == c[(name, "size")], name
        for f in structs[name]:
            assert getattr(cls, f).offset == c[(name, f)], (name, f)


def test_oracle_ctypes_structs_match_its_header(tmp_path):
    """The same check for the oracle's model, chain and trace structs (oracle/ce_oracle.h)."""
    import oracle as O
    pairs = {"orc_model": O.OrcModel, "orc_chain": O.OrcChain, "orc_trace": O.OrcTrace}
    structs = {name: [f[0] for f in cls._fields_] for name, cls in pairs.items()}
    c = _c_layout(tmp_path, structs, header="ce_oracle.h", include=os.path.join(ROOT, "oracle"))
    for name, cls in pairs.items():
        assert C.sizeof(cls) == c[(name, "size")], name
        for f in structs[name]:
            assert getattr(cls, f).offset == c[(name, f)], (name, f)
