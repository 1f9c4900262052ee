"""The C-ABI library exports every entry point its header declares (CPU)."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    names = []
    for h in os.listdir(os.path.join(ROOT, "include")):
        if not h.endswith(".h"):
            continue
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_ \*]*?\b(lcg_[a-z0-9_]+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = header_functions()
    assert "lcg_align_pairs" in names and "lcg_engine_create" in names


def test_library_exports_every_declared_symbol():
    from locarna_gb300.build import build_engine
    lib = C.CDLL(build_engine())
    missing = [n for n in header_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_abi_version():
    from locarna_gb300.build import build_engine
    lib = C.CDLL(build_engine())
    lib.lcg_abi_version.restype = C.c_int32
    assert lib.lcg_abi_version() == 4


def test_ctypes_structs_match_c_layout(tmp_path):
    """Every ctypes mirror in locarna_gb300.abi / .prep has the size and field offsets
    the C compiler gives the header's struct of the same name."""
    import subprocess

    from locarna_gb300 import abi, prep
    structs = {name: cls for mod in (abi, prep) for name, cls in vars(mod).items()
               if name.startswith("lcg_") and isinstance(cls, type) and issubclass(cls, C.Structure)}
    assert "lcg_pf_opts" in structs and "lcg_pair_tables" in structs and "lcg_prep_opts" in structs
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "locarna_gb300.h"', "int main(void) {"]
    for name, cls in sorted(structs.items()):
        lines.append(f'printf("{name} %zu\\n", sizeof({name}));')
        for f in cls._fields_:
            lines.append(f'printf("{name}.{f[0]} %zu\\n", offsetof({name}, {f[0]}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    got = dict(l.split() for l in subprocess.check_output([str(exe)], text=True).splitlines())
    for name, cls in structs.items():
        assert int(got[name]) == C.sizeof(cls), name
        for f in cls._fields_:
            assert int(got[f"{name}.{f[0]}"]) == getattr(cls, f[0]).offset, (name, f[0])
