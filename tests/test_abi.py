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


def test_prepared_rows_and_anchor_lines():
    """lcg_prepared_row: the inputs' rows and names, and (which 4 / 5) their
    #A<k> anchor lines, the blocks of each k concatenated; NULL past the end
    and for an unknown `which`."""
    import sys
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from golden_io import Golden
    from locarna_gb300.prep import _lib, prep_options
    lib = _lib()
    lib.lcg_prepared_row.argtypes = [C.c_void_p, C.c_int32, C.c_int32]
    lib.lcg_prepared_row.restype = C.c_char_p
    g = Golden("a150_anchors")

    def anchor_lines(pp):
        lines = {}
        for line in pp.splitlines():
            if line.startswith("#SECTION"):
                break
            if line.startswith("#A") and line[2:3].isdigit():
                k, s = line[2:].split()
                lines[int(k)] = lines.get(int(k), "") + s
        return [lines[k] for k in sorted(lines)]

    h = C.c_void_p()
    o = prep_options()
    assert lib.lcg_prepare_pair(g.pp_a.encode(), g.pp_b.encode(), C.byref(o), C.byref(h)) == 0
    try:
        for side, pp in ((0, g.pp_a), (1, g.pp_b)):
            want = anchor_lines(pp)
            assert want and len(want[0]) == len(lib.lcg_prepared_row(h, side, 0))
            got = []
            while (r := lib.lcg_prepared_row(h, side + 4, len(got))) is not None:
                got.append(r.decode())
            assert got == want
            assert lib.lcg_prepared_row(h, side + 2, 0).decode()  # the row's name
        assert lib.lcg_prepared_row(h, 6, 0) is None
        assert lib.lcg_prepared_row(h, 0, 1) is None  # single-sequence inputs: one row
    finally:
        lib.lcg_prepared_free(h)
