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
    assert lib.lcg_abi_version() == 1
