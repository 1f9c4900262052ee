"""ctypes access to the plain-C oracle (oracle/sankoff_oracle.c). Test infrastructure."""
import ctypes as C
import os

from locarna_gb300.abi import (ResultBuffers, lcg_align_opts, lcg_align_result,
                               lcg_pair_tables, lcg_work_counts, make_opts)

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
_lib = None


def load_oracle():
    global _lib
    if _lib is None:
        from locarna_gb300.build import build_oracle
        path = build_oracle()
        lib = C.CDLL(path)
        lib.lcg_oracle_align.argtypes = [C.POINTER(lcg_pair_tables), C.POINTER(lcg_align_opts),
                                         C.POINTER(lcg_align_result), C.POINTER(lcg_work_counts)]
        lib.lcg_oracle_align.restype = C.c_int
        _lib = lib
    return _lib


def oracle_align(tables, counts=False, **kw):
    lib = load_oracle()
    o = make_opts(**kw)
    rb = ResultBuffers(tables.len_a, tables.len_b)
    cnt = lcg_work_counts()
    ct = tables.to_c()
    rc = lib.lcg_oracle_align(C.byref(ct), C.byref(o), C.byref(rb.c), C.byref(cnt) if counts else None)
    assert rc == 0
    r = rb.decode()
    if counts:
        return r, cnt
    return r
