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


def oracle_kbest(tables, k, threshold=-1000000, stale=False, **kw):
    """Aligner::suboptimal restated (oracle/kbest_oracle.cc): up to k hits,
    each an AlignResult whose score is the hit's score. With stale=True also
    the number of interval top levels whose argmax the reference takes from a
    cell outside the band."""
    lib = load_oracle()
    if not getattr(lib, "_kbest_ready", False):
        lib.lcg_oracle_kbest.argtypes = [C.POINTER(lcg_pair_tables), C.POINTER(lcg_align_opts), C.c_int,
                                         C.c_longlong, C.POINTER(lcg_align_result), C.POINTER(C.c_int)]
        lib.lcg_oracle_kbest.restype = C.c_int
        lib._kbest_ready = True
    o = make_opts(**kw)
    bufs = [ResultBuffers(tables.len_a, tables.len_b) for _ in range(k)]
    arr = (lcg_align_result * k)(*[b.c for b in bufs])
    ct = tables.to_c()
    ns = C.c_int(0)
    nh = lib.lcg_oracle_kbest(C.byref(ct), C.byref(o), k, threshold, arr, C.byref(ns))
    assert nh >= 0
    out = []
    for h in range(nh):
        bufs[h].c = arr[h]
        out.append(bufs[h].decode())
    return (out, ns.value) if stale else out


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


_pflib = None


def load_pf_oracle():
    global _pflib
    if _pflib is None:
        from locarna_gb300.build import build_oracle
        build_oracle()
        lib = C.CDLL(os.path.join(ROOT, "oracle", "_build", "libpforacle.so"))
        lib.lcg_oracle_pf.argtypes = [C.POINTER(lcg_pair_tables), C.c_double, C.c_double, C.c_double,
                                      C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                      C.POINTER(C.c_double)]
        lib.lcg_oracle_pf.restype = C.c_int
        _pflib = lib
    return _pflib


def oracle_pf(tables, temperature=300.0, pf_scale=1.0, min_am_prob=0.0, include_am=False, probs=True):
    """LocARNA-P oracle: returns (Z, am_prob per arc match, bm_prob (n+1)x(m+1))."""
    import numpy as np
    lib = load_pf_oracle()
    ct = tables.to_c()
    Z = C.c_double()
    am = np.zeros(max(1, tables.num_arcmatches), dtype=np.float64)
    bm = np.zeros((tables.len_a + 1) * (tables.len_b + 1), dtype=np.float64)
    P = C.POINTER(C.c_double)
    rc = lib.lcg_oracle_pf(C.byref(ct), temperature, pf_scale, min_am_prob, int(include_am), C.byref(Z),
                           am.ctypes.data_as(P) if probs else None, bm.ctypes.data_as(P) if probs else None)
    assert rc == 0
    return Z.value, am[:tables.num_arcmatches], bm.reshape(tables.len_a + 1, tables.len_b + 1)
