"""The allocation-free entry point (lcg_align_score_static) against the
allocating one (lcg_align_pairs), through the C ABI, on a GPU.

lcg_align_score_static exists for callers that must not allocate device
memory while they run (CUDA-graph recording, memory owned by another
framework, real-time loops): it keeps all its device data in one fixed
file-scope device array instead of cudaMalloc'd buffers. Its scores must equal
lcg_align_pairs' exactly (integer scores), call after call, even though every
call reuses the same array. This file is collected last on purpose.
"""
import ctypes as C

import pytest

from golden_io import Golden
from locarna_gb300.abi import lcg_align_opts, lcg_pair_tables, make_opts

CASES = ["c150_global", "c120_opening0", "c200_global", "c150_freeright", "c150_nolp", "h150_stack",
         "h150_newstack_nolp"]


def _static_fn():
    from locarna_gb300.build import build_engine
    from locarna_gb300.engine import load_library
    build_engine()
    lib = load_library()
    fn = lib.lcg_align_score_static
    fn.argtypes = [C.POINTER(lcg_pair_tables), C.POINTER(lcg_align_opts), C.POINTER(C.c_int64),
                   C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.c_void_p]
    fn.restype = C.c_int32
    return lib, fn


def _static_score(lib, fn, g):
    opts = make_opts(do_trace=False, **g.align_kwargs())
    ct = g.tables.to_c()
    s, i, j = C.c_int64(), C.c_int32(), C.c_int32()
    rc = fn(C.byref(ct), C.byref(opts), C.byref(s), C.byref(i), C.byref(j), None)
    assert rc == 0, lib.lcg_last_error().decode()
    return s.value, (i.value, j.value)


@pytest.mark.gpu
def test_static_entry_point_matches_allocating_entry_point():
    from locarna_gb300.engine import Engine
    lib, fn = _static_fn()
    goldens = [Golden(n) for n in CASES]
    eng = Engine(0)
    try:
        expected = [eng.align_pairs([g.tables], do_trace=False, **g.align_kwargs())[0] for g in goldens]
    finally:
        eng.close()
    for _ in range(2):  # two calls in a row per case: the shared array is reused
        for g, exp in zip(goldens, expected):
            score, end = _static_score(lib, fn, g)
            assert score == exp.score == g.score, g.name
            assert end == exp.max_ij, g.name


@pytest.mark.gpu
def test_static_entry_point_rejects_unsupported_options():
    lib, fn = _static_fn()
    g = Golden("c60_short")
    ct = g.tables.to_c()
    s = C.c_int64()
    opts = make_opts(do_trace=True)
    assert fn(C.byref(ct), C.byref(opts), C.byref(s), None, None, None) != 0
    assert b"score only" in lib.lcg_last_error()
