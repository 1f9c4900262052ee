"""The allocation-free entry point (lcg_align_score_static) against the
allocating one (lcg_align_pairs), through the C ABI, on a GPU.

lcg_align_score_static exists for callers that cannot allocate device memory
while they run (GPU memory reserved up front by another framework's
allocator, real-time loops in which cudaMalloc / cudaFree would synchronise
the device): it keeps all its device data in one fixed file-scope device
array instead of cudaMalloc'd buffers. Its scores must equal lcg_align_pairs'
exactly (integer scores), call after call, even though every call reuses the
same array; the device's free memory must not move across calls; pairs
beyond the array's size are refused with LCG_ERR_RANGE. This file is
collected last on purpose.
"""
import ctypes as C

import pytest

from golden_io import Golden
from locarna_gb300.abi import lcg_align_opts, lcg_pair_tables, make_opts

CASES = ["c150_global", "c120_opening0", "c200_global", "c150_freeright", "c150_seqlocal", "c150_nolp",
         "h150_stack", "h150_newstack_nolp", "a150_anchors"]
LCG_ERR_RANGE = -4


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


def _static_call(fn, g, tables=None):
    opts = make_opts(do_trace=False, **(g.align_kwargs() if g is not None else {}))
    ct = (tables if tables is not None else g.tables).to_c()
    s, i, j = C.c_int64(), C.c_int32(), C.c_int32()
    rc = fn(C.byref(ct), C.byref(opts), C.byref(s), C.byref(i), C.byref(j), None)
    return rc, s.value, (i.value, j.value)


def _static_score(lib, fn, g):
    rc, score, end = _static_call(fn, g)
    assert rc == 0, lib.lcg_last_error().decode()
    return score, end


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
def test_static_entry_point_allocates_no_device_memory():
    import torch
    lib, fn = _static_fn()
    goldens = [Golden(n) for n in CASES]
    for g in goldens:  # first calls: address look-up and lazy kernel loading
        _static_score(lib, fn, g)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        for g in goldens:
            _static_score(lib, fn, g)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)


@pytest.mark.gpu
def test_static_entry_point_rejects_pairs_beyond_its_array():
    from locarna_gb300.prep import prepare_pair
    from locarna_gb300.synth import make_rna
    lib, fn = _static_fn()
    # 3000 x 3000 nt without an envelope: the top-level matrix alone is 36 MB,
    # the per-cell arc-match index as much again
    a, b = make_rna(3000, 71, q=0.0), make_rna(3000, 72, q=0.0)
    big = prepare_pair(a.to_pp(), b.to_pp(), min_trace_probability=0.0)
    rc, _, _ = _static_call(fn, None, big)
    assert rc == LCG_ERR_RANGE
    msg = lib.lcg_last_error().decode()
    assert "limit" in msg and str(64 << 20) in msg, msg
    # the array is still usable after a refusal
    g = Golden("c150_global")
    assert _static_score(lib, fn, g)[0] == g.score


@pytest.mark.gpu
def test_static_entry_point_rejects_unsupported_options():
    lib, fn = _static_fn()
    g = Golden("c60_short")
    ct = g.tables.to_c()
    s = C.c_int64()
    opts = make_opts(do_trace=True)
    assert fn(C.byref(ct), C.byref(opts), C.byref(s), None, None, None) != 0
    assert b"score only" in lib.lcg_last_error()
