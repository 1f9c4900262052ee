"""Bounded device waits (CPU host, GPU kernel): a consumer that waits for an
arc-match entry nobody writes gives up after its iteration limit, the call
returns LCG_ERR_TIMEOUT, and the context stays usable for the next call.

The test builds a variant of the library (its own folder) with a short wait
limit (LCG_SPIN_LIMIT) and one D write left out per pair
(LCG_TEST_DROP_LAST_D_WRITE: the last group's last write moved to a row the
group never reaches, so the top level waits for that entry until the limit).
It runs in a child process that loads only that variant. No fault, trap or
unbounded loop is involved: the wait polls a flag that stays unset and
returns an error status.
"""
import os
import subprocess
import sys
import textwrap

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = textwrap.dedent("""
    import ctypes as C, sys, time
    sys.path.insert(0, {root!r}); sys.path.insert(0, {tests!r})
    from golden_io import Golden
    from locarna_gb300.abi import PairTables, ResultBuffers, lcg_align_opts, lcg_align_result, lcg_pair_tables, make_opts
    from oracle_ffi import oracle_align
    lib = C.CDLL({lib!r})
    lib.lcg_engine_create.argtypes = [C.c_int32, C.c_void_p, C.POINTER(C.c_void_p)]
    lib.lcg_align_pairs.argtypes = [C.c_void_p, C.POINTER(lcg_pair_tables), C.c_int32, C.POINTER(lcg_align_opts),
                                    C.POINTER(lcg_align_result)]
    lib.lcg_last_error.restype = C.c_char_p
    lib.lcg_engine_destroy.argtypes = [C.c_void_p]
    h = C.c_void_p()
    assert lib.lcg_engine_create(0, None, C.byref(h)) == 0
    def run(t):
        rb = ResultBuffers(t.len_a, t.len_b)
        ct = t.to_c()
        o = make_opts()
        rc = lib.lcg_align_pairs(h, C.byref(ct), 1, C.byref(o), C.byref(rb.c))
        return rc, rb.decode()
    g = Golden("c150_global")
    t0 = time.time()
    rc, _ = run(g.tables)
    print("first", rc, lib.lcg_last_error().decode(), round(time.time() - t0, 3))
    t = g.tables
    bare = PairTables(t.len_a, t.len_b, t.sigma, t.gap_a, t.gap_b, t.indel_opening, t.exclusion,
                      [], [], [], [], t.min_col, t.max_col)
    rc2, r = run(bare)
    ref = oracle_align(bare)
    print("second", rc2, r.score == ref.score and r.edges == ref.edges)
    lib.lcg_engine_destroy(h)
""")


@pytest.mark.gpu
def test_unwritten_entry_times_out_and_the_context_stays_usable(tmp_path):
    from locarna_gb300.build import OUT, build_engine
    out = os.path.join(OUT, "wait_timeout_test")
    lib = build_engine(out=out, defs=["-DLCG_SPIN_LIMIT=(1ll<<12)", "-DLCG_TEST_DROP_LAST_D_WRITE"])
    code = CHILD.format(root=ROOT, tests=os.path.join(ROOT, "tests"), lib=lib)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = dict(l.split(" ", 1) for l in r.stdout.strip().splitlines())
    rc, rest = lines["first"].split(" ", 1)
    assert int(rc) == -5 and "timed out" in rest, lines["first"]  # LCG_ERR_TIMEOUT
    assert lines["second"] == "0 True", lines["second"]
