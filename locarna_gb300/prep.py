"""Host preparation (lcg_prepare_pair): PP 2.0 texts -> PairTables.

Mirror of the reference locarna driver's input side (src/locarna.cc:398-703):
the options have the command line's names and defaults.
"""
import ctypes as C
import threading

import numpy as np

from .abi import LCG_FREE_LEFT_1, PairTables, lcg_pair_tables, lcg_pf_grad_spec
from .engine import LcgError, load_library


class lcg_prep_opts(C.Structure):
    _fields_ = [
        ("min_prob", C.c_double), ("indel", C.c_int32), ("indel_opening", C.c_int32),
        ("struct_weight", C.c_int32), ("tau", C.c_int32), ("exclusion", C.c_int32),
        ("match", C.c_int32), ("mismatch", C.c_int32), ("use_ribosum", C.c_int32),
        ("min_trace_probability", C.c_double), ("max_diff", C.c_int32),
        ("max_diff_am", C.c_int32), ("max_diff_at_am", C.c_int32),
        ("temperature_alipf", C.c_int32), ("sequ_local", C.c_int32),
        ("free_endgaps", C.c_int32), ("pf_precision", C.c_int32), ("exp_prob", C.c_double),
        ("stacking", C.c_int32), ("new_stacking", C.c_int32), ("relaxed_anchors", C.c_int32),
        ("unpaired_penalty", C.c_int32),
    ]


_ready = False
_ready_lock = threading.Lock()


def _lib():
    # ctypes caches a function object per attribute on first access; two
    # threads that race on that first access can each cache their own object,
    # so the signatures are declared once, under a lock.
    global _ready
    lib = load_library()
    if _ready:
        return lib
    with _ready_lock:
        if _ready:
            return lib
        lib.lcg_prep_opts_default.argtypes = [C.POINTER(lcg_prep_opts)]
        lib.lcg_prep_opts_default.restype = None
        lib.lcg_prepare_pair.argtypes = [C.c_char_p, C.c_char_p, C.POINTER(lcg_prep_opts), C.POINTER(C.c_void_p)]
        lib.lcg_prepare_pair.restype = C.c_int32
        lib.lcg_prepared_tables.argtypes = [C.c_void_p, C.POINTER(lcg_pair_tables)]
        lib.lcg_prepared_tables.restype = C.c_int32
        lib.lcg_prepared_sequence.argtypes = [C.c_void_p, C.c_int32]
        lib.lcg_prepared_sequence.restype = C.c_char_p
        lib.lcg_prepared_envelope_ok.argtypes = [C.c_void_p]
        lib.lcg_prepared_envelope_ok.restype = C.c_int32
        lib.lcg_prepared_free.argtypes = [C.c_void_p]
        lib.lcg_prepared_grad_spec.argtypes = [C.c_void_p, C.POINTER(lcg_pf_grad_spec)]
        lib.lcg_prepared_grad_spec.restype = C.c_int32
        lib.lcg_prepared_free.restype = C.c_int32
        lib.lcg_prepare_pairs.argtypes = [C.c_void_p, C.POINTER(C.c_char_p), C.POINTER(C.c_char_p), C.c_int32,
                                          C.POINTER(lcg_prep_opts), C.POINTER(C.c_void_p), C.POINTER(C.c_int32)]
        lib.lcg_prepare_pairs.restype = C.c_int32
        _ready = True
    return lib


def _fe_bits(spec):
    bits = 0
    for k, ch in enumerate(spec[:4]):
        if ch == "+":
            bits |= LCG_FREE_LEFT_1 << k
    return bits


def prep_options(**kw):
    lib = _lib()
    o = lcg_prep_opts()
    lib.lcg_prep_opts_default(C.byref(o))
    for k, v in kw.items():
        if k == "free_endgaps" and isinstance(v, str):
            v = _fe_bits(v)
        if not hasattr(o, k):
            raise KeyError(f"unknown preparation option {k}")
        setattr(o, k, v)
    return o


def _arr(ptr, n):
    if n == 0:
        return np.zeros(0, dtype=np.int32)
    return np.ctypeslib.as_array(ptr, shape=(n,)).copy()


def prepare_pair(pp_a, pp_b, **kw):
    """Build the tables of one pair from two PP 2.0 texts."""
    lib = _lib()
    o = prep_options(**kw)
    h = C.c_void_p()
    rc = lib.lcg_prepare_pair(pp_a.encode(), pp_b.encode(), C.byref(o), C.byref(h))
    if rc != 0:
        raise LcgError(rc, lib.lcg_last_error().decode())
    try:
        return _tables_of(lib, h)
    finally:
        lib.lcg_prepared_free(h)


def prepare_pairs(engine, pp_pairs, **kw):
    """lcg_prepare_pairs: the tables of many pairs [(pp_a, pp_b), ...] with the
    sequence envelopes computed on the engine's GPU. Returns (tables, number of
    pairs whose envelope took the host path)."""
    lib = _lib()
    o = prep_options(**kw)
    n = len(pp_pairs)
    enc_a = [a.encode() for a, _ in pp_pairs]
    enc_b = [b.encode() for _, b in pp_pairs]
    arr_a = (C.c_char_p * n)(*enc_a)
    arr_b = (C.c_char_p * n)(*enc_b)
    hs = (C.c_void_p * n)()
    nhost = C.c_int32()
    rc = lib.lcg_prepare_pairs(engine.h, arr_a, arr_b, n, C.byref(o), hs, C.byref(nhost))
    if rc != 0:
        raise LcgError(rc, lib.lcg_last_error().decode())
    try:
        return [_tables_of(lib, C.c_void_p(h)) for h in hs], nhost.value
    finally:
        for h in hs:
            if h:
                lib.lcg_prepared_free(C.c_void_p(h))


class PreparedBatch:
    """Handles of lcg_prepare_pairs kept alive: the tables stay in the
    library's memory and c_tables() gives the lcg_pair_tables views for
    lcg_align_pairs without copying them into Python. close() frees them."""

    def __init__(self, lib, handles, host_envelopes):
        self.lib, self.handles, self.host_envelopes = lib, handles, host_envelopes

    def __len__(self):
        return len(self.handles)

    def c_tables(self):
        arr = (lcg_pair_tables * len(self.handles))()
        for k, h in enumerate(self.handles):
            self.lib.lcg_prepared_tables(h, C.byref(arr[k]))
        return arr

    def close(self):
        for h in self.handles:
            if h:
                self.lib.lcg_prepared_free(h)
        self.handles = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def prepare_pairs_batch(engine, pp_pairs, **kw):
    """lcg_prepare_pairs returning the prepared handles (PreparedBatch)."""
    lib = _lib()
    o = prep_options(**kw)
    n = len(pp_pairs)
    arr_a = (C.c_char_p * n)(*[a.encode() for a, _ in pp_pairs])
    arr_b = (C.c_char_p * n)(*[b.encode() for _, b in pp_pairs])
    hs = (C.c_void_p * n)()
    nhost = C.c_int32()
    rc = lib.lcg_prepare_pairs(engine.h, arr_a, arr_b, n, C.byref(o), hs, C.byref(nhost))
    if rc != 0:
        raise LcgError(rc, lib.lcg_last_error().decode())
    return PreparedBatch(lib, [C.c_void_p(h) for h in hs], nhost.value)


def _tables_of(lib, h):
    """PairTables of a prepared handle (copies)."""
    t = lcg_pair_tables()
    lib.lcg_prepared_tables(h, C.byref(t))
    n, m = t.len_a, t.len_b
    na, nb, nam = t.num_arcs_a, t.num_arcs_b, t.num_arcmatches
    pt = PairTables(
        n, m, _arr(t.sigma, (n + 1) * (m + 1)), _arr(t.gap_a, n + 1), _arr(t.gap_b, m + 1),
        t.indel_opening, t.exclusion, _arr(t.arcs_a, 2 * na), _arr(t.arcs_b, 2 * nb),
        _arr(t.am_arcs, 2 * nam), _arr(t.am_score, nam), _arr(t.min_col, n + 1), _arr(t.max_col, n + 1),
        seq_a=lib.lcg_prepared_sequence(h, 0).decode(), seq_b=lib.lcg_prepared_sequence(h, 1).decode(),
        am_stack_score=_arr(t.am_stack_score, nam) if t.am_stack_score else None,
        am_stackable=(np.ctypeslib.as_array(t.am_stackable, shape=(nam,)).copy() if nam else np.zeros(0, np.uint8))
        if t.am_stack_score else None,
        anchors=({"match_lo": _arr(t.match_lo, n + 1), "match_hi": _arr(t.match_hi, n + 1),
                  "del_lo": _arr(t.del_lo, n + 1), "del_hi": _arr(t.del_hi, n + 1),
                  "ins_lo": _arr(t.ins_lo, m + 1), "ins_hi": _arr(t.ins_hi, m + 1)} if t.match_lo else None),
        right_anchor=(t.right_anchor_a, t.right_anchor_b), left_anchor=(t.left_anchor_a, t.left_anchor_b))
    pt.name_a = lib.lcg_prepared_sequence(h, 2).decode()
    pt.name_b = lib.lcg_prepared_sequence(h, 3).decode()
    pt.envelope_ok = bool(lib.lcg_prepared_envelope_ok(h))
    g = lcg_pf_grad_spec()
    if lib.lcg_prepared_grad_spec(h, C.byref(g)) == 0:
        pt.code_a = np.ctypeslib.as_array(g.code_a, shape=(n + 1,)).copy()
        pt.code_b = np.ctypeslib.as_array(g.code_b, shape=(m + 1,)).copy()
        pt.am_dsw = (np.ctypeslib.as_array(g.am_dscore_dsw, shape=(nam,)).copy() if nam
                     else np.zeros(0))
    return pt
