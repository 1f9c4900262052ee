"""ctypes mirror of include/locarna_gb300.h.

The structures here are byte-for-byte the C structures of the public C ABI;
``PairTables`` keeps the numpy arrays alive that a ``lcg_pair_tables`` points
into.
"""
import ctypes as C

import numpy as np

LCG_NEG_INF = -(1 << 40)
LCG_STACK_NONE = -(1 << 29)
LCG_FREE_LEFT_1, LCG_FREE_RIGHT_1, LCG_FREE_LEFT_2, LCG_FREE_RIGHT_2 = 1, 2, 4, 8

_P32 = C.POINTER(C.c_int32)


class lcg_pair_tables(C.Structure):
    _fields_ = [
        ("len_a", C.c_int32), ("len_b", C.c_int32),
        ("sigma", _P32), ("gap_a", _P32), ("gap_b", _P32),
        ("indel_opening", C.c_int32), ("exclusion", C.c_int32),
        ("num_arcs_a", C.c_int32), ("num_arcs_b", C.c_int32),
        ("arcs_a", _P32), ("arcs_b", _P32),
        ("num_arcmatches", C.c_int32),
        ("am_arcs", _P32), ("am_score", _P32),
        ("min_col", _P32), ("max_col", _P32),
        ("match_lo", _P32), ("match_hi", _P32),
        ("del_lo", _P32), ("del_hi", _P32),
        ("ins_lo", _P32), ("ins_hi", _P32),
        ("right_anchor_a", C.c_int32), ("right_anchor_b", C.c_int32),
        ("left_anchor_a", C.c_int32), ("left_anchor_b", C.c_int32),
        ("am_stack_score", _P32), ("am_stackable", C.POINTER(C.c_uint8)),
    ]


class lcg_align_opts(C.Structure):
    _fields_ = [("struct_local", C.c_int32), ("sequ_local", C.c_int32),
                ("free_endgaps", C.c_int32), ("do_trace", C.c_int32),
                ("no_lonely_pairs", C.c_int32), ("normalized", C.c_int32), ("normalized_L", C.c_int32),
                ("penalized", C.c_int32), ("position_penalty", C.c_int32)]


class lcg_align_result(C.Structure):
    _fields_ = [
        ("score", C.c_int64),
        ("max_i", C.c_int32), ("max_j", C.c_int32),
        ("min_i", C.c_int32), ("min_j", C.c_int32),
        ("num_edges", C.c_int32), ("num_traced_am", C.c_int32),
        ("edges", _P32), ("traced_am", _P32),
    ]


class lcg_work_counts(C.Structure):
    _fields_ = [("groups", C.c_int64), ("cells", C.c_int64),
                ("arc_terms", C.c_int64), ("valid_arc_terms", C.c_int64)]


LCG_TUNE_BUCKETS = 4


class lcg_tune_entry(C.Structure):
    _fields_ = [("max_len", C.c_int32), ("pairs_sampled", C.c_int32), ("blocks_per_sm", C.c_int32),
                ("wave_mb", C.c_double), ("best_ms", C.c_double), ("default_ms", C.c_double),
                ("trials", C.c_int32)]


_PD = C.POINTER(C.c_double)
_P8 = C.POINTER(C.c_int8)


class lcg_pf_opts(C.Structure):
    _fields_ = [("temperature", C.c_double), ("pf_scale", C.c_double), ("precision", C.c_int32),
                ("param_delta", C.c_double * 19), ("min_am_prob", C.c_double), ("min_bm_prob", C.c_double),
                ("gap_gradients", C.c_int32)]


class lcg_pf_grad_spec(C.Structure):
    _fields_ = [("code_a", _P8), ("code_b", _P8), ("am_dscore_dsw", _PD)]


class lcg_pf_result(C.Structure):
    _fields_ = [
        ("am_prob", _PD), ("bm_prob", _PD),
        ("log_z", C.c_double), ("gap_ext_uses", C.c_double), ("gap_open_uses", C.c_double),
        ("dlogz_dindel", C.c_double), ("dlogz_dindel_opening", C.c_double),
        ("dlogz_dstruct_weight", C.c_double), ("dlogz_dbasematch", C.c_double * 16),
    ]


def _i32(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.int32))


def _ptr(a):
    return a.ctypes.data_as(_P32) if a is not None else None


class PairTables:
    """Prepared tables of one pair (see lcg_pair_tables in the C header)."""

    FIELDS = ("sigma", "gap_a", "gap_b", "arcs_a", "arcs_b", "am_arcs",
              "am_score", "min_col", "max_col")
    ANCHOR_FIELDS = ("match_lo", "match_hi", "del_lo", "del_hi", "ins_lo", "ins_hi")

    def __init__(self, len_a, len_b, sigma, gap_a, gap_b, indel_opening,
                 exclusion, arcs_a, arcs_b, am_arcs, am_score, min_col,
                 max_col, anchors=None, right_anchor=(0, 0), left_anchor=None,
                 seq_a="", seq_b="", am_stack_score=None, am_stackable=None):
        self.len_a, self.len_b = int(len_a), int(len_b)
        self.sigma = _i32(sigma).reshape(-1)
        self.gap_a, self.gap_b = _i32(gap_a), _i32(gap_b)
        self.indel_opening, self.exclusion = int(indel_opening), int(exclusion)
        self.arcs_a = _i32(arcs_a).reshape(-1)
        self.arcs_b = _i32(arcs_b).reshape(-1)
        self.am_arcs = _i32(am_arcs).reshape(-1)
        self.am_score = _i32(am_score)
        self.min_col, self.max_col = _i32(min_col), _i32(max_col)
        self.anchors = None
        if anchors is not None:
            self.anchors = {k: _i32(anchors[k]) for k in self.ANCHOR_FIELDS}
        self.right_anchor = tuple(right_anchor)
        self.left_anchor = tuple(left_anchor) if left_anchor else (self.len_a + 1, self.len_b + 1)
        self.seq_a, self.seq_b = seq_a, seq_b
        # stacking (both None = off): Scoring::arcmatch(am, true) and is_stackable_am
        self.am_stack_score = None if am_stack_score is None else _i32(am_stack_score)
        self.am_stackable = (None if am_stackable is None else
                             np.ascontiguousarray(np.asarray(am_stackable, dtype=np.uint8)))
        self._check()

    def _check(self):
        n, m = self.len_a, self.len_b
        assert self.sigma.size == (n + 1) * (m + 1)
        assert self.gap_a.size == n + 1 and self.gap_b.size == m + 1
        assert self.min_col.size == n + 1 and self.max_col.size == n + 1
        assert self.am_arcs.size == 2 * self.am_score.size
        assert (self.am_stack_score is None) == (self.am_stackable is None)
        if self.am_stack_score is not None:
            assert self.am_stack_score.size == self.am_stackable.size == self.am_score.size

    @property
    def num_arcs_a(self):
        return self.arcs_a.size // 2

    @property
    def num_arcs_b(self):
        return self.arcs_b.size // 2

    @property
    def num_arcmatches(self):
        return self.am_score.size

    def to_c(self):
        t = lcg_pair_tables()
        t.len_a, t.len_b = self.len_a, self.len_b
        t.sigma, t.gap_a, t.gap_b = _ptr(self.sigma), _ptr(self.gap_a), _ptr(self.gap_b)
        t.indel_opening, t.exclusion = self.indel_opening, self.exclusion
        t.num_arcs_a, t.num_arcs_b = self.num_arcs_a, self.num_arcs_b
        t.arcs_a, t.arcs_b = _ptr(self.arcs_a), _ptr(self.arcs_b)
        t.num_arcmatches = self.num_arcmatches
        t.am_arcs, t.am_score = _ptr(self.am_arcs), _ptr(self.am_score)
        t.min_col, t.max_col = _ptr(self.min_col), _ptr(self.max_col)
        if self.anchors is not None:
            for k in self.ANCHOR_FIELDS:
                setattr(t, k, _ptr(self.anchors[k]))
        t.right_anchor_a, t.right_anchor_b = self.right_anchor
        t.left_anchor_a, t.left_anchor_b = self.left_anchor
        if self.am_stack_score is not None:
            # numpy gives even an empty array a non-NULL data pointer
            t.am_stack_score = _ptr(self.am_stack_score)
            t.am_stackable = self.am_stackable.ctypes.data_as(C.POINTER(C.c_uint8))
        return t


class AlignResult:
    """Decoded lcg_align_result."""

    def __init__(self, score, max_ij, min_ij, edges, traced_am):
        self.score = score
        self.max_ij = max_ij
        self.min_ij = min_ij
        self.edges = edges          # list of (a, b), -1 = gap
        self.traced_am = traced_am  # list of arc-match indices

    def __repr__(self):
        return f"AlignResult(score={self.score}, edges={len(self.edges)}, am={len(self.traced_am)})"


class ResultBuffers:
    """Caller-owned output buffers for one pair."""

    def __init__(self, len_a, len_b):
        self.edges = np.zeros(2 * (len_a + len_b) + 2, dtype=np.int32)
        self.tam = np.zeros(min(len_a, len_b) + 1, dtype=np.int32)
        self.c = lcg_align_result()
        self.c.edges = _ptr(self.edges)
        self.c.traced_am = _ptr(self.tam)

    def decode(self):
        r = self.c
        ne, nt = r.num_edges, r.num_traced_am
        e = self.edges[: 2 * ne].reshape(-1, 2)
        return AlignResult(int(r.score), (r.max_i, r.max_j), (r.min_i, r.min_j),
                           [tuple(map(int, x)) for x in e], [int(x) for x in self.tam[:nt]])


def make_opts(struct_local=False, sequ_local=False, free_endgaps="----", do_trace=True,
              no_lonely_pairs=False, normalized=None, penalized=None):
    """lcg_align_opts; normalized = L of --normalized, penalized = PP of
    --penalized (None = off)."""
    fe = 0
    if isinstance(free_endgaps, str):
        for k, ch in enumerate(free_endgaps[:4]):
            if ch == "+":
                fe |= 1 << k
    else:
        fe = int(free_endgaps)
    return lcg_align_opts(int(bool(struct_local)), int(bool(sequ_local)), fe, int(bool(do_trace)),
                          int(bool(no_lonely_pairs)), int(normalized is not None), int(normalized or 0),
                          int(penalized is not None), int(penalized or 0))
