"""Python binding of the C ABI (include/locarna_gb300.h) through ctypes.

This is a thin mirror of the C entry points: ``Engine.align_pairs`` is
``lcg_align_pairs``. The CUDA library must have been built
(``locarna_gb300.build.build_engine``); there is no fallback path.
"""
import ctypes as C
import os
import threading

import numpy as np

from .abi import (LCG_TUNE_BUCKETS, ResultBuffers, lcg_align_opts, lcg_align_result, lcg_pair_tables,
                  lcg_tune_entry,
                  lcg_pf_grad_spec, lcg_pf_opts, lcg_pf_result, lcg_work_counts, make_opts)

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "liblocarna_gb300.so")
ABI_VERSION = 4  # LCG_ABI_VERSION the structures of abi.py / prep.py mirror

_lib = None
_lib_lock = threading.Lock()


class LcgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"lcg error {code}: {msg}")
        self.code = code


def load_library(path=LIB_PATH):
    """Load the engine library; raises if it has not been built."""
    if _lib is not None:
        return _lib
    with _lib_lock:
        return _load_locked(path)


def _load_locked(path):
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"locarna_gb300 CUDA library missing ({path}); run __graft_entry__.build()")
    lib = C.CDLL(path)
    lib.lcg_last_error.restype = C.c_char_p
    lib.lcg_abi_version.restype = C.c_int32
    if lib.lcg_abi_version() != ABI_VERSION:
        raise RuntimeError(f"locarna_gb300 library {path} has ABI version {lib.lcg_abi_version()}, the binding "
                           f"expects {ABI_VERSION}; rebuild with __graft_entry__.build()")
    lib.lcg_engine_create.argtypes = [C.c_int32, C.c_void_p, C.POINTER(C.c_void_p)]
    lib.lcg_engine_create.restype = C.c_int32
    lib.lcg_engine_destroy.argtypes = [C.c_void_p]
    lib.lcg_engine_destroy.restype = C.c_int32
    lib.lcg_align_pairs.argtypes = [C.c_void_p, C.POINTER(lcg_pair_tables), C.c_int32,
                                    C.POINTER(lcg_align_opts), C.POINTER(lcg_align_result)]
    lib.lcg_align_pairs.restype = C.c_int32
    lib.lcg_align_kbest.argtypes = [C.c_void_p, C.POINTER(lcg_pair_tables), C.c_int32, C.POINTER(lcg_align_opts),
                                    C.c_int32, C.c_int64, C.POINTER(lcg_align_result), C.POINTER(C.c_int32)]
    lib.lcg_align_kbest.restype = C.c_int32
    lib.lcg_engine_last_stats.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int64)]
    lib.lcg_engine_last_stats.restype = C.c_int32
    lib.lcg_engine_last_timing.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    lib.lcg_engine_last_timing.restype = C.c_int32
    lib.lcg_engine_last_phases.argtypes = [C.c_void_p] + [C.POINTER(C.c_double)] * 4
    lib.lcg_engine_last_phases.restype = C.c_int32
    lib.lcg_engine_last_transfer.argtypes = [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
    lib.lcg_engine_last_transfer.restype = C.c_int32
    lib.lcg_engine_last_prep_transfer.argtypes = [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
    lib.lcg_engine_last_prep_transfer.restype = C.c_int32
    lib.lcg_engine_set_chunk_pairs.argtypes = [C.c_void_p, C.c_int32]
    lib.lcg_engine_set_chunk_pairs.restype = C.c_int32
    lib.lcg_engine_set_counting.argtypes = [C.c_void_p, C.c_int32]
    lib.lcg_engine_set_counting.restype = C.c_int32
    lib.lcg_engine_last_work.argtypes = [C.c_void_p, C.POINTER(lcg_work_counts)]
    lib.lcg_engine_last_work.restype = C.c_int32
    lib.lcg_pair_work.argtypes = [C.POINTER(lcg_pair_tables), C.POINTER(lcg_align_opts), C.POINTER(lcg_work_counts)]
    lib.lcg_pair_work.restype = C.c_int32
    lib.lcg_engine_autotune.argtypes = [C.c_void_p, C.POINTER(lcg_pair_tables), C.c_int32, C.POINTER(lcg_align_opts),
                                        C.c_int32, C.POINTER(lcg_tune_entry)]
    lib.lcg_engine_autotune.restype = C.c_int32
    lib.lcg_engine_set_autotune.argtypes = [C.c_void_p, C.c_int32]
    lib.lcg_engine_set_autotune.restype = C.c_int32
    lib.lcg_align_pp_pairs.argtypes = [C.c_void_p, C.POINTER(C.c_char_p), C.POINTER(C.c_char_p), C.c_int32,
                                       C.c_void_p, C.POINTER(lcg_align_opts), C.POINTER(lcg_align_result),
                                       C.POINTER(C.c_int32)]
    lib.lcg_align_pp_pairs.restype = C.c_int32
    lib.lcg_engine_set_graphs.argtypes = [C.c_void_p, C.c_int32]
    lib.lcg_engine_set_graphs.restype = C.c_int32
    lib.lcg_engine_last_graphs.argtypes = [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
    lib.lcg_engine_last_graphs.restype = C.c_int32
    lib.lcg_pf_opts_default.argtypes = [C.POINTER(lcg_pf_opts)]
    lib.lcg_pf_opts_default.restype = None
    lib.lcg_pf_forward.argtypes = [C.c_void_p, C.POINTER(lcg_pair_tables), C.c_int32, C.POINTER(lcg_pf_opts),
                                   C.POINTER(lcg_pf_grad_spec), C.POINTER(C.c_double)]
    lib.lcg_pf_forward.restype = C.c_int32
    lib.lcg_pf_backward.argtypes = [C.c_void_p, C.POINTER(lcg_pf_grad_spec), C.POINTER(lcg_pf_result)]
    lib.lcg_pf_backward.restype = C.c_int32
    lib.lcg_engine_set_rect_budget.argtypes = [C.c_void_p, C.c_int64]
    lib.lcg_engine_set_rect_budget.restype = C.c_int32
    lib.lcg_pf_last_timing.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    lib.lcg_pf_last_timing.restype = C.c_int32
    _lib = lib
    return lib


def _check(lib, rc):
    if rc != 0:
        raise LcgError(rc, lib.lcg_last_error().decode())


def pair_work(tables, **kw):
    """lcg_pair_work: (groups, cells, D entries) of one pair, on the host."""
    lib = load_library()
    o = make_opts(**kw)
    w = lcg_work_counts()
    ct = tables.to_c()
    _check(lib, lib.lcg_pair_work(C.byref(ct), C.byref(o), C.byref(w)))
    return w.groups, w.cells, w.arc_terms


class Engine:
    """One GPU engine (lcg_engine): owns device buffers, launches on a stream."""

    def __init__(self, device=0, stream=None):
        self.lib = load_library()
        h = C.c_void_p()
        _check(self.lib, self.lib.lcg_engine_create(int(device), stream, C.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            self.lib.lcg_engine_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def prepare_call(self, tables, opts=None, **kw):
        """Build the C argument arrays once (see run_call / decode_call)."""
        if opts is None:
            opts = make_opts(**kw)
        n = len(tables)
        arr = (lcg_pair_tables * n)(*[t.to_c() for t in tables])
        bufs = [ResultBuffers(t.len_a, t.len_b) for t in tables]
        res = (lcg_align_result * n)(*[b.c for b in bufs])
        return (arr, n, opts, res, bufs, tables)

    def run_call(self, call):
        """One lcg_align_pairs call on prepared arguments (the timed unit)."""
        arr, n, opts, res, _, _ = call
        _check(self.lib, self.lib.lcg_align_pairs(self.h, arr, n, C.byref(opts), res))

    @staticmethod
    def decode_call(call):
        _, _, _, res, bufs, _ = call
        out = []
        for k, b in enumerate(bufs):
            b.c = res[k]
            out.append(b.decode())
        return out

    def align_pairs(self, tables, opts=None, **kw):
        """Align a list of PairTables; returns a list of AlignResult."""
        call = self.prepare_call(tables, opts, **kw)
        self.run_call(call)
        return self.decode_call(call)

    def prepare_pp_call(self, pp_pairs, lens, prep=None, **kw):
        """Arguments of lcg_align_pp_pairs built once: the PP texts, the
        preparation options (a lcg_prep_opts, None = defaults), the alignment
        options and result buffers for the pairs' sequence lengths
        lens[q] = (len_a, len_b)."""
        n = len(pp_pairs)
        enc = [(a.encode(), b.encode()) for a, b in pp_pairs]
        arr_a = (C.c_char_p * n)(*[a for a, _ in enc])
        arr_b = (C.c_char_p * n)(*[b for _, b in enc])
        bufs = [ResultBuffers(la, lb) for la, lb in lens]
        res = (lcg_align_result * n)(*[b.c for b in bufs])
        return (arr_a, arr_b, n, prep, make_opts(**kw), res, bufs, enc)

    def run_pp_call(self, call):
        """One lcg_align_pp_pairs call; returns the number of host envelopes."""
        arr_a, arr_b, n, prep, opts, res, _, _ = call
        nhost = C.c_int32()
        _check(self.lib, self.lib.lcg_align_pp_pairs(self.h, arr_a, arr_b, n,
                                                      C.byref(prep) if prep is not None else None,
                                                      C.byref(opts), res, C.byref(nhost)))
        return nhost.value

    @staticmethod
    def decode_pp_call(call):
        _, _, _, _, _, res, bufs, _ = call
        out = []
        for k, b in enumerate(bufs):
            b.c = res[k]
            out.append(b.decode())
        return out

    def align_kbest(self, tables, k, threshold=-1000000, **kw):
        """lcg_align_kbest: per pair the list of its (up to k) hits, each an
        AlignResult whose score is the hit's score."""
        opts = make_opts(**kw)
        n = len(tables)
        arr = (lcg_pair_tables * n)(*[t.to_c() for t in tables])
        bufs = [ResultBuffers(t.len_a, t.len_b) for t in tables for _ in range(k)]
        res = (lcg_align_result * (n * k))(*[b.c for b in bufs])
        hits = (C.c_int32 * n)()
        _check(self.lib, self.lib.lcg_align_kbest(self.h, arr, n, C.byref(opts), int(k), int(threshold), res, hits))
        out = []
        for q in range(n):
            row = []
            for h in range(hits[q]):
                b = bufs[q * k + h]
                b.c = res[q * k + h]
                row.append(b.decode())
            out.append(row)
        return out

    def last_stats(self):
        ms = C.c_double()
        nl = C.c_int64()
        _check(self.lib, self.lib.lcg_engine_last_stats(self.h, C.byref(ms), C.byref(nl)))
        return ms.value, nl.value

    def last_timing(self):
        a, b = C.c_double(), C.c_double()
        _check(self.lib, self.lib.lcg_engine_last_timing(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def last_phases(self):
        """(prep, pack, copies + kernels, results) wall ms of the last call."""
        v = [C.c_double() for _ in range(4)]
        _check(self.lib, self.lib.lcg_engine_last_phases(self.h, *[C.byref(x) for x in v]))
        return tuple(x.value for x in v)

    def last_transfer(self):
        a, b = C.c_int64(), C.c_int64()
        _check(self.lib, self.lib.lcg_engine_last_transfer(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def last_prep_transfer(self):
        a, b = C.c_int64(), C.c_int64()
        _check(self.lib, self.lib.lcg_engine_last_prep_transfer(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def set_chunk_pairs(self, n):
        """Pairs per chunk of lcg_align_pairs' pipeline (0: automatic)."""
        _check(self.lib, self.lib.lcg_engine_set_chunk_pairs(self.h, int(n)))

    def autotune(self, tables, sample_pairs=64, **kw):
        """lcg_engine_autotune: per length bucket, the measured best launch
        configuration of the fill (a list of dicts, one per bucket)."""
        o = make_opts(**kw)
        n = len(tables)
        arr = (lcg_pair_tables * n)(*[t.to_c() for t in tables])
        rep = (lcg_tune_entry * LCG_TUNE_BUCKETS)()
        _check(self.lib, self.lib.lcg_engine_autotune(self.h, arr, n, C.byref(o), int(sample_pairs), rep))
        return [dict(max_len=r.max_len, pairs_sampled=r.pairs_sampled, blocks_per_sm=r.blocks_per_sm,
                     wave_mb=r.wave_mb, best_ms=r.best_ms, default_ms=r.default_ms, trials=r.trials) for r in rep]

    def set_graphs(self, on):
        _check(self.lib, self.lib.lcg_engine_set_graphs(self.h, int(bool(on))))

    def last_graphs(self):
        """(captures, replays) of CUDA graphs in the last lcg_align_pairs call."""
        a, b = C.c_int64(), C.c_int64()
        _check(self.lib, self.lib.lcg_engine_last_graphs(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def set_rect_budget(self, nbytes):
        """lcg_engine_set_rect_budget: bytes of kept group rectangles per
        chunk (0: the traceback always recomputes; negative: the defaults,
        4 GiB for plain and 32 GiB for structure-local chunks)."""
        _check(self.lib, self.lib.lcg_engine_set_rect_budget(self.h, int(nbytes)))

    def set_autotune(self, on):
        _check(self.lib, self.lib.lcg_engine_set_autotune(self.h, int(bool(on))))

    def set_counting(self, on):
        _check(self.lib, self.lib.lcg_engine_set_counting(self.h, int(bool(on))))

    def last_work(self):
        w = lcg_work_counts()
        _check(self.lib, self.lib.lcg_engine_last_work(self.h, C.byref(w)))
        return dict(groups=w.groups, cells=w.cells, visits=w.arc_terms, arc_terms=w.valid_arc_terms)

    # ------------------------------------------------------------ LocARNA-P

    def pf_opts(self, temperature=300.0, pf_scale=1.0, precision=64, param_delta=None, min_am_prob=0.001,
                min_bm_prob=0.001, gap_gradients=True):
        """lcg_pf_opts; min_am_prob = 0 gives the exact base-match marginals,
        > 0 the truncated ones locarna_p reports (its default 0.001);
        gap_gradients = False: probabilities only (no gap counts, NaN
        indel / indel-opening gradients)."""
        o = lcg_pf_opts()
        self.lib.lcg_pf_opts_default(C.byref(o))
        o.temperature, o.pf_scale, o.precision = float(temperature), float(pf_scale), int(precision)
        o.min_am_prob, o.min_bm_prob = float(min_am_prob), float(min_bm_prob)
        o.gap_gradients = 1 if gap_gradients else 0
        if param_delta is not None:
            for k, v in enumerate(param_delta):
                o.param_delta[k] = float(v)
        return o

    @staticmethod
    def _specs(tables):
        """lcg_pf_grad_spec array from PairTables carrying code_a/code_b/am_dsw
        (prepare_pair sets them); None when a table lacks them."""
        if not all(hasattr(t, "code_a") for t in tables):
            return None, None
        keep = []
        arr = (lcg_pf_grad_spec * len(tables))()
        for k, t in enumerate(tables):
            ca = np.ascontiguousarray(t.code_a, dtype=np.int8)
            cb = np.ascontiguousarray(t.code_b, dtype=np.int8)
            dsw = np.ascontiguousarray(t.am_dsw, dtype=np.float64) if getattr(t, "am_dsw", None) is not None else None
            keep += [ca, cb, dsw]
            arr[k].code_a = ca.ctypes.data_as(C.POINTER(C.c_int8))
            arr[k].code_b = cb.ctypes.data_as(C.POINTER(C.c_int8))
            arr[k].am_dscore_dsw = (dsw.ctypes.data_as(C.POINTER(C.c_double))
                                    if dsw is not None and dsw.size else None)
        return arr, keep

    def pf_forward(self, tables, temperature=300.0, pf_scale=1.0, precision=64, param_delta=None,
                   min_am_prob=0.001, min_bm_prob=0.001, gap_gradients=True):
        """lcg_pf_forward: log Z of each pair (numpy float64 array)."""
        o = self.pf_opts(temperature, pf_scale, precision, param_delta, min_am_prob, min_bm_prob, gap_gradients)
        n = len(tables)
        arr = (lcg_pair_tables * n)(*[t.to_c() for t in tables])
        specs, keep = self._specs(tables)
        out = np.zeros(n, dtype=np.float64)
        self._pf_tables = (arr, tables, specs, keep)
        _check(self.lib, self.lib.lcg_pf_forward(self.h, arr, n, C.byref(o), specs,
                                                 out.ctypes.data_as(C.POINTER(C.c_double))))
        return out

    def pf_backward(self, probs=True):
        """lcg_pf_backward for the last pf_forward: one dict per pair with
        log_z, am_prob, bm_prob ((n+1) x (m+1)), expected gap counts and the
        derivatives of log Z."""
        arr, tables, specs, _ = self._pf_tables
        n = len(tables)
        res = (lcg_pf_result * n)()
        bufs = []
        for k, t in enumerate(tables):
            am = np.zeros(max(1, t.num_arcmatches))
            bm = np.zeros((t.len_a + 1) * (t.len_b + 1))
            bufs.append((am, bm))
            if probs:
                res[k].am_prob = am.ctypes.data_as(C.POINTER(C.c_double))
                res[k].bm_prob = bm.ctypes.data_as(C.POINTER(C.c_double))
        _check(self.lib, self.lib.lcg_pf_backward(self.h, specs, res))
        out = []
        for k, t in enumerate(tables):
            r = res[k]
            d = dict(log_z=r.log_z, gap_ext_uses=r.gap_ext_uses, gap_open_uses=r.gap_open_uses,
                     dlogz_dindel=r.dlogz_dindel, dlogz_dindel_opening=r.dlogz_dindel_opening,
                     dlogz_dstruct_weight=r.dlogz_dstruct_weight,
                     dlogz_dbasematch=np.array(list(r.dlogz_dbasematch)))
            if probs:
                d["am_prob"] = bufs[k][0][:t.num_arcmatches]
                d["bm_prob"] = bufs[k][1].reshape(t.len_a + 1, t.len_b + 1)
            out.append(d)
        return out

    def pf_last_timing(self):
        a, b = C.c_double(), C.c_double()
        _check(self.lib, self.lib.lcg_pf_last_timing(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value
