"""Parser of the reference harness output (oracle/ref_harness.cc).

Test infrastructure: turns one ``LCGREF 1`` text block into the prepared
tables (``PairTables``) plus the reference's results.
"""
import numpy as np

from locarna_gb300.abi import LCG_STACK_NONE, PairTables


def _pairs(tokens, conv=int):
    return [tuple(conv(x) for x in t.split(":")) for t in tokens]


def parse_ref(text):
    rec = {}
    hits, khits, kstruct = [], [], []
    for line in text.splitlines():
        if not line.strip():
            continue
        key, _, rest = line.partition(" ")
        # k-best: "HIT score startA startA endB endB" (Aligner::suboptimal's own
        # output), "khit score edges..." / "kstruct A B" (the harness's hits)
        if key == "HIT":
            v = [int(x) for x in rest.split()]
            hits.append((v[0], v[1], v[3]))
            continue
        if key == "khit":
            t = rest.split()
            khits.append((int(t[0]), _pairs(t[1:])))
            continue
        if key == "klocal":
            khits[-1] = khits[-1] + (_pairs(rest.split()),)
            continue
        if key == "kstruct":
            kstruct.append(tuple(rest.split()))
            continue
        rec[key] = rest.split() if key not in ("seqA", "seqB", "structA", "structB") else rest.strip()
    n, m = (int(x) for x in rec["lens"])
    out = {"len_a": n, "len_b": m, "seq_a": rec["seqA"], "seq_b": rec["seqB"]}
    io, ex = (int(x) for x in rec["params"])
    band = _pairs(rec["band"])
    out["min_col"] = [b[0] for b in band]
    out["max_col"] = [b[1] for b in band]
    out["num_arcs"] = tuple(int(x) for x in rec["narcs"])
    out["num_am"] = int(rec["nam"][0])
    out["score"] = int(rec["score"][0])
    out["edges"] = _pairs(rec["edges"])
    out["struct_a"] = rec["structA"]
    out["struct_b"] = rec["structB"]
    out["align_seconds"] = float(rec["align_seconds"][0])
    out["hits"], out["khits"], out["kstruct"] = hits, khits, kstruct
    if "sigma" in rec:
        sig = np.zeros((n + 1, m + 1), dtype=np.int32)
        sig[1:, 1:] = np.array([int(x) for x in rec["sigma"]], dtype=np.int32).reshape(n, m)
        arcs_a = np.array(_pairs(rec["arcsA"]), dtype=np.int32).reshape(-1, 2)
        arcs_b = np.array(_pairs(rec["arcsB"]), dtype=np.int32).reshape(-1, 2)
        am = np.array(_pairs(rec["am"]), dtype=np.int32).reshape(-1, 3)
        st = sst = None
        if "amstack" in rec:
            # the reference's 64-bit stacked scores; values outside the int32
            # tables' range become LCG_STACK_NONE
            raw = [tuple(int(x) for x in t.split(":")) for t in rec["amstack"]]
            st = np.array([v if -(1 << 29) < v < (1 << 29) else LCG_STACK_NONE for v, _ in raw], dtype=np.int32)
            sst = np.array([f for _, f in raw], dtype=np.uint8)
        out["tables"] = PairTables(
            n, m, sig, [int(x) for x in rec["gapA"]], [int(x) for x in rec["gapB"]],
            io, ex, arcs_a, arcs_b, am[:, :2], am[:, 2], out["min_col"], out["max_col"],
            seq_a=rec["seqA"], seq_b=rec["seqB"], am_stack_score=st, am_stackable=sst)
        out["anchor_match"] = _pairs(rec["anchor_match"])
        if "anchor_ends" in rec:
            ra_a, ra_b, la_a, la_b, empty, intervals = (int(x) for x in rec["anchor_ends"])
            assert intervals, "anchor ranges are not intervals"
            out["anchor_empty"] = bool(empty)
            if not empty:
                # ranges per position, index 0 unused (include/locarna_gb300.h)
                def arr(pairs, k):
                    return np.array([0] + [p[k] for p in pairs], dtype=np.int32)
                m_ = _pairs(rec["anchor_match"])
                d_ = _pairs(rec["anchor_del"])
                i_ = _pairs(rec["anchor_ins"])
                anchors = {"match_lo": arr(m_, 0), "match_hi": arr(m_, 1), "del_lo": arr(d_, 0),
                           "del_hi": arr(d_, 1), "ins_lo": arr(i_, 0), "ins_hi": arr(i_, 1)}
                t0 = out["tables"]
                out["tables"] = PairTables(
                    t0.len_a, t0.len_b, t0.sigma, t0.gap_a, t0.gap_b, t0.indel_opening, t0.exclusion,
                    t0.arcs_a, t0.arcs_b, t0.am_arcs, t0.am_score, t0.min_col, t0.max_col,
                    anchors=anchors, right_anchor=(ra_a, ra_b), left_anchor=(la_a, la_b),
                    seq_a=t0.seq_a, seq_b=t0.seq_b, am_stack_score=t0.am_stack_score,
                    am_stackable=t0.am_stackable)
    return out
