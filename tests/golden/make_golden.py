"""Generate the golden fixtures of tests/golden/ from the REFERENCE itself.

Test infrastructure. Runs the reference's own code (oracle/_ref/ref_harness,
built from the reference sources by oracle/build_ref.sh) on seeded synthetic
PP inputs (locarna_gb300/synth.py) and stores, per case, the inputs, the
prepared tables the reference's Scoring/ArcMatches/TraceController objects
hold, and the reference's results (score, traceback edges, structure strings).

Usage: python tests/golden/make_golden.py   (needs the reference sources)
"""
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from locarna_gb300.synth import make_homolog, make_profile, make_rna  # noqa: E402
from refdump import parse_ref  # noqa: E402

HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")

# name: (lenA, seedA, lenB, seedB, options, keep_tables); lenB = "h" makes B a
# homolog of A (make_homolog with seed seedB); a length ("p", L, rows) makes a
# profile (make_profile: an alignment of rows homologs of one RNA)
CASES = {
    "c150_global": (150, 1, 150, 2, {}, True),
    "c150_seqlocal": (150, 1, 150, 2, {"sequ_local": "1"}, True),
    "c150_structlocal": (150, 1, 150, 2, {"struct_local": "1"}, True),
    "c150_freeall": (150, 1, 150, 2, {"free_endgaps": "++++"}, True),
    "c150_freeright": (150, 1, 150, 2, {"free_endgaps": "-+-+"}, True),
    "c150_freeleft": (150, 1, 150, 2, {"free_endgaps": "+-+-"}, True),
    "c150_noenv": (150, 1, 150, 2, {"min_trace_prob": "0"}, True),
    "c150_b": (150, 11, 140, 12, {}, True),
    "c120_opening0": (120, 21, 130, 22, {"indel_opening": "0"}, True),
    "c90_seqlocal_b": (90, 31, 100, 32, {"sequ_local": "1"}, True),
    "c60_short": (60, 41, 70, 42, {}, True),
    "c200_global": (200, 5, 200, 6, {}, True),
    "c400_global": (400, 3, 400, 4, {}, True),
    "c400_structlocal": (400, 3, 400, 4, {"struct_local": "1"}, True),
    # locarna --noLP: no lonely base pairs in the aligned structure
    "c150_nolp": (150, 1, 150, 2, {"no_lonely_pairs": "1"}, True),
    "c150_nolp_b": (150, 11, 140, 12, {"no_lonely_pairs": "1"}, True),
    "c150_nolp_seqlocal": (150, 1, 150, 2, {"no_lonely_pairs": "1", "sequ_local": "1"}, True),
    "c150_nolp_structlocal": (150, 1, 150, 2, {"no_lonely_pairs": "1", "struct_local": "1"}, True),
    "c150_nolp_freeall": (150, 1, 150, 2, {"no_lonely_pairs": "1", "free_endgaps": "++++"}, True),
    "c120_nolp_opening0": (120, 21, 130, 22, {"no_lonely_pairs": "1", "indel_opening": "0"}, True),
    "c300_nolp": (300, 61, 280, 62, {"no_lonely_pairs": "1"}, True),
    # locarna --stacking / --new-stacking: PP inputs with #STACK joint probabilities
    "c150_stack": (150, 1, 150, 2, {"stacking": "1", "exp_prob": "0.005"}, True),
    "c150_newstack": (150, 1, 150, 2, {"new_stacking": "1"}, True),
    "c150_bothstack": (150, 1, 150, 2, {"stacking": "1", "new_stacking": "1", "exp_prob": "0.005"}, True),
    "c150_stack_noexp": (150, 1, 150, 2, {"stacking": "1"}, True),
    "c150_stack_nolp": (150, 1, 150, 2, {"stacking": "1", "exp_prob": "0.005", "no_lonely_pairs": "1"}, True),
    "c150_stack_structlocal": (150, 1, 150, 2, {"stacking": "1", "exp_prob": "0.005", "struct_local": "1"}, True),
    "c150_newstack_nolp_sl": (150, 11, 140, 12, {"new_stacking": "1", "no_lonely_pairs": "1",
                                                 "struct_local": "1"}, True),
    "c120_stack_seqlocal": (120, 21, 130, 22, {"stacking": "1", "exp_prob": "0.01", "sequ_local": "1"}, True),
    "c250_newstack_b": (250, 71, 240, 72, {"new_stacking": "1"}, True),
    # homologous pairs (shared stems): most of the structure is aligned
    "h150_global": (150, 81, "h", 82, {}, True),
    "h150_nolp": (150, 81, "h", 82, {"no_lonely_pairs": "1"}, True),
    "h150_stack": (150, 81, "h", 82, {"stacking": "1", "exp_prob": "0.005"}, True),
    "h150_newstack_nolp": (150, 81, "h", 82, {"new_stacking": "1", "no_lonely_pairs": "1"}, True),
    "h200_bothstack_sl": (200, 83, "h", 84, {"stacking": "1", "new_stacking": "1", "exp_prob": "0.004",
                                             "struct_local": "1"}, True),
    "h180_nolp_sl": (180, 85, "h", 86, {"no_lonely_pairs": "1", "struct_local": "1"}, True),
    "h160_stack_nolp_seqlocal": (160, 87, "h", 88, {"stacking": "1", "exp_prob": "0.006",
                                                    "no_lonely_pairs": "1", "sequ_local": "1"}, True),
    # locarna --normalized L / --penalized PP (sequence-local top level, modified scoring)
    "h150_normalized": (150, 81, "h", 82, {"sequ_local": "1", "normalized": "100"}, True),
    "c150_normalized": (150, 1, 150, 2, {"sequ_local": "1", "normalized": "50"}, True),
    "h180_normalized_nolp": (180, 85, "h", 86, {"sequ_local": "1", "normalized": "300",
                                                "no_lonely_pairs": "1"}, True),
    "h150_penalized": (150, 81, "h", 82, {"sequ_local": "1", "penalized": "40"}, True),
    "c150_penalized": (150, 1, 150, 2, {"sequ_local": "1", "penalized": "20"}, True),
    "h200_penalized_global": (200, 83, "h", 84, {"penalized": "30", "free_endgaps": "++++"}, True),
    "h180_penalized_sl": (180, 85, "h", 86, {"sequ_local": "1", "penalized": "25", "struct_local": "1"}, True),
    # locarna --kbest k [--better t] (Aligner::suboptimal: k best local alignments by interval splitting)
    "c150_kbest": (150, 1, 150, 2, {"sequ_local": "1", "kbest": "6"}, True),
    "h200_kbest": (200, 83, "h", 84, {"sequ_local": "1", "kbest": "8"}, True),
    "h180_kbest_nolp_better": (180, 85, "h", 86, {"sequ_local": "1", "kbest": "10", "no_lonely_pairs": "1",
                                                  "better": "3000"}, True),
    "c150_kbest_global": (150, 11, 140, 12, {"kbest": "4", "free_endgaps": "++++"}, True),
    "h200_kbest_normalized": (200, 83, "h", 84, {"sequ_local": "1", "kbest": "5", "normalized": "100"}, True),
    "c150_kbest_normalized_nolp": (150, 1, 150, 2, {"sequ_local": "1", "kbest": "4", "normalized": "50",
                                                    "no_lonely_pairs": "1"}, True),
    # profile (multiple alignment) inputs, as in mlocarna's progressive stage
    "p120_global": (("p", 120, 3), 5, ("p", 110, 2), 6, {}, True),
    "p150_vs_seq": (("p", 150, 4), 91, 140, 92, {}, True),
    "p140_seqlocal": (("p", 140, 3), 95, ("p", 130, 3), 96, {"sequ_local": "1"}, True),
    "p140_structlocal": (("p", 140, 3), 95, ("p", 130, 3), 96, {"struct_local": "1"}, True),
    "p140_nolp_free": (("p", 140, 3), 97, ("p", 150, 2), 98, {"no_lonely_pairs": "1", "free_endgaps": "++++"},
                       True),
    "p130_noenv": (("p", 130, 5), 99, ("p", 120, 3), 100, {"min_trace_prob": "0"}, True),
    "p250_global": (("p", 250, 3), 101, ("p", 240, 3), 102, {}, True),
    # anchor constraints (#A1 lines; "anchors" = matched positions A:B, named
    # A, B, C, ... in order; the reference's strict anchors)
    "a150_anchors": (150, 81, "h", 82, {"anchors": "20:20,75:75,130:130"}, True),
    "a150_anchors_seqlocal": (150, 81, "h", 82, {"anchors": "40:40,90:90", "sequ_local": "1"}, True),
    "a150_anchors_structlocal": (150, 81, "h", 82, {"anchors": "20:20,75:75", "struct_local": "1"}, True),
    "a150_anchors_free": (150, 81, "h", 82, {"anchors": "30:30,110:110", "free_endgaps": "++++"}, True),
    "a150_anchors_nolp": (150, 81, "h", 82, {"anchors": "60:60", "no_lonely_pairs": "1"}, True),
    "a120_anchors_unrel": (120, 21, 130, 22, {"anchors": "10:15,60:70,100:120"}, True),
    # --max-diff (band around the diagonal), --max-diff-am / --max-diff-at-am (arc-match filters)
    "c150_maxdiff": (150, 1, 150, 2, {"max_diff": "20"}, True),
    "h150_maxdiff_am": (150, 81, "h", 82, {"max_diff_am": "5", "max_diff_at_am": "12"}, True),
    "p120_maxdiff": (("p", 120, 3), 5, ("p", 110, 2), 6, {"max_diff": "30", "sequ_local": "1"}, True),
}

STACK_KEYS = ("stacking", "new_stacking")


def make_case(name, spec, workdir):
    la, sa, lb, sb, opts, keep = spec
    ra = make_profile(la[1], sa, la[2]) if isinstance(la, tuple) else make_rna(la, sa)
    if lb == "h":
        rb = make_homolog(ra, sb)
    else:
        rb = make_profile(lb[1], sb, lb[2]) if isinstance(lb, tuple) else make_rna(lb, sb)
    st = any(k in opts for k in STACK_KEYS)  # inputs with joint (stacking) probabilities
    anc_a = anc_b = None
    if "anchors" in opts:
        anc_a, anc_b = ["."] * len(ra.seq), ["."] * len(rb.seq)
        for k, ab in enumerate(opts["anchors"].split(",")):
            x, y = (int(v) for v in ab.split(":"))
            anc_a[x - 1] = anc_b[y - 1] = chr(ord("A") + k)
        anc_a, anc_b = "".join(anc_a), "".join(anc_b)
    pa, pb = os.path.join(workdir, name + "_A.pp"), os.path.join(workdir, name + "_B.pp")
    pp_a = ra.to_pp(stacking=st) if st else (ra.to_pp(anchors=anc_a) if anc_a else ra.to_pp())
    pp_b = rb.to_pp(stacking=st) if st else (rb.to_pp(anchors=anc_b) if anc_b else rb.to_pp())
    with open(pa, "w") as f:
        f.write(pp_a)
    with open(pb, "w") as f:
        f.write(pp_b)
    args = [HARNESS, pa, pb] + [f"{k}={v}" for k, v in opts.items() if k != "anchors"]
    txt = subprocess.run(args, capture_output=True, text=True, check=True).stdout
    ref = parse_ref(txt)
    t = ref["tables"]
    out = {
        "pp_a": pp_a, "pp_b": pp_b, "opts": json.dumps(opts),
        "score": ref["score"], "edges": np.array(ref["edges"], dtype=np.int32),
        "struct_a": ref["struct_a"], "struct_b": ref["struct_b"],
        "min_col": np.array(ref["min_col"], dtype=np.int32),
        "max_col": np.array(ref["max_col"], dtype=np.int32),
        "num_arcs": np.array(ref["num_arcs"], dtype=np.int32),
        "num_am": ref["num_am"],
        "seq_a": ref["seq_a"], "seq_b": ref["seq_b"],
        "indel_opening": t.indel_opening, "exclusion": t.exclusion,
        "gap_a": t.gap_a, "gap_b": t.gap_b,
        "arcs_a": t.arcs_a, "arcs_b": t.arcs_b,
        "am_arcs": t.am_arcs, "am_score": t.am_score,
        "sigma": t.sigma.astype(np.int16) if np.abs(t.sigma).max() < 32000 else t.sigma,
    }
    if t.anchors is not None:
        for k_, v_ in t.anchors.items():
            out["anchor_" + k_] = v_
        out["anchor_ends"] = np.array(list(t.right_anchor) + list(t.left_anchor), dtype=np.int32)
    if t.am_stack_score is not None:
        out["am_stack_score"] = t.am_stack_score
        out["am_stackable"] = t.am_stackable
    if ref["khits"]:
        # the harness's enumeration must give the reference's own hits
        # (score, first position in A, last position in B)
        mine = []
        for sc, _, local in ref["khits"]:
            pa = [a for a, _ in local if a > 0]
            pb = [b for _, b in local if b > 0]
            mine.append((sc, pa[0] if pa else 0, pb[-1] if pb else 0))
        assert mine == ref["hits"], (name, mine, ref["hits"])
        out["kbest_scores"] = np.array([h[0] for h in ref["khits"]], dtype=np.int64)  # hit scores
        out["kbest_edges"] = np.concatenate([np.array(h[1], dtype=np.int32) for h in ref["khits"]])
        out["kbest_nedges"] = np.array([len(h[1]) for h in ref["khits"]], dtype=np.int32)
        out["kbest_struct"] = "|".join(a + " " + b for a, b in ref["kstruct"])
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    return ref


def main():
    if not os.path.exists(HARNESS):
        raise SystemExit("build the reference oracle first: oracle/build_ref.sh")
    names = sys.argv[1:] or list(CASES)
    with tempfile.TemporaryDirectory(prefix="golden_pp_") as work:
        for name in names:
            ref = make_case(name, CASES[name], work)
            print(name, "score", ref["score"], "am", ref["num_am"])


if __name__ == "__main__" and not os.environ.get("LCG_GOLDEN_PF"):
    main()


# ---------------------------------------------------------------- LocARNA-P

HARNESS_P = os.path.join(ROOT, "oracle", "_ref", "ref_harness_p")

# name: (lenA, seedA, lenB, seedB, options)
PF_CASES = {
    "pf150": (150, 1, 150, 2, {}),
    "pf200": (200, 5, 200, 6, {}),
    "pf90_b": (90, 51, 110, 52, {}),
    # profile inputs (alignment rows)
    "pf_p100": (("p", 100, 3), 61, ("p", 90, 2), 62, {}),
    # locarna_p's default --min-am-prob 0.001: base-match probabilities
    # truncated under arc matches of probability <= sqrt(0.001)
    "pf90_b_default": (90, 51, 110, 52, {"min_am_prob": "0.001"}),
    "pf100_default": (100, 55, 95, 56, {"min_am_prob": "0.001"}),
    "pf80_default": (80, 57, 85, 58, {"min_am_prob": "0.001"}),
}


def parse_pf(txt):
    lines = {}
    for l in txt.splitlines():
        k, _, v = l.partition(" ")
        lines[k] = v
    fake = txt + "\nscore 0\nedges 1:1\nstructA .\nstructB .\nalign_seconds 0\nanchor_match 1:1\n"
    ref = parse_ref(fake)
    am = []
    for tok in lines["amprobs"].split():
        a1, a2, b1, b2, p = tok.split(":")
        am.append((int(a1), int(a2), int(b1), int(b2), float(p)))
    bm = []
    for tok in lines["bmprobs"].split():
        i, j, p = tok.split(":")
        bm.append((int(i), int(j), float(p)))
    return ref, float(lines["Z"]), am, bm


def make_pf_case(name, spec, workdir):
    la, sa, lb, sb, opts = spec
    ra = make_profile(la[1], sa, la[2]) if isinstance(la, tuple) else make_rna(la, sa)
    rb = make_profile(lb[1], sb, lb[2]) if isinstance(lb, tuple) else make_rna(lb, sb)
    pa, pb = os.path.join(workdir, name + "_A.pp"), os.path.join(workdir, name + "_B.pp")
    with open(pa, "w") as f:
        f.write(ra.to_pp())
    with open(pb, "w") as f:
        f.write(rb.to_pp())
    args = [HARNESS_P, pa, pb, "min_am_prob=0"] + [f"{k}={v}" for k, v in opts.items()]
    txt = subprocess.run(args, capture_output=True, text=True, check=True).stdout
    ref, Z, am, bm = parse_pf(txt)
    t = ref["tables"]
    out = {
        "pp_a": ra.to_pp(), "pp_b": rb.to_pp(), "opts": json.dumps(opts), "Z": Z,
        "am": np.array([x[:4] for x in am], dtype=np.int32).reshape(-1, 4),
        "am_p": np.array([x[4] for x in am], dtype=np.float64),
        "bm": np.array([x[:2] for x in bm], dtype=np.int32).reshape(-1, 2),
        "bm_p": np.array([x[2] for x in bm], dtype=np.float64),
        "min_col": np.array(ref["min_col"], dtype=np.int32),
        "max_col": np.array(ref["max_col"], dtype=np.int32),
        "seq_a": ref["seq_a"], "seq_b": ref["seq_b"],
        "indel_opening": t.indel_opening, "exclusion": t.exclusion,
        "gap_a": t.gap_a, "gap_b": t.gap_b, "arcs_a": t.arcs_a, "arcs_b": t.arcs_b,
        "am_arcs": t.am_arcs, "am_score": t.am_score, "sigma": t.sigma.astype(np.int16),
    }
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    return Z, len(am)


def main_pf():
    with tempfile.TemporaryDirectory(prefix="golden_pp_") as work:
        for name in sys.argv[1:] or list(PF_CASES):
            print(name, *make_pf_case(name, PF_CASES[name], work))


if __name__ == "__main__" and os.environ.get("LCG_GOLDEN_PF"):
    main_pf()
