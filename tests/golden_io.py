"""Loader of the golden fixtures in tests/golden/*.npz (made by make_golden.py)."""
import glob
import json
import os

import numpy as np

from locarna_gb300.abi import PairTables

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden_names():
    """Golden cases (one .npz each); *_marginals.npz are companion fixtures."""
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN_DIR, "*.npz"))
                  if not p.endswith("_marginals.npz"))


def sankoff_golden_names():
    return [n for n in golden_names() if not n.startswith("pf")]


class Golden:
    def __init__(self, name):
        z = np.load(os.path.join(GOLDEN_DIR, name + ".npz"))
        self.name = name
        self.opts = json.loads(str(z["opts"]))
        self.pp_a, self.pp_b = str(z["pp_a"]), str(z["pp_b"])
        self.seq_a, self.seq_b = str(z["seq_a"]), str(z["seq_b"])
        self.score = int(z["score"])
        self.edges = [tuple(int(v) for v in e) for e in z["edges"]]
        self.struct_a, self.struct_b = str(z["struct_a"]), str(z["struct_b"])
        self.min_col, self.max_col = z["min_col"], z["max_col"]
        self.num_arcs = tuple(int(x) for x in z["num_arcs"])
        self.num_am = int(z["num_am"])
        n, m = len(self.seq_a), len(self.seq_b)
        self.tables = PairTables(
            n, m, z["sigma"].astype(np.int32), z["gap_a"], z["gap_b"],
            int(z["indel_opening"]), int(z["exclusion"]), z["arcs_a"], z["arcs_b"],
            z["am_arcs"], z["am_score"], self.min_col, self.max_col,
            seq_a=self.seq_a, seq_b=self.seq_b,
            am_stack_score=z["am_stack_score"] if "am_stack_score" in z else None,
            am_stackable=z["am_stackable"] if "am_stackable" in z else None,
            anchors=({k: z["anchor_" + k] for k in PairTables.ANCHOR_FIELDS} if "anchor_match_lo" in z else None),
            right_anchor=tuple(int(v) for v in z["anchor_ends"][:2]) if "anchor_ends" in z else (0, 0),
            left_anchor=tuple(int(v) for v in z["anchor_ends"][2:]) if "anchor_ends" in z else None)

    @property
    def struct_local(self):
        return self.opts.get("struct_local") == "1"

    @property
    def sequ_local(self):
        return self.opts.get("sequ_local") == "1"

    @property
    def free_endgaps(self):
        return self.opts.get("free_endgaps", "----")

    @property
    def kbest(self):
        """(k, threshold) of --kbest k --better t, or None"""
        if "kbest" not in self.opts:
            return None
        return int(self.opts["kbest"]), int(self.opts.get("better", -1000000))

    def kbest_hits(self):
        """The reference's k-best hits: [(score, full edges, (structA, structB))]"""
        z = np.load(os.path.join(GOLDEN_DIR, self.name + ".npz"))
        out, pos = [], 0
        structs = str(z["kbest_struct"]).split("|")
        for sc, ne, st in zip(z["kbest_scores"], z["kbest_nedges"], structs):
            e = [tuple(int(v) for v in x) for x in z["kbest_edges"][pos:pos + ne]]
            pos += ne
            out.append((int(sc), e, tuple(st.split(" "))))
        return out

    @property
    def has_anchors(self):
        """inputs with #A anchor lines (the host preparation does not read them)"""
        return "anchors" in self.opts

    @property
    def no_lonely_pairs(self):
        return self.opts.get("no_lonely_pairs") == "1"

    def align_kwargs(self):
        kw = dict(struct_local=self.struct_local, sequ_local=self.sequ_local,
                  free_endgaps=self.free_endgaps)
        if self.no_lonely_pairs:
            kw["no_lonely_pairs"] = True
        for k in ("normalized", "penalized"):
            if k in self.opts:
                kw[k] = int(self.opts[k])
        return kw


class GoldenPF:
    """LocARNA-P golden case (made by make_golden.py with LCG_GOLDEN_PF=1)."""

    def __init__(self, name):
        z = np.load(os.path.join(GOLDEN_DIR, name + ".npz"))
        self.name = name
        self.pp_a, self.pp_b = str(z["pp_a"]), str(z["pp_b"])
        self.seq_a, self.seq_b = str(z["seq_a"]), str(z["seq_b"])
        self.Z = float(z["Z"])
        self.am_ends = z["am"]
        self.am_p = z["am_p"]
        self.bm_ij = z["bm"]
        self.bm_p = z["bm_p"]
        self.opts = json.loads(str(z["opts"])) if "opts" in z else {}
        # AlignerPParams::min_am_prob the reference ran with (0: exact marginals)
        self.min_am_prob = float(self.opts.get("min_am_prob", 0.0))
        self.min_col, self.max_col = z["min_col"], z["max_col"]
        n, m = len(self.seq_a), len(self.seq_b)
        self.tables = PairTables(
            n, m, z["sigma"].astype(np.int32), z["gap_a"], z["gap_b"],
            int(z["indel_opening"]), int(z["exclusion"]), z["arcs_a"], z["arcs_b"],
            z["am_arcs"], z["am_score"], self.min_col, self.max_col,
            seq_a=self.seq_a, seq_b=self.seq_b,
            am_stack_score=z["am_stack_score"] if "am_stack_score" in z else None,
            am_stackable=z["am_stackable"] if "am_stackable" in z else None)

    def am_by_ends(self):
        return {tuple(int(v) for v in e): float(p) for e, p in zip(self.am_ends, self.am_p)}

    def bm_dense(self):
        n, m = len(self.seq_a), len(self.seq_b)
        out = np.zeros((n + 1, m + 1))
        for (i, j), p in zip(self.bm_ij, self.bm_p):
            out[i, j] = p
        return out


def pf_golden_names():
    return [n for n in golden_names() if n.startswith("pf")]
