"""The reference's own example input (Data/Examples/example.pp of the
reference tree: a two-row alignment with two-line anchor names, #BPCUT,
stacking columns and comment lines) through the host preparation and the
oracle, against the reference's harness on the same file (CPU). Runs only
where the reference tree and its compiled harness exist: $LOCARNA_REF or a
checkout named "reference" beside the repository (oracle/build_ref.sh builds
the harness)."""
import os
import subprocess

import numpy as np
import pytest

from locarna_gb300.build import reference_tree
from refdump import parse_ref

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")


def _example():
    path = os.path.join(reference_tree(), "Data", "Examples", "example.pp")
    if not os.path.exists(path) or not os.path.exists(HARNESS):
        pytest.skip("reference tree or its harness not available")
    return path


@pytest.mark.parametrize("opts", [{}, {"sequ_local": "1"}, {"struct_local": "1"}])
def test_reference_example_tables_and_alignment(opts):
    from checks import assert_matches_golden
    from locarna_gb300.prep import prepare_pair
    from oracle_ffi import oracle_align
    path = _example()
    out = subprocess.run([HARNESS, path, path] + [f"{k}={v}" for k, v in opts.items()],
                         capture_output=True, text=True, check=True).stdout
    ref = parse_ref(out)
    r = ref["tables"]
    pp = open(path).read()
    t = prepare_pair(pp, pp, sequ_local=int(opts.get("sequ_local", 0)))
    for f in ("sigma", "gap_a", "gap_b", "arcs_a", "arcs_b", "am_arcs", "am_score", "min_col", "max_col"):
        assert np.array_equal(getattr(t, f), getattr(r, f)), f
    for k in r.anchors:
        assert np.array_equal(t.anchors[k], r.anchors[k]), k
    assert (t.right_anchor, t.left_anchor) == (r.right_anchor, r.left_anchor)

    class G:  # the reference's result in the shape assert_matches_golden reads
        name = "example.pp"
        tables = t
        score = ref["score"]
        edges = [tuple(e) for e in ref["edges"]]
        struct_a, struct_b = ref["struct_a"], ref["struct_b"]

    res = oracle_align(t, struct_local=opts.get("struct_local") == "1", sequ_local=opts.get("sequ_local") == "1")
    assert_matches_golden(G, res)


def test_relaxed_anchors_against_reference(tmp_path):
    """--relaxed-anchors: anchor names in any order; the host preparation's
    ranges, band and arc matches and the oracle's alignment against the
    reference's harness on an anchored synthetic pair."""
    from checks import assert_matches_golden
    from locarna_gb300.prep import prepare_pair
    from locarna_gb300.synth import make_homolog, make_rna
    from oracle_ffi import oracle_align
    _example()  # needs the reference tree and its harness
    a = make_rna(150, 81)
    b = make_homolog(a, 82)
    sa, sb = ["."] * 150, ["."] * 150
    for name, x, y in (("C", 20, 20), ("A", 75, 75), ("B", 130, 130)):  # not in lexicographic order
        sa[x - 1] = sb[y - 1] = name
    pa, pb = tmp_path / "a.pp", tmp_path / "b.pp"
    pa.write_text(a.to_pp(anchors="".join(sa)))
    pb.write_text(b.to_pp(anchors="".join(sb)))
    out = subprocess.run([HARNESS, str(pa), str(pb), "relaxed_anchors=1"], capture_output=True, text=True,
                         check=True).stdout
    ref = parse_ref(out)
    r = ref["tables"]
    t = prepare_pair(pa.read_text(), pb.read_text(), relaxed_anchors=1)
    for f in ("min_col", "max_col", "am_arcs", "am_score"):
        assert np.array_equal(getattr(t, f), getattr(r, f)), f
    for k in r.anchors:
        assert np.array_equal(t.anchors[k], r.anchors[k]), k

    class G:
        name = "relaxed anchors"
        tables = t
        score = ref["score"]
        edges = [tuple(e) for e in ref["edges"]]
        struct_a, struct_b = ref["struct_a"], ref["struct_b"]

    assert_matches_golden(G, oracle_align(t))
