"""Host preparation errors reported as the reference reports them (CPU):
anchor names out of order or of the wrong length, stacking columns without
the #STACK keyword, alignment rows of different lengths."""
import pytest

from locarna_gb300.engine import LcgError
from locarna_gb300.prep import prepare_pair
from locarna_gb300.synth import make_rna


def _pp(seq_lines, pairs="1 10 0.5"):
    return "\n".join(["#PP 2.0", ""] + seq_lines + ["", "#END", "", "#SECTION BASEPAIRS", "", pairs, "", "#END", ""])


def test_strict_anchor_names_must_be_ordered():
    a = make_rna(40, 1)
    anc = ["."] * 40
    anc[5], anc[20] = "B", "A"
    pp = a.to_pp(anchors="".join(anc))
    with pytest.raises(LcgError, match="lexicographic"):
        prepare_pair(pp, pp)
    prepare_pair(pp, pp, relaxed_anchors=1)  # relaxed names may come in any order


def test_anchor_line_length_must_match_the_sequence():
    seq = "ACGUACGUACGUACGU"
    pp = _pp([f"s {seq}", "#A1 ..A.."])
    with pytest.raises(LcgError, match="same length"):
        prepare_pair(pp, pp)


def test_stacking_columns_need_the_stack_keyword():
    seq = "ACGUACGUACGUACGU"
    pp = _pp([f"s {seq}"], pairs="1 10 0.5 0.2")
    with pytest.raises(LcgError, match="stack keyword"):
        prepare_pair(pp, pp, new_stacking=1)
    prepare_pair(pp, pp)  # without stacking the fourth column is not read


def test_alignment_rows_must_have_equal_lengths():
    pp = _pp(["r1 ACGUACGUACGU", "r2 ACGUACGUAC"])
    with pytest.raises(LcgError, match="different lengths"):
        prepare_pair(pp, pp)


def test_unpaired_penalty_shifts_base_match_and_gap_tables():
    """--unpaired-penalty (Scoring::apply_unpaired_penalty, scoring.cc:65-74):
    every base-match score lowered by twice the penalty and every gap cost by
    the penalty; with RIBOSUM the arc-match scores do not read σ and stay."""
    import numpy as np
    from locarna_gb300.synth import make_rna
    a, b = make_rna(70, 41).to_pp(), make_rna(80, 42).to_pp()
    t0 = prepare_pair(a, b)
    t1 = prepare_pair(a, b, unpaired_penalty=30)
    assert np.array_equal(np.asarray(t1.sigma), np.asarray(t0.sigma) - 60)
    assert np.array_equal(np.asarray(t1.gap_a), np.asarray(t0.gap_a) - 30)
    assert np.array_equal(np.asarray(t1.gap_b), np.asarray(t0.gap_b) - 30)
    assert np.array_equal(np.asarray(t1.am_score), np.asarray(t0.am_score))
