"""Host preparation (PP reading, scoring tables, arcs, arc matches, band with
the sequence envelope) against the reference's own tables (CPU)."""
import numpy as np
import pytest

from golden_io import Golden, sankoff_golden_names as golden_names

_OPT_MAP = {"sequ_local": ("sequ_local", int), "free_endgaps": ("free_endgaps", str),
            "min_trace_prob": ("min_trace_probability", float), "indel_opening": ("indel_opening", int),
            "struct_local": None, "no_lonely_pairs": None, "stacking": ("stacking", int),
            "new_stacking": ("new_stacking", int), "exp_prob": ("exp_prob", float),
            "normalized": None, "penalized": None, "kbest": None, "better": None, "anchors": None,
            "max_diff": ("max_diff", int), "max_diff_am": ("max_diff_am", int),
            "max_diff_at_am": ("max_diff_at_am", int)}


def prep_kwargs(g):
    kw = {}
    for k, v in g.opts.items():
        m = _OPT_MAP[k]
        if m is None:
            continue
        kw[m[0]] = m[1](v)
    return kw


@pytest.mark.parametrize("name", golden_names())
def test_prep_matches_reference_tables(name):
    from locarna_gb300.prep import prepare_pair
    g = Golden(name)
    t = prepare_pair(g.pp_a, g.pp_b, **prep_kwargs(g))
    r = g.tables
    assert t.seq_a == g.seq_a and t.seq_b == g.seq_b
    assert np.array_equal(t.min_col, r.min_col), "band min_col differs"
    assert np.array_equal(t.max_col, r.max_col), "band max_col differs"
    assert np.array_equal(t.gap_a, r.gap_a) and np.array_equal(t.gap_b, r.gap_b)
    assert t.indel_opening == r.indel_opening and t.exclusion == r.exclusion
    sig = t.sigma.reshape(t.len_a + 1, t.len_b + 1)[1:, 1:]
    assert np.array_equal(sig, r.sigma.reshape(r.len_a + 1, r.len_b + 1)[1:, 1:]), "sigma differs"
    assert np.array_equal(t.arcs_a, r.arcs_a) and np.array_equal(t.arcs_b, r.arcs_b), "arcs differ"
    assert np.array_equal(t.am_arcs, r.am_arcs), "arc match list differs"
    assert np.array_equal(t.am_score, r.am_score), "arc match scores differ"
    assert (t.anchors is None) == (r.anchors is None), "anchors on/off differ"
    if r.anchors is not None:
        for k in r.anchors:
            assert np.array_equal(t.anchors[k], r.anchors[k]), f"anchor ranges {k} differ"
        assert t.right_anchor == r.right_anchor and t.left_anchor == r.left_anchor, "outermost anchors differ"
    assert (t.am_stack_score is None) == (r.am_stack_score is None), "stacking on/off differs"
    if r.am_stack_score is not None:
        assert np.array_equal(t.am_stack_score, r.am_stack_score), "stacked arc match scores differ"
        assert np.array_equal(t.am_stackable, r.am_stackable), "stackable flags differ"
