"""Anchor constraints against the reference's own known-answer test
(src/Tests/anchor_constraints.cc: names of length 1, strict semantics,
sequences of 10 positions "A...B.C.EF" and "..A.BDEF.."): the allowed
match / deletion / insertion ranges the host preparation derives from the
PP #A1 lines, and the outermost anchors (AnchorConstraints::allowed_match,
allowed_del, allowed_ins, leftmost_anchor, rightmost_anchor; semantics in
anchor_constraints.hh:147-254)."""
from locarna_gb300.prep import prepare_pair
from locarna_gb300.synth import make_rna

ANCH_A, ANCH_B = "A...B.C.EF", "..A.BDEF.."


def _tables():
    a, b = make_rna(10, 101), make_rna(10, 202)
    return prepare_pair(a.to_pp(anchors=ANCH_A), b.to_pp(anchors=ANCH_B))


def test_anchor_ranges_match_the_reference_known_answers():
    t = _tables()
    r = t.anchors

    def match(i, j):
        return r["match_lo"][i] <= j <= r["match_hi"][i]

    def dele(i, j):
        return r["del_lo"][i] <= j <= r["del_hi"][i]

    def ins(i, j):  # insert j immediately right of i
        return r["ins_lo"][j] <= i <= r["ins_hi"][j]

    # allowed_match() works as expected
    assert match(5, 5)
    assert not match(4, 5)
    assert not match(5, 4)
    assert not match(5, 7)
    assert not match(3, 6)
    assert not match(6, 6)  # lexicographic order of constraints 3 and 4
    assert match(8, 6)
    assert not match(7, 6)
    # allowed_del() works as expected
    assert dele(6, 5)
    assert not dele(7, 6)
    assert not dele(5, 5)
    assert not dele(6, 4)  # 5~5 is anchored: 6 cannot go immediately right of 4
    assert not dele(6, 7)
    assert not dele(6, 6)
    # allowed_ins() works as expected
    assert ins(7, 6)
    assert not ins(5, 6)


def test_outermost_anchors_match_the_reference():
    t = _tables()
    assert tuple(t.left_anchor) == (1, 3)
    assert tuple(t.right_anchor) == (10, 8)
    # without anchors: leftmost (n+1, m+1), rightmost (0, 0)
    a, b = make_rna(10, 101), make_rna(10, 202)
    u = prepare_pair(a.to_pp(), b.to_pp())
    assert u.anchors is None
    assert tuple(u.left_anchor) == (11, 11) and tuple(u.right_anchor) == (0, 0)
