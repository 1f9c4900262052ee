"""Comparison of an engine/oracle result with the reference's golden result."""
from locarna_gb300.alignment import alignment_edges, structure_strings


def traced_arcs(tables, traced_am):
    out = []
    for k in traced_am:
        ia, ib = int(tables.am_arcs[2 * k]), int(tables.am_arcs[2 * k + 1])
        out.append(((int(tables.arcs_a[2 * ia]), int(tables.arcs_a[2 * ia + 1])),
                    (int(tables.arcs_b[2 * ib]), int(tables.arcs_b[2 * ib + 1]))))
    return out


def full_edges(tables, res):
    return alignment_edges(res.edges, tables.len_a, tables.len_b)


def assert_matches_golden(g, res):
    t = g.tables
    assert res.score == g.score, (g.name, res.score, g.score)
    edges = full_edges(t, res)
    assert edges == g.edges, (g.name, "edges differ")
    sa, sb = structure_strings(edges, t.len_a, t.len_b, traced_arcs(t, res.traced_am))
    assert sa == g.struct_a and sb == g.struct_b, (g.name, "structure strings differ")


def assert_same_result(a, b, name=""):
    assert a.score == b.score, (name, a.score, b.score)
    assert a.max_ij == b.max_ij, (name, a.max_ij, b.max_ij)
    assert a.edges == b.edges, (name, "raw edges differ")
    assert a.traced_am == b.traced_am, (name, "traced arc matches differ")


def assert_kbest_matches_golden(g, hits):
    """k-best hits (Aligner::suboptimal) against the reference's: score,
    full edges and structure strings of every hit, in order."""
    t = g.tables
    ref = g.kbest_hits()
    assert len(hits) == len(ref), (g.name, len(hits), len(ref))
    for h, (res, (sc, edges, (sa, sb))) in enumerate(zip(hits, ref)):
        assert res.score == sc, (g.name, h, res.score, sc)
        e = full_edges(t, res)
        assert e == edges, (g.name, h, "edges differ")
        ga, gb = structure_strings(e, t.len_a, t.len_b, traced_arcs(t, res.traced_am))
        assert (ga, gb) == (sa, sb), (g.name, h, "structure strings differ")
