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
