"""Alignment output formatting from raw traceback edges.

The engine returns the raw edges in the order the reference's traceback
appends them (Alignment::append, src/LocARNA/alignment.cc:91-95) and the traced
arc matches. These helpers restate the reference's post-processing:

* ``alignment_edges`` = Alignment::alignment_edges (alignment.cc:120-167):
  positions skipped by a local alignment become ``locality`` gaps;
* ``structure_strings`` = Alignment::dot_bracket_structureA/B
  (alignment.cc:215-239) with Alignment::add_basepairA/B (alignment.cc:97-107);
* ``alignment_strings`` = the per-row alignment strings the CLUSTAL writer
  prints (MultipleAlignment(const Alignment&), multiple_alignment.cc:153).

Edge ends are encoded as ints: a position p >= 1, or a gap ``-1 - code`` with
the reference's Gap codes (aux.hh:132-137): regular 0, loop 1, locality 2.
"""

GAP_REGULAR = -1
GAP_LOCALITY = -3
_SIMPLIFIED_GAP = "---."  # aux.cc:28, gap_symbol()


def _is_pos(x):
    return x > 0


def alignment_edges(raw_edges, len_a, len_b, only_local=False):
    res = []
    last_a, last_b = 1, 1
    for a, b in raw_edges:
        if _is_pos(a):
            for j in range(last_a, a):
                if not only_local:
                    res.append((j, GAP_LOCALITY))
                last_a += 1
        if _is_pos(b):
            for j in range(last_b, b):
                if not only_local:
                    res.append((GAP_LOCALITY, j))
                last_b += 1
        if _is_pos(a):
            last_a += 1
        if _is_pos(b):
            last_b += 1
        res.append((a if a > 0 else GAP_REGULAR, b if b > 0 else GAP_REGULAR))
    if not only_local:
        for j in range(last_a, len_a + 1):
            res.append((j, GAP_LOCALITY))
            last_a += 1
        for j in range(last_b, len_b + 1):
            res.append((GAP_LOCALITY, j))
            last_b += 1
    return res


def _gap_char(code):
    return _SIMPLIFIED_GAP[-1 - code]


def structure_strings(edges, len_a, len_b, traced_arcs):
    """traced_arcs: list of ((al, ar), (bl, br)) of the traced arc matches."""
    str_a = ["."] * (len_a + 1)
    str_b = ["."] * (len_b + 1)
    for (al, ar), (bl, br) in traced_arcs:
        str_a[al], str_a[ar] = "(", ")"
        str_b[bl], str_b[br] = "(", ")"
    sa = "".join(str_a[a] if a > 0 else _gap_char(a) for a, _ in edges)
    sb = "".join(str_b[b] if b > 0 else _gap_char(b) for _, b in edges)
    return sa, sb


def alignment_strings(edges, seq_a, seq_b):
    sa = "".join(seq_a[a - 1] if a > 0 else _gap_char(a) for a, _ in edges)
    sb = "".join(seq_b[b - 1] if b > 0 else _gap_char(b) for _, b in edges)
    return sa, sb
