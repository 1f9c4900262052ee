"""LocARNA-P oracle (oracle/pf_oracle.c) against the reference's own partition
function and match probabilities (CPU). Identical arithmetic: exact match."""
import numpy as np
import pytest

from golden_io import GoldenPF, pf_golden_names
from oracle_ffi import oracle_pf


@pytest.mark.parametrize("name", pf_golden_names())
def test_pf_oracle_matches_reference(name):
    g = GoldenPF(name)
    t = g.tables
    Z, am, bm = oracle_pf(t)
    assert Z == g.Z
    A, B, AM = t.arcs_a.reshape(-1, 2), t.arcs_b.reshape(-1, 2), t.am_arcs.reshape(-1, 2)
    mine = {(int(A[a][0]), int(A[a][1]), int(B[b][0]), int(B[b][1])): am[k] for k, (a, b) in enumerate(AM)}
    for key, p in g.am_by_ends().items():
        assert mine[key] == p
    ref_bm = g.bm_dense()
    assert np.array_equal(bm[ref_bm != 0], ref_bm[ref_bm != 0])
