"""LocARNA-P oracle (oracle/pf_oracle.c) against the reference's own partition
function and match probabilities (CPU). Identical arithmetic: exact match."""
import os

import numpy as np
import pytest

from golden_io import GOLDEN_DIR, GoldenPF, pf_golden_names
from oracle_ffi import oracle_pf


@pytest.mark.parametrize("name", pf_golden_names())
def test_pf_oracle_matches_reference(name):
    g = GoldenPF(name)
    t = g.tables
    Z, am, bm = oracle_pf(t, min_am_prob=g.min_am_prob)
    assert Z == g.Z
    A, B, AM = t.arcs_a.reshape(-1, 2), t.arcs_b.reshape(-1, 2), t.am_arcs.reshape(-1, 2)
    mine = {(int(A[a][0]), int(A[a][1]), int(B[b][0]), int(B[b][1])): am[k] for k, (a, b) in enumerate(AM)}
    for key, p in g.am_by_ends().items():
        assert mine[key] == p
    ref_bm = g.bm_dense()
    assert np.array_equal(bm[ref_bm != 0], ref_bm[ref_bm != 0])


@pytest.mark.parametrize("name", [n for n in pf_golden_names()
                                  if os.path.exists(os.path.join(GOLDEN_DIR, n + "_marginals.npz"))])
def test_pf_marginal_fixtures(name):
    """The finite-difference marginals of the reference's log Z are
    probabilities, and the fixture's reference values are the oracle's."""
    f = np.load(os.path.join(GOLDEN_DIR, name + "_marginals.npz"))
    assert f["am_fd"].min() >= -1e-9 and f["am_fd"].max() <= 1 + 1e-9
    assert f["bm_fd"].min() >= -1e-9 and f["bm_fd"].max() <= 1 + 1e-9
    _, am, bm = oracle_pf(GoldenPF(name).tables)
    assert np.array_equal(am[f["am_idx"]], f["am_ref"])
    assert np.array_equal(bm.reshape(-1)[f["bm_idx"]], f["bm_ref"])
