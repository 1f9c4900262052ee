"""The plain-C oracle against the reference's own golden results (CPU)."""
import pytest

from checks import assert_kbest_matches_golden, assert_matches_golden
from golden_io import Golden, sankoff_golden_names as golden_names
from oracle_ffi import oracle_align, oracle_kbest

CPU_CASES = [n for n in golden_names() if not n.startswith("c400")]


@pytest.mark.parametrize("name", CPU_CASES)
def test_oracle_matches_reference(name):
    g = Golden(name)
    if g.kbest:
        hits, stale = oracle_kbest(g.tables, *g.kbest, stale=True, **g.align_kwargs())
        assert stale == 0  # no out-of-band argmax: the defined rule is the reference's
        assert_kbest_matches_golden(g, hits)
        return
    res = oracle_align(g.tables, **g.align_kwargs())
    assert_matches_golden(g, res)
