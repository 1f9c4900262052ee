"""The plain-C oracle against the reference's own golden results (CPU)."""
import pytest

from checks import assert_matches_golden
from golden_io import Golden, sankoff_golden_names as golden_names
from oracle_ffi import oracle_align

CPU_CASES = [n for n in golden_names() if not n.startswith("c400")]


@pytest.mark.parametrize("name", CPU_CASES)
def test_oracle_matches_reference(name):
    g = Golden(name)
    res = oracle_align(g.tables, **g.align_kwargs())
    assert_matches_golden(g, res)
