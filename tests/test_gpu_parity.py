"""GPU engine parity: through the C ABI, bit-exact against the reference's
golden results and against the oracle on the same tables."""
import pytest

from checks import assert_matches_golden, assert_same_result
from golden_io import Golden, sankoff_golden_names as golden_names
from oracle_ffi import oracle_align

GPU_CASES = golden_names()


@pytest.mark.gpu
@pytest.mark.parametrize("name", GPU_CASES)
def test_gpu_matches_reference(engine, name):
    g = Golden(name)
    res = engine.align_pairs([g.tables], **g.align_kwargs())[0]
    assert_matches_golden(g, res)


@pytest.mark.gpu
def test_gpu_batch_matches_oracle(engine):
    names = [n for n in GPU_CASES if not n.startswith("c400")]
    gs = [Golden(n) for n in names]
    # one batch per mode (the options are per call)
    by_mode = {}
    for g in gs:
        by_mode.setdefault(tuple(sorted(g.align_kwargs().items())), []).append(g)
    for mode, group in by_mode.items():
        kw = dict(mode)
        res = engine.align_pairs([g.tables for g in group] * 3, **kw)
        for k, r in enumerate(res):
            g = group[k % len(group)]
            assert_same_result(r, oracle_align(g.tables, **kw), g.name)
