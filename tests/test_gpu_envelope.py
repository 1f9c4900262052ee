"""Batched table preparation with the sequence envelope on the GPU
(lcg_prepare_pairs): the tables equal the host path's (lcg_prepare_pair, the
reference's envelope in its own precision) and the reference's golden tables,
and almost every envelope is decided on the GPU."""
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

from golden_io import Golden, sankoff_golden_names
from test_prep_golden import prep_kwargs

FIELDS = ("sigma", "gap_a", "gap_b", "arcs_a", "arcs_b", "am_arcs", "am_score", "min_col", "max_col")


def _same_tables(t, r, what):
    assert (t.len_a, t.len_b) == (r.len_a, r.len_b), what
    for f in FIELDS:
        assert np.array_equal(getattr(t, f), getattr(r, f)), f"{what}: {f} differs"
    assert t.envelope_ok == r.envelope_ok, what


@pytest.mark.gpu
@pytest.mark.parametrize("name", sankoff_golden_names())
def test_gpu_envelope_matches_reference_tables(engine, name):
    from locarna_gb300.prep import prepare_pairs
    g = Golden(name)
    (t,), nhost = prepare_pairs(engine, [(g.pp_a, g.pp_b)], **prep_kwargs(g))
    r = g.tables
    assert np.array_equal(t.min_col, r.min_col) and np.array_equal(t.max_col, r.max_col), "band differs"
    assert np.array_equal(t.am_arcs, r.am_arcs) and np.array_equal(t.am_score, r.am_score)
    # profiles (alignment rows) take the host envelope; sequences the GPU's
    def rows(pp):
        sec = pp.split("#END")[0].splitlines()[1:]
        return sum(1 for l in sec if l.strip() and not l[0].isspace() and not l.startswith("#"))
    profile = rows(g.pp_a) > 1 or rows(g.pp_b) > 1
    if prep_kwargs(g).get("min_trace_probability", 1e-4) > 0:
        assert nhost == (1 if profile else 0)


OPTION_SETS = [
    {},
    {"pf_precision": 0, "min_trace_probability": 1e-5},
    {"sequ_local": 1},
    {"free_endgaps": "+-+-"},
    {"free_endgaps": "++++", "indel_opening": -500},
    {"max_diff": 25},
]


@pytest.mark.gpu
@pytest.mark.parametrize("kw", OPTION_SETS, ids=lambda k: ",".join(f"{a}={b}" for a, b in k.items()) or "default")
def test_gpu_envelope_matches_host_prep(engine, kw):
    from locarna_gb300.prep import prepare_pair, prepare_pairs
    from locarna_gb300.synth import make_family
    fam = make_family(16, 40, 220, 404, q=0.05)
    pp = [r.to_pp() for r in fam]
    pairs = [(pp[a], pp[b]) for a in range(len(pp)) for b in range(a + 1, len(pp))]
    got, nhost = prepare_pairs(engine, pairs, **kw)
    with ThreadPoolExecutor(8) as ex:
        ref = list(ex.map(lambda ab: prepare_pair(ab[0], ab[1], **kw), pairs))
    for k, (t, r) in enumerate(zip(got, ref)):
        _same_tables(t, r, f"pair {k}")
    assert nhost <= max(2, len(pairs) // 50), f"{nhost} of {len(pairs)} envelopes took the host path"


@pytest.mark.gpu
def test_gpu_envelope_off_and_errors(engine):
    from locarna_gb300.engine import LcgError
    from locarna_gb300.prep import prepare_pair, prepare_pairs
    from locarna_gb300.synth import make_rna
    a, b = make_rna(80, 1).to_pp(), make_rna(90, 2).to_pp()
    (t,), nhost = prepare_pairs(engine, [(a, b)], min_trace_probability=0.0)
    _same_tables(t, prepare_pair(a, b, min_trace_probability=0.0), "no envelope")
    assert nhost == 0
    with pytest.raises(LcgError):
        prepare_pairs(engine, [(a, b), (a, "not a PP file")])
