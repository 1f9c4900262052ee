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


@pytest.mark.gpu
def test_gpu_allpairs_workload_sample_matches_oracle(engine):
    """The all-pairs workload itself (64 RNAs of 60-400 nt, seed 2024, the
    benchmark's family): a length-stratified sample of 202 of its 2,016 pairs
    (every 10th pair in order of lenA x lenB) aligned in one lcg_align_pairs
    call, every pair equal to the oracle: score, end cells, raw traceback
    edges and traced arc matches."""
    from concurrent.futures import ThreadPoolExecutor

    import bench
    from locarna_gb300.prep import prepare_pair
    from oracle_pool import oracle_align_many
    pp, pairs = bench.workload_pp()
    from locarna_gb300.synth import make_family
    W = bench.WORKLOAD
    fam = make_family(W["count"], W["len_lo"], W["len_hi"], W["seed"], q=W["q"])
    lens = [len(r.seq) for r in fam]
    order = sorted(range(len(pairs)), key=lambda k: (lens[pairs[k][0]] * lens[pairs[k][1]], k))
    sample = [pairs[k] for k in order[::10]]
    assert len(sample) >= 200
    with ThreadPoolExecutor(8) as ex:
        tables = list(ex.map(lambda ab: prepare_pair(pp[ab[0]], pp[ab[1]]), sample))
    got = engine.align_pairs(tables)
    ref = oracle_align_many(tables)
    for k, (r, o) in enumerate(zip(got, ref)):
        assert_same_result(r, o, f"workload pair {sample[k]}")


@pytest.mark.gpu
def test_gpu_chunk_pipeline_matches_oracle(engine):
    """lcg_align_pairs' chunk pipeline (two buffer sets, host preparation of
    chunk k+1 during the device work of chunk k): automatic chunks for a
    300-pair batch, then 7-pair chunks, equal the oracle pair by pair and the
    one-chunk call bit for bit."""
    from concurrent.futures import ThreadPoolExecutor

    from locarna_gb300.prep import prepare_pair
    from locarna_gb300.synth import make_family
    fam = make_family(25, 50, 110, 77, q=0.05)
    pp = [r.to_pp() for r in fam]
    pairs = [(a, b) for a in range(len(fam)) for b in range(a + 1, len(fam))]
    with ThreadPoolExecutor(8) as ex:
        tables = list(ex.map(lambda ab: prepare_pair(pp[ab[0]], pp[ab[1]]), pairs))
    assert len(tables) == 300
    try:
        engine.set_chunk_pairs(len(tables))
        one = engine.align_pairs(tables)
        assert engine.last_stats()[1] == 2
        engine.set_chunk_pairs(0)
        auto = engine.align_pairs(tables)
        assert engine.last_stats()[1] == 4  # two chunks of 150 pairs
        engine.set_chunk_pairs(7)
        small = engine.align_pairs(tables)
        assert engine.last_stats()[1] == 2 * 43
    finally:
        engine.set_chunk_pairs(0)
    for k, t in enumerate(tables):
        ref = oracle_align(t)
        assert_same_result(one[k], ref, f"pair {k}")
        assert_same_result(auto[k], ref, f"pair {k} (automatic chunks)")
        assert_same_result(small[k], ref, f"pair {k} (7-pair chunks)")


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [{}, {"struct_local": True}, {"sequ_local": True},
                                  {"free_endgaps": "+-+-"}])
def test_gpu_no_lonely_pairs_matches_oracle(engine, mode):
    """locarna --noLP (fill_D_entries_noLP, trace_arcmatch_noLP): a batch of
    synthetic pairs with planted stems, every pair bit-exact against the
    oracle (score, end cells, edges, traced arc matches)."""
    from locarna_gb300.prep import prepare_pair
    from locarna_gb300.synth import make_family
    fam = make_family(9, 60, 170, 91, q=0.05)
    pp = [r.to_pp() for r in fam]
    tables = [prepare_pair(pp[a], pp[b]) for a in range(len(fam)) for b in range(a + 1, len(fam))]
    kw = dict(mode, no_lonely_pairs=True)
    res = engine.align_pairs(tables, **kw)
    stacked = 0
    for k, t in enumerate(tables):
        ref = oracle_align(t, **kw)
        assert_same_result(res[k], ref, f"pair {k}")
        stacked += len(ref.traced_am)
    assert stacked > 0


def _homolog_tables(prep_kw, count=4, length=140, seed=301):
    """All pairs of a few RNAs and their homologs (shared stems), with #STACK
    joint probabilities in the inputs."""
    from locarna_gb300.prep import prepare_pair
    from locarna_gb300.synth import make_homolog, make_rna
    recs = []
    for k in range(count):
        r = make_rna(length + 7 * k, seed + k)
        recs += [r, make_homolog(r, seed + 100 + k)]
    pp = [r.to_pp(stacking=True) for r in recs]
    return [prepare_pair(pp[a], pp[b], **prep_kw) for a in range(len(pp)) for b in range(a + 1, len(pp))]


@pytest.mark.gpu
@pytest.mark.parametrize("prep_kw,mode", [
    ({"stacking": 1, "exp_prob": 0.005}, {}),
    ({"new_stacking": 1}, {"no_lonely_pairs": True}),
    ({"stacking": 1, "new_stacking": 1, "exp_prob": 0.004}, {"struct_local": True}),
    ({"stacking": 1, "exp_prob": 0.006}, {"sequ_local": True, "no_lonely_pairs": True}),
    ({"new_stacking": 1}, {"struct_local": True, "no_lonely_pairs": True}),
])
def test_gpu_stacking_matches_oracle(engine, prep_kw, mode):
    """locarna --stacking / --new-stacking (stacked arc-match scores in
    fill_D_entries, fill_D_entries_noLP and trace_arcmatch): homologous pairs,
    every pair bit-exact against the oracle."""
    tables = _homolog_tables(prep_kw)
    assert all(t.am_stack_score is not None for t in tables)
    res = engine.align_pairs(tables, **mode)
    traced = 0
    for k, t in enumerate(tables):
        ref = oracle_align(t, **mode)
        assert_same_result(res[k], ref, f"pair {k}")
        traced += len(ref.traced_am)
    assert traced > 50


@pytest.mark.gpu
@pytest.mark.parametrize("prep_kw,mode", [
    ({}, {"sequ_local": True, "normalized": 100}),
    ({}, {"sequ_local": True, "normalized": 0, "no_lonely_pairs": True}),
    ({"stacking": 1, "exp_prob": 0.005}, {"sequ_local": True, "normalized": 400}),
    ({}, {"sequ_local": True, "penalized": 30}),
    ({}, {"penalized": 15, "free_endgaps": "++++"}),
    ({"new_stacking": 1}, {"sequ_local": True, "penalized": 20, "struct_local": True}),
])
def test_gpu_normalized_penalized_matches_oracle(engine, prep_kw, mode):
    """locarna --normalized L (Dinkelbach iterations of the top level) and
    --penalized PP: homologous and unrelated pairs in one batch, every pair
    bit-exact against the oracle (score, end cells, edges, traced arc
    matches)."""
    tables = _homolog_tables(prep_kw, count=3, length=120, seed=401)
    res = engine.align_pairs(tables, **mode)
    for k, t in enumerate(tables):
        ref = oracle_align(t, **mode)
        assert_same_result(res[k], ref, f"pair {k}")
        assert res[k].min_ij == ref.min_ij, (k, res[k].min_ij, ref.min_ij)


@pytest.mark.gpu
def test_gpu_normalized_rejects_global_mode(engine):
    from locarna_gb300.engine import LcgError
    g = Golden("c60_short")
    with pytest.raises(LcgError):
        engine.align_pairs([g.tables], normalized=100)
    with pytest.raises(LcgError):
        engine.align_pairs([g.tables], sequ_local=True, normalized=100, penalized=10)


@pytest.mark.gpu
@pytest.mark.parametrize("name", [n for n in GPU_CASES if "kbest" in n])
def test_gpu_kbest_matches_reference(engine, name):
    """locarna --kbest k (Aligner::suboptimal, interval splitting): every hit
    of the reference's enumeration, in order, bit-exact through
    lcg_align_kbest."""
    from checks import assert_kbest_matches_golden
    g = Golden(name)
    hits = engine.align_kbest([g.tables], *g.kbest, **g.align_kwargs())[0]
    assert_kbest_matches_golden(g, hits)


@pytest.mark.gpu
@pytest.mark.parametrize("prep_kw,mode,k,thr", [
    ({}, {"sequ_local": True}, 7, -1000000),
    ({}, {"sequ_local": True, "no_lonely_pairs": True}, 5, 800),
    ({"stacking": 1, "exp_prob": 0.005}, {"sequ_local": True, "struct_local": True}, 4, -1000000),
    ({}, {"free_endgaps": "++++"}, 3, -1000000),
    ({}, {}, 4, -1000000),
])
def test_gpu_kbest_matches_oracle(engine, prep_kw, mode, k, thr):
    """k-best hits of a batch of homologous and unrelated pairs against the
    oracle's restatement of Aligner::suboptimal, pair by pair and hit by hit.
    (Global intervals can end on cells outside the band, which both count as
    -inf; the reference reads stale matrix cells there.)"""
    from oracle_ffi import oracle_kbest
    tables = _homolog_tables(prep_kw, count=3, length=110, seed=501)
    got = engine.align_kbest(tables, k, thr, **mode)
    total = 0
    for q, t in enumerate(tables):
        ref = oracle_kbest(t, k, thr, **mode)
        assert len(got[q]) == len(ref), (q, len(got[q]), len(ref))
        for h, (a, b) in enumerate(zip(got[q], ref)):
            assert_same_result(a, b, f"pair {q} hit {h}")
        total += len(ref)
    assert total > len(tables)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [{}, {"sequ_local": True}, {"struct_local": True},
                                  {"no_lonely_pairs": True, "free_endgaps": "++++"}])
def test_gpu_profiles_match_oracle(engine, mode):
    """Profile (multiple alignment) inputs as in progressive alignment:
    profiles of 2-4 rows and single sequences, all pairs, prepared by
    lcg_prepare_pairs (profiles take the host envelope), bit-exact against
    the oracle."""
    from locarna_gb300.prep import prepare_pairs
    from locarna_gb300.synth import make_profile, make_rna
    recs = [make_profile(90 + 13 * k, 700 + k, 2 + k % 3) for k in range(5)] + [make_rna(100, 790)]
    pp = [r.to_pp() for r in recs]
    pairs = [(pp[a], pp[b]) for a in range(len(pp)) for b in range(a + 1, len(pp))]
    tables, nhost = prepare_pairs(engine, pairs)
    assert nhost == len(pairs)  # every pair has a profile
    res = engine.align_pairs(tables, **mode)
    for k, t in enumerate(tables):
        assert_same_result(res[k], oracle_align(t, **mode), f"pair {k}")


@pytest.mark.gpu
def test_gpu_kbest_normalized_matches_oracle(engine):
    """--kbest with --normalized: every interval scored by its Dinkelbach
    iterations; hits against the oracle, pair by pair."""
    from oracle_ffi import oracle_kbest
    tables = _homolog_tables({}, count=2, length=100, seed=601)
    mode = {"sequ_local": True, "normalized": 80}
    got = engine.align_kbest(tables, 4, -1000000, **mode)
    for q, t in enumerate(tables):
        ref = oracle_kbest(t, 4, -1000000, **mode)
        assert len(got[q]) == len(ref), (q, len(got[q]), len(ref))
        for h, (a, b) in enumerate(zip(got[q], ref)):
            assert_same_result(a, b, f"pair {q} hit {h}")


@pytest.mark.gpu
def test_gpu_pp_pipeline_matches_two_calls(engine):
    """lcg_align_pp_pairs (tables built chunk by chunk while the device aligns
    the previous chunk) gives what lcg_prepare_pairs + lcg_align_pairs give,
    in one chunk and in 9-pair chunks."""
    from locarna_gb300.prep import prepare_pairs
    from locarna_gb300.synth import make_family
    fam = make_family(12, 50, 160, 303, q=0.05)
    pp = [r.to_pp() for r in fam]
    pp_pairs = [(pp[a], pp[b]) for a in range(len(fam)) for b in range(a + 1, len(fam))]
    tables, _ = prepare_pairs(engine, pp_pairs)
    ref = engine.align_pairs(tables)
    lens = [(t.len_a, t.len_b) for t in tables]
    try:
        for chunk in (0, 9):
            engine.set_chunk_pairs(chunk)
            call = engine.prepare_pp_call(pp_pairs, lens)
            engine.run_pp_call(call)
            got = engine.decode_pp_call(call)
            for k, (a, b) in enumerate(zip(got, ref)):
                assert_same_result(a, b, f"pair {k} (chunk {chunk})")
    finally:
        engine.set_chunk_pairs(0)
