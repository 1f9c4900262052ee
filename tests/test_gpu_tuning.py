"""The autotuner (lcg_engine_autotune / lcg_engine_set_autotune) on a GPU:
per length bucket a measured launch configuration of the fill; with it on,
lcg_align_pairs orders the batch by bucket and launches each bucket's chunks
with its configuration, and every pair's result is the same as without it
(and the oracle's)."""
import pytest

from checks import assert_same_result
from oracle_ffi import oracle_align


@pytest.mark.gpu
def test_autotuned_batches_give_the_same_alignments(engine):
    from concurrent.futures import ThreadPoolExecutor

    from locarna_gb300.prep import prepare_pair
    from locarna_gb300.synth import make_family
    fam = make_family(22, 60, 400, 515, q=0.05)
    pp = [r.to_pp() for r in fam]
    pairs = [(a, b) for a in range(len(fam)) for b in range(a + 1, len(fam))]
    with ThreadPoolExecutor(8) as ex:
        tables = list(ex.map(lambda ab: prepare_pair(pp[ab[0]], pp[ab[1]]), pairs))
    report = engine.autotune(tables, sample_pairs=12)
    assert len(report) == 4
    used = [r for r in report if r["pairs_sampled"] > 0]
    assert len(used) >= 3
    for r in used:
        assert r["trials"] == 12 and r["best_ms"] <= r["default_ms"]
        assert r["blocks_per_sm"] in (0, 2, 3) and r["wave_mb"] in (0, 4, 16, 64)
    base = engine.align_pairs(tables)
    try:
        engine.set_autotune(True)
        tuned = engine.align_pairs(tables)
        assert engine.last_stats()[1] >= 2 * len(used)  # at least one chunk per bucket
    finally:
        engine.set_autotune(False)
    for k, (a, b) in enumerate(zip(tuned, base)):
        assert_same_result(a, b, f"pair {k}")
    for k in range(0, len(tables), 37):
        assert_same_result(tuned[k], oracle_align(tables[k]), f"pair {k} vs oracle")


@pytest.mark.gpu
def test_chunks_replay_their_cuda_graph(engine):
    """lcg_align_pairs records each chunk's device work as a CUDA graph and
    replays it for a chunk with the same launch parameters; results equal the
    directly launched ones."""
    from golden_io import Golden, sankoff_golden_names
    gs = [Golden(n) for n in sankoff_golden_names() if n.startswith(("c150_g", "c150_b", "c200", "h150_g"))]
    tabs = [g.tables for g in gs] * 8
    try:
        engine.set_graphs(False)
        direct = engine.align_pairs(tabs)
        assert engine.last_graphs() == (0, 0)
        engine.set_graphs(True)
        call = engine.prepare_call(tabs)
        engine.run_call(call)
        first = engine.last_graphs()
        engine.run_call(call)
        again = engine.last_graphs()
        res = engine.decode_call(call)
    finally:
        engine.set_graphs(True)
    assert first[0] >= 1
    assert again[1] >= 1 and again[0] == 0
    for k, (a, b) in enumerate(zip(res, direct)):
        assert_same_result(a, b, f"pair {k}")


@pytest.mark.gpu
def test_graph_across_many_layouts_keeps_results(engine):
    """70 chunk layouts in a row through one engine (the arena, staging and
    scratch grow along the way, which drops the buffer set's graph before
    the old buffers are freed): every new layout is captured, a repeat of
    the last one replays, and every call aligns like the oracle."""
    from golden_io import Golden
    from oracle_ffi import oracle_align
    from locarna_gb300.engine import Engine
    gs = [Golden(n) for n in ("c150_global", "c150_b", "c60_short", "c120_opening0")]
    ref = [oracle_align(g.tables) for g in gs]
    eng = Engine(0)  # fresh buffers and graphs
    try:
        for n in range(1, 71):  # 70 batch sizes = 70 layouts
            tabs = [gs[k % 4].tables for k in range(n)]
            res = eng.align_pairs(tabs)
            assert eng.last_graphs() == (1, 0), n
            for k, r in enumerate(res):
                assert_same_result(r, ref[k % 4], f"batch {n} pair {k}")
            if n % 10 == 0:
                again = eng.align_pairs(tabs)
                assert eng.last_graphs() == (0, 1), n
                for k, r in enumerate(again):
                    assert_same_result(r, ref[k % 4], f"replay {n} pair {k}")
    finally:
        eng.close()


@pytest.mark.gpu
def test_kept_rectangles_give_the_same_alignments(engine):
    """With the group rectangles kept (the traceback walks the fill's
    rectangles; eight state matrices for structure-local alignment) and
    without (it recomputes them), every golden case, a batch and the
    alignment modes give the same results."""
    from golden_io import Golden, sankoff_golden_names
    gs = [Golden(n) for n in sankoff_golden_names()]
    try:
        for g in gs:
            kw = g.align_kwargs()
            if g.kbest:
                continue
            engine.set_rect_budget(4 << 30)
            a = engine.align_pairs([g.tables], **kw)[0]
            engine.set_rect_budget(0)
            b = engine.align_pairs([g.tables], **kw)[0]
            assert_same_result(a, b, g.name)
        plain = dict(struct_local=False, sequ_local=False, free_endgaps="----")
        tabs = [g.tables for g in gs if not g.kbest and g.align_kwargs() == plain][:24]
        assert len(tabs) >= 8
        for kw in ({}, {"sequ_local": True}, {"sequ_local": True, "normalized": 100}, {"penalized": 50},
                   {"struct_local": True}, {"struct_local": True, "sequ_local": True}):
            engine.set_rect_budget(64 << 30)
            a = engine.align_pairs(tabs, **kw)
            engine.set_rect_budget(0)
            b = engine.align_pairs(tabs, **kw)
            for k, (x, y) in enumerate(zip(a, b)):
                assert_same_result(x, y, f"{kw} pair {k}")
        engine.set_rect_budget(4 << 30)
        ka = engine.align_kbest(tabs[:6], 4, sequ_local=True)
        engine.set_rect_budget(0)
        kb = engine.align_kbest(tabs[:6], 4, sequ_local=True)
        for k, (hx, hy) in enumerate(zip(ka, kb)):
            assert len(hx) == len(hy)
            for x, y in zip(hx, hy):
                assert_same_result(x, y, f"kbest pair {k}")
    finally:
        engine.set_rect_budget(-1)
