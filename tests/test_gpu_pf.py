"""LocARNA-P on the GPU through the C ABI (lcg_pf_forward / lcg_pf_backward).

* log Z (FP64) equals the reference's Z (golden, from the reference itself).
* Probabilities (FP64) are the match probabilities of the reference's own
  partition function: T * d log Z / d score, evaluated on the reference's
  log Z by finite differences (tests/golden/make_pf_marginals.py), within
  1e-9. Where the reference's outside pass (AlignerP::align_outside,
  aligner_p.icc:1113-1139) is consistent with its Z, they equal the
  reference's printed probabilities within 1e-9 (pf90_b: every arc match and
  base match). On pf150 / pf200 the reference's outside pass returns
  negative probabilities for hundreds of arc matches and its values change
  with pf_scale; the adjoint pass does neither. The cause is in the
  reference: case 5 of comp_Mprime_entry reads Mprime cells outside the band
  that hold the debugging fill value -1 (aligner_p.icc:921;
  tests/test_pf_outside_fill.py shows that with 0 there its outside pass
  gives these marginals).
* These compare the exact marginals (min_am_prob = 0). With locarna_p's
  default min_am_prob = 0.001 the base-match probabilities leave out the
  contributions inside arc matches of probability <= sqrt(min_am_prob), as
  the reference's compute_basematch_probabilities does
  (aligner_p.icc:1201-1327); test_pf64_default_semantics_match_reference
  checks them against the reference's default output.
* FP32 with per-position scaling: probabilities within 1e-5 absolute of the
  FP64 values, log Z within 1e-5 relative.
* Gradients of log Z from the backward pass against central finite differences
  of the FP64 forward (h = 1e-3 on the continuous parameter offsets), 1e-4
  relative.
"""
import math
import os

import numpy as np
import pytest

from golden_io import GOLDEN_DIR, GoldenPF, pf_golden_names
from oracle_ffi import oracle_pf

PF_CASES = pf_golden_names()
FD_CASES = [n for n in PF_CASES if os.path.exists(os.path.join(GOLDEN_DIR, n + "_marginals.npz"))]
EXACT_CASES = ["pf90_b"]  # the reference's own probabilities are its marginals here

P64_TOL = 1e-9   # FP64 probabilities: same quantity, different summation order
P32_TOL = 1e-5   # FP32 probabilities vs FP64 (absolute)
LZ32_REL = 1e-5  # FP32 log Z (relative)
GRAD_REL = 1e-4  # adjoint gradient vs central finite differences (relative)
FD_H = 1e-3


def _prepared(g):
    from locarna_gb300.prep import prepare_pair
    t = prepare_pair(g.pp_a, g.pp_b, min_trace_probability=1e-5, pf_precision=0)
    return t


@pytest.mark.gpu
@pytest.mark.parametrize("name", PF_CASES)
def test_pf64_log_z_matches_reference(engine, name):
    g = GoldenPF(name)
    lz = engine.pf_forward([g.tables], precision=64, min_am_prob=0.0)[0]
    assert abs(lz - math.log(g.Z)) <= 1e-10 * max(1.0, abs(lz)), (lz, math.log(g.Z))
    r = engine.pf_backward()[0]
    assert r["log_z"] == lz
    assert r["am_prob"].min() >= -1e-12 and r["am_prob"].max() <= 1 + 1e-9
    assert r["bm_prob"].min() >= -1e-12 and r["bm_prob"].max() <= 1 + 1e-9


@pytest.mark.gpu
@pytest.mark.parametrize("name", FD_CASES)
def test_pf64_probabilities_are_marginals_of_reference_z(engine, name):
    g = GoldenPF(name)
    f = np.load(os.path.join(GOLDEN_DIR, name + "_marginals.npz"))
    engine.pf_forward([g.tables], precision=64, min_am_prob=0.0)
    r = engine.pf_backward()[0]
    assert np.max(np.abs(r["am_prob"][f["am_idx"]] - f["am_fd"])) <= P64_TOL
    assert np.max(np.abs(r["bm_prob"].reshape(-1)[f["bm_idx"]] - f["bm_fd"])) <= P64_TOL
    # where the reference's own value is its marginal, ours equals it
    ok = np.abs(f["am_ref"] - f["am_fd"]) <= 1e-10
    assert ok.sum() > 0
    assert np.max(np.abs(r["am_prob"][f["am_idx"][ok]] - f["am_ref"][ok])) <= P64_TOL


@pytest.mark.gpu
@pytest.mark.parametrize("name", EXACT_CASES)
def test_pf64_matches_reference_probabilities(engine, name):
    g = GoldenPF(name)
    t = g.tables
    engine.pf_forward([t], precision=64, min_am_prob=0.0)
    r = engine.pf_backward()[0]
    Z, am, bm = oracle_pf(t)
    assert np.max(np.abs(r["am_prob"] - am)) <= P64_TOL
    assert np.max(np.abs(r["bm_prob"] - bm)) <= P64_TOL
    # the probabilities the reference printed
    A, B, AM = t.arcs_a.reshape(-1, 2), t.arcs_b.reshape(-1, 2), t.am_arcs.reshape(-1, 2)
    mine = {(int(A[a][0]), int(A[a][1]), int(B[b][0]), int(B[b][1])): r["am_prob"][k]
            for k, (a, b) in enumerate(AM)}
    for key, p in g.am_by_ends().items():
        assert abs(mine[key] - p) <= P64_TOL


@pytest.mark.gpu
@pytest.mark.parametrize("name", PF_CASES)
def test_pf32_scaled_within_tolerance(engine, name):
    g = GoldenPF(name)
    t = g.tables
    engine.pf_forward([t], precision=64, min_am_prob=0.0)
    r64 = engine.pf_backward()[0]
    lz = engine.pf_forward([t], precision=32, min_am_prob=0.0)[0]
    r = engine.pf_backward()[0]
    assert abs(lz - math.log(g.Z)) <= LZ32_REL * abs(math.log(g.Z))
    err_am = np.max(np.abs(r["am_prob"] - r64["am_prob"]))
    err_bm = np.max(np.abs(r["bm_prob"] - r64["bm_prob"]))
    assert err_am <= P32_TOL, err_am
    assert err_bm <= P32_TOL, err_bm


@pytest.mark.gpu
def test_pf_probabilities_only_pass(engine):
    """gap_gradients = 0: the backward pass reads only M of each recomputed
    rectangle; the probabilities (exact and truncated) and the struct-weight /
    base-match gradients are those of the full pass, the gap counts NaN."""
    gs = [GoldenPF(n) for n in PF_CASES]
    tabs = [_prepared(g) for g in gs]
    for prec in (64, 32):
        tol = 1e-12 if prec == 64 else 1e-6
        for mam in (0.0, 0.001):
            engine.pf_forward(tabs, precision=prec, min_am_prob=mam)
            full = engine.pf_backward()
            engine.pf_forward(tabs, precision=prec, min_am_prob=mam, gap_gradients=False)
            lean = engine.pf_backward()
            for a, b in zip(full, lean):
                # the forward pass is the same; its arc-term sums are shared-
                # memory atomics, so the summation order may differ
                assert abs(a["log_z"] - b["log_z"]) <= tol * max(1.0, abs(a["log_z"]))
                assert np.max(np.abs(a["am_prob"] - b["am_prob"])) <= tol
                assert np.max(np.abs(a["bm_prob"] - b["bm_prob"])) <= tol
                assert abs(a["dlogz_dstruct_weight"] - b["dlogz_dstruct_weight"]) <= tol * max(
                    1.0, abs(a["dlogz_dstruct_weight"]))
                assert np.max(np.abs(a["dlogz_dbasematch"] - b["dlogz_dbasematch"])) <= tol * max(
                    1.0, np.max(np.abs(a["dlogz_dbasematch"])))
                assert math.isfinite(a["dlogz_dindel"]) and math.isnan(b["dlogz_dindel"])
                assert math.isnan(b["gap_ext_uses"]) and math.isnan(b["gap_open_uses"])


@pytest.mark.gpu
def test_pf_batch_equals_single(engine):
    gs = [GoldenPF(n) for n in PF_CASES]
    tabs = [g.tables for g in gs] * 2
    for prec in (64, 32):
        lzb = engine.pf_forward(tabs, precision=prec, min_am_prob=0.0)
        rb = engine.pf_backward()
        for k, t in enumerate(tabs):
            lz = engine.pf_forward([t], precision=prec, min_am_prob=0.0)[0]
            r = engine.pf_backward()[0]
            tol = 1e-12 if prec == 64 else 1e-6
            assert abs(lzb[k] - lz) <= tol * max(1.0, abs(lz))
            assert np.max(np.abs(rb[k]["am_prob"] - r["am_prob"])) <= (1e-12 if prec == 64 else 1e-6)


@pytest.mark.gpu
def test_pf_scale_and_temperature(engine):
    """log Z follows the reference for other pf_scale / temperature values;
    probabilities do not depend on pf_scale (a numerical scale factor)."""
    g = GoldenPF(PF_CASES[0])
    t = g.tables
    engine.pf_forward([t], precision=64, min_am_prob=0.0)
    base = engine.pf_backward()[0]
    for temp, scale in ((300.0, 2.0), (300.0, 0.5)):
        lz = engine.pf_forward([t], temperature=temp, pf_scale=scale, precision=64, min_am_prob=0.0)[0]
        r = engine.pf_backward()[0]
        Z, _, _ = oracle_pf(t, temperature=temp, pf_scale=scale, probs=False)
        assert abs(lz - math.log(Z)) <= 1e-10 * max(1.0, abs(lz))
        assert np.max(np.abs(r["am_prob"] - base["am_prob"])) <= 1e-12
        assert np.max(np.abs(r["bm_prob"] - base["bm_prob"])) <= 1e-12
    ge = GoldenPF(EXACT_CASES[0])
    for temp in (150.0, 600.0):
        lz = engine.pf_forward([ge.tables], temperature=temp, precision=64, min_am_prob=0.0)[0]
        r = engine.pf_backward()[0]
        Z, am, bm = oracle_pf(ge.tables, temperature=temp)
        assert abs(lz - math.log(Z)) <= 1e-10 * max(1.0, abs(lz))
        assert np.max(np.abs(r["am_prob"] - am)) <= P64_TOL
        assert np.max(np.abs(r["bm_prob"] - bm)) <= P64_TOL


def _fd_check(engine, t, k_param, grad, precision=64):
    d = np.zeros(19)
    d[k_param] = FD_H
    lp = engine.pf_forward([t], precision=precision, param_delta=d, min_am_prob=0.0)[0]
    lm = engine.pf_forward([t], precision=precision, param_delta=-d, min_am_prob=0.0)[0]
    fd = (lp - lm) / (2 * FD_H)
    assert abs(grad - fd) <= GRAD_REL * max(abs(fd), 1e-8), (k_param, grad, fd)


@pytest.mark.gpu
@pytest.mark.parametrize("name", PF_CASES)
def test_pf_gradients_match_finite_differences(engine, name):
    g = GoldenPF(name)
    t = _prepared(g)
    engine.pf_forward([t], precision=64, min_am_prob=0.0)
    r = engine.pf_backward()[0]
    grads = [r["dlogz_dindel"], r["dlogz_dindel_opening"], r["dlogz_dstruct_weight"]] + \
        list(r["dlogz_dbasematch"])
    for k, gr in enumerate(grads):
        if k >= 3 and gr == 0.0:
            continue  # base-type pair absent from the pair
        _fd_check(engine, t, k, gr)


@pytest.mark.gpu
def test_pf32_gradients(engine):
    """FP32 backward: gradients within 1e-4 relative of the FP64 ones."""
    g = GoldenPF(PF_CASES[0])
    t = _prepared(g)
    engine.pf_forward([t], precision=64, min_am_prob=0.0)
    r64 = engine.pf_backward()[0]
    engine.pf_forward([t], precision=32, min_am_prob=0.0)
    r32 = engine.pf_backward()[0]
    for key in ("dlogz_dindel", "dlogz_dindel_opening", "dlogz_dstruct_weight"):
        assert abs(r32[key] - r64[key]) <= GRAD_REL * abs(r64[key]), key
    np.testing.assert_allclose(r32["dlogz_dbasematch"], r64["dlogz_dbasematch"], rtol=GRAD_REL, atol=1e-9)


@pytest.mark.gpu
def test_pf_backward_needs_forward(engine):
    from locarna_gb300.engine import LcgError
    g = GoldenPF(PF_CASES[0])
    engine.pf_forward([g.tables], min_am_prob=0.0)
    engine.pf_backward()
    with pytest.raises(LcgError):
        engine.pf_backward()


DEFAULT_CASES = [n for n in PF_CASES if n.endswith("_default")]


@pytest.mark.gpu
@pytest.mark.parametrize("name", DEFAULT_CASES)
def test_pf64_default_semantics_match_reference(engine, name):
    """locarna_p's default --min-am-prob 0.001: arc-match probabilities and
    the truncated base-match probabilities (no contributions from inside arc
    matches of probability <= sqrt(0.001)) against the reference's own output
    of the same run (cases where its outside pass agrees with its Z)."""
    g = GoldenPF(name)
    assert g.min_am_prob == 0.001
    t = g.tables
    engine.pf_forward([t], precision=64, min_am_prob=g.min_am_prob)
    r = engine.pf_backward()[0]
    A, B, AM = t.arcs_a.reshape(-1, 2), t.arcs_b.reshape(-1, 2), t.am_arcs.reshape(-1, 2)
    mine = {(int(A[a][0]), int(A[a][1]), int(B[b][0]), int(B[b][1])): r["am_prob"][k]
            for k, (a, b) in enumerate(AM)}
    for key, p in g.am_by_ends().items():
        assert abs(mine[key] - p) <= P64_TOL, (key, mine[key], p)
    ref_bm = g.bm_dense()
    assert np.max(np.abs(r["bm_prob"] - ref_bm)) <= P64_TOL
    # the exact marginals differ: the truncation is what the reference reports
    engine.pf_forward([t], precision=64, min_am_prob=0.0)
    exact = engine.pf_backward()[0]
    assert np.max(np.abs(exact["bm_prob"] - ref_bm)) > 10 * P64_TOL


@pytest.mark.gpu
def test_pf_kept_rectangles_give_the_same_results(engine):
    """With the groups' rectangles kept by the forward pass (the backward
    reads them; M alone, or M, E and F for the gap gradients) and without
    (the backward recomputes them), log Z, the probabilities (exact and
    truncated) and every gradient agree."""
    gs = [GoldenPF(n) for n in PF_CASES]
    tabs = [_prepared(g) for g in gs]
    keys = ("dlogz_dindel", "dlogz_dindel_opening", "dlogz_dstruct_weight")
    try:
        for prec in (64, 32):
            tol = 1e-12 if prec == 64 else 1e-6
            for mam in (0.0, 0.001):
                for grads in (True, False):
                    out = []
                    for budget in (16 << 30, 0):
                        engine.set_rect_budget(budget)
                        lz = engine.pf_forward(tabs, precision=prec, min_am_prob=mam, gap_gradients=grads)
                        out.append((lz, engine.pf_backward()))
                    (lza, ra), (lzb, rb) = out
                    for k, (a, b) in enumerate(zip(ra, rb)):
                        assert abs(lza[k] - lzb[k]) <= tol * max(1.0, abs(lzb[k]))
                        assert np.max(np.abs(a["am_prob"] - b["am_prob"])) <= tol
                        assert np.max(np.abs(a["bm_prob"] - b["bm_prob"])) <= tol
                        for key in keys if grads else keys[2:]:
                            assert abs(a[key] - b[key]) <= tol * max(1.0, abs(b[key])), key
                        assert np.max(np.abs(a["dlogz_dbasematch"] - b["dlogz_dbasematch"])) <= tol * max(
                            1.0, np.max(np.abs(b["dlogz_dbasematch"])))
    finally:
        engine.set_rect_budget(-1)
