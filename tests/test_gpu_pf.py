"""LocARNA-P on the GPU through the C ABI (lcg_pf_forward / lcg_pf_backward).

* FP64: log Z against the reference's Z (golden) and the oracle; arc-match and
  base-match probabilities against the oracle (restatement of AlignerP, exact
  against the reference) within 1e-9 absolute (summation order differs).
* FP32 with per-position scaling: probabilities within 1e-5 absolute of the
  FP64 oracle, log Z within 1e-5 relative.
* Gradients of log Z from the backward pass against central finite differences
  of the FP64 forward (h = 1e-3 on the continuous parameter offsets), 1e-4
  relative.
"""
import math

import numpy as np
import pytest

from golden_io import GoldenPF, pf_golden_names
from oracle_ffi import oracle_pf

PF_CASES = pf_golden_names()

P64_TOL = 1e-9   # FP64 probabilities: same recursion, different summation order
P32_TOL = 1e-5   # FP32 probabilities vs FP64 oracle (absolute)
LZ32_REL = 1e-5  # FP32 log Z (relative)
GRAD_REL = 1e-4  # adjoint gradient vs central finite differences (relative)
FD_H = 1e-3


def _prepared(g):
    from locarna_gb300.prep import prepare_pair
    t = prepare_pair(g.pp_a, g.pp_b, min_trace_probability=1e-5, pf_precision=0)
    return t


@pytest.mark.gpu
@pytest.mark.parametrize("name", PF_CASES)
def test_pf64_matches_oracle(engine, name):
    g = GoldenPF(name)
    t = g.tables
    lz = engine.pf_forward([t], precision=64)[0]
    assert abs(lz - math.log(g.Z)) <= 1e-10 * max(1.0, abs(lz)), (lz, math.log(g.Z))
    r = engine.pf_backward()[0]
    Z, am, bm = oracle_pf(t)
    assert abs(r["log_z"] - math.log(Z)) <= 1e-10 * max(1.0, abs(lz))
    assert np.max(np.abs(r["am_prob"] - am)) <= P64_TOL
    assert np.max(np.abs(r["bm_prob"] - bm)) <= P64_TOL
    # the reference's own written probabilities (those it printed)
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
    lz = engine.pf_forward([t], precision=32)[0]
    r = engine.pf_backward()[0]
    Z, am, bm = oracle_pf(t)
    assert abs(lz - math.log(Z)) <= LZ32_REL * abs(math.log(Z))
    err_am = np.max(np.abs(r["am_prob"] - am))
    err_bm = np.max(np.abs(r["bm_prob"] - bm))
    assert err_am <= P32_TOL, err_am
    assert err_bm <= P32_TOL, err_bm


@pytest.mark.gpu
def test_pf_batch_equals_single(engine):
    gs = [GoldenPF(n) for n in PF_CASES]
    tabs = [g.tables for g in gs] * 2
    for prec in (64, 32):
        lzb = engine.pf_forward(tabs, precision=prec)
        rb = engine.pf_backward()
        for k, t in enumerate(tabs):
            lz = engine.pf_forward([t], precision=prec)[0]
            r = engine.pf_backward()[0]
            tol = 1e-12 if prec == 64 else 1e-6
            assert abs(lzb[k] - lz) <= tol * max(1.0, abs(lz))
            assert np.max(np.abs(rb[k]["am_prob"] - r["am_prob"])) <= (1e-12 if prec == 64 else 1e-6)


@pytest.mark.gpu
def test_pf_scale_and_temperature(engine):
    g = GoldenPF(PF_CASES[0])
    t = g.tables
    for temp, scale in ((300.0, 2.0), (150.0, 0.5)):
        lz = engine.pf_forward([t], temperature=temp, pf_scale=scale, precision=64)[0]
        r = engine.pf_backward()[0]
        Z, am, bm = oracle_pf(t, temperature=temp, pf_scale=scale)
        assert abs(lz - math.log(Z)) <= 1e-10 * max(1.0, abs(lz))
        assert np.max(np.abs(r["am_prob"] - am)) <= P64_TOL
        assert np.max(np.abs(r["bm_prob"] - bm)) <= P64_TOL


def _fd_check(engine, t, k_param, grad, precision=64):
    d = np.zeros(19)
    d[k_param] = FD_H
    lp = engine.pf_forward([t], precision=precision, param_delta=d)[0]
    lm = engine.pf_forward([t], precision=precision, param_delta=-d)[0]
    fd = (lp - lm) / (2 * FD_H)
    assert abs(grad - fd) <= GRAD_REL * max(abs(fd), 1e-8), (k_param, grad, fd)


@pytest.mark.gpu
@pytest.mark.parametrize("name", PF_CASES)
def test_pf_gradients_match_finite_differences(engine, name):
    g = GoldenPF(name)
    t = _prepared(g)
    engine.pf_forward([t], precision=64)
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
    engine.pf_forward([t], precision=64)
    r64 = engine.pf_backward()[0]
    engine.pf_forward([t], precision=32)
    r32 = engine.pf_backward()[0]
    for key in ("dlogz_dindel", "dlogz_dindel_opening", "dlogz_dstruct_weight"):
        assert abs(r32[key] - r64[key]) <= GRAD_REL * abs(r64[key]), key
    np.testing.assert_allclose(r32["dlogz_dbasematch"], r64["dlogz_dbasematch"], rtol=GRAD_REL, atol=1e-9)


@pytest.mark.gpu
def test_pf_backward_needs_forward(engine):
    from locarna_gb300.engine import LcgError
    g = GoldenPF(PF_CASES[0])
    engine.pf_forward([g.tables])
    engine.pf_backward()
    with pytest.raises(LcgError):
        engine.pf_backward()
