"""Finite-difference match probabilities of the reference's own partition
function, for the LocARNA-P golden cases (test infrastructure).

The probability that an alignment contains arc match k is T * d log Z /
d score(k), and the probability of the base match (i,j) is T * d log Z /
d sigma(i,j) (Boltzmann weights exp(score / T)). This script evaluates both
with the oracle's log Z (oracle/pf_oracle.c, which equals the reference's Z
bit for bit; see test_pf_oracle_golden.py) by Richardson-extrapolated central
differences on the integer score tables:
    D(h) = T (log Z(s+h) - log Z(s-h)) / (2h),  P = (4 D(1) - D(2)) / 3,
whose truncation error is O(T^-4). Sample per case: every arc match whose
reference probability (AlignerP::compute_arcmatch_probabilities) is negative,
up to 60 more of the arc matches with the largest reference probabilities,
60 seeded random arc matches with reference probability > 1e-4, and 80
seeded random base-match cells of the band.

Usage: python tests/golden/make_pf_marginals.py   (CPU only; a few minutes)
"""
import math
import os
import sys
from multiprocessing import get_context

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

T = 300.0
CASES = ("pf150", "pf200")


def _job(args):
    name, kind, idx = args
    from golden_io import GoldenPF
    from oracle_ffi import oracle_pf
    t = GoldenPF(name).tables
    tab = t.am_score if kind == "am" else t.sigma
    s0 = int(tab[idx])
    lz = {}
    for h in (-2, -1, 1, 2):
        tab[idx] = s0 + h
        lz[h] = math.log(oracle_pf(t, probs=False)[0])
    tab[idx] = s0
    d1 = T * (lz[1] - lz[-1]) / 2.0
    d2 = T * (lz[2] - lz[-2]) / 4.0
    return (4.0 * d1 - d2) / 3.0


def make(name, pool):
    from golden_io import GoldenPF
    from oracle_ffi import oracle_pf
    g = GoldenPF(name)
    t = g.tables
    _, am, bm = oracle_pf(t)
    rng = np.random.default_rng(20261203)
    neg = np.nonzero(am < 0)[0]
    top = np.argsort(-am)[:60]
    rnd = rng.choice(np.nonzero(am > 1e-4)[0], 60, replace=False)
    am_idx = np.unique(np.concatenate([neg, top, rnd])).astype(np.int64)
    n, m = t.len_a, t.len_b
    cells = [(i, j) for i in range(1, n + 1) for j in range(max(1, t.min_col[i]), min(m, t.max_col[i]) + 1)
             if t.min_col[i - 1] <= j - 1 <= t.max_col[i - 1]]
    pick = rng.choice(len(cells), 80, replace=False)
    bm_idx = np.array(sorted(cells[k][0] * (m + 1) + cells[k][1] for k in pick), dtype=np.int64)
    jobs = [(name, "am", int(k)) for k in am_idx] + [(name, "bm", int(q)) for q in bm_idx]
    vals = pool.map(_job, jobs)
    am_fd = np.array(vals[:len(am_idx)])
    bm_fd = np.array(vals[len(am_idx):])
    out = os.path.join(HERE, f"{name}_marginals.npz")
    np.savez_compressed(out, am_idx=am_idx, am_fd=am_fd, am_ref=am[am_idx], bm_idx=bm_idx, bm_fd=bm_fd,
                        bm_ref=bm.reshape(-1)[bm_idx])
    print(name, "arc matches", len(am_idx), "(reference negative:", len(neg), ") base matches", len(bm_idx),
          "max |ref - fd| am %.3g bm %.3g" % (np.max(np.abs(am[am_idx] - am_fd)),
                                            np.max(np.abs(bm.reshape(-1)[bm_idx] - bm_fd))))


if __name__ == "__main__":
    with get_context("fork").Pool(os.cpu_count() or 4) as pool:
        for name in CASES:
            make(name, pool)
