"""Where the reference's LocARNA-P probabilities leave the marginals of its own
partition function (pf150, pf200): the outside pass reads Mprime entries
outside the band that it never wrote, and they hold the debugging fill value
-1 (aligner_p.icc:921, read through virtual_Mprime in case 5 of
comp_Mprime_entry, :785-797 / :862-878). The oracle restates the pass with
the reference's fill; built with fill 0 instead, its arc-match probabilities
equal the Richardson-extrapolated finite-difference marginals of Z
(tests/golden/*_marginals.npz) at two pf_scale values, and none is negative,
while the reference's fill gives negative, pf_scale-dependent values."""
import ctypes as C
import os
import subprocess
import tempfile

import numpy as np
import pytest

from golden_io import GoldenPF

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _oracle(fill, out):
    so = os.path.join(out, f"libpf_fill{fill}.so")
    subprocess.check_call(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off",
                           f"-DLCG_ORACLE_MPRIME_FILL={fill}", os.path.join(ROOT, "oracle", "pf_oracle.c"),
                           "-o", so, "-lm"])
    lib = C.CDLL(so)
    lib.lcg_oracle_pf.restype = C.c_int
    return lib


def _am_probs(lib, t, pf_scale):
    ct = t.to_c()
    Z = C.c_double()
    am = np.zeros(max(1, t.num_arcmatches))
    bm = np.zeros((t.len_a + 1) * (t.len_b + 1))
    P = C.POINTER(C.c_double)
    rc = lib.lcg_oracle_pf(C.byref(ct), C.c_double(300.0), C.c_double(pf_scale), C.c_double(0.0), 0,
                           C.byref(Z), am.ctypes.data_as(P), bm.ctypes.data_as(P))
    assert rc == 0
    return am[:t.num_arcmatches]


@pytest.mark.parametrize("case", ["pf150", "pf200"])
def test_outside_fill_value_explains_the_reference_probabilities(case):
    g = GoldenPF(case)
    mk = np.load(os.path.join(ROOT, "tests", "golden", case + "_marginals.npz"))
    with tempfile.TemporaryDirectory() as tmp:
        as_ref, fixed = _oracle(-1, tmp), _oracle(0, tmp)
        for s in (1.0, 1.7):
            am = _am_probs(fixed, g.tables, s)
            assert (am >= -1e-12).all()
            assert np.abs(am[mk["am_idx"]] - mk["am_fd"]).max() < 1e-9, s
        ref1, ref2 = _am_probs(as_ref, g.tables, 1.0), _am_probs(as_ref, g.tables, 1.7)
        assert (ref1 < -1e-6).sum() > 100
        assert np.abs(ref1 - ref2).max() > 1e-4  # depends on pf_scale
        # the reference's fill is what the committed reference outputs show
        assert np.abs(ref1[mk["am_idx"]] - mk["am_ref"]).max() < 1e-6
