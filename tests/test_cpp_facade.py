"""The C++ facade (include/locarna_gb300.hpp): compiles against the library
(CPU); run on the GPU, its Aligner / AlignerP reproduce the reference's golden
score and alignment and the partition function."""
import math
import os
import subprocess

import numpy as np
import pytest

from golden_io import Golden, GoldenPF

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _build(tmp_path):
    from locarna_gb300.build import build_engine
    lib = build_engine()
    exe = tmp_path / "facade_demo"
    subprocess.check_call(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "cpp", "facade_demo.cc"), "-o", str(exe),
                           "-L", os.path.dirname(lib), "-llocarna_gb300", "-Wl,-rpath," + os.path.dirname(lib)])
    return exe


def test_facade_compiles_and_reports_failures(tmp_path):
    exe = _build(tmp_path)
    bad = tmp_path / "bad.pp"
    bad.write_text("not a pp file\n")
    r = subprocess.run([str(exe), str(bad), str(bad)], capture_output=True, text=True)
    assert r.returncode == 1 and "failure:" in r.stderr


def _run(exe, tmp_path, pp_a, pp_b, *args):
    a, b = tmp_path / "a.pp", tmp_path / "b.pp"
    a.write_text(pp_a)
    b.write_text(pp_b)
    out = subprocess.run([str(exe), str(a), str(b), *args], capture_output=True, text=True, check=True).stdout
    return dict(line.split(" ", 1) if " " in line else (line, "") for line in out.splitlines())


@pytest.mark.gpu
def test_facade_aligner_matches_engine_and_oracle(tmp_path, engine):
    """Same PP inputs through the facade and through the Python binding (both
    prepare the tables on this host), and against the oracle."""
    from checks import assert_same_result
    from locarna_gb300.prep import prepare_pair
    from oracle_ffi import oracle_align
    exe = _build(tmp_path)
    g = Golden("c150_global")
    res = _run(exe, tmp_path, g.pp_a, g.pp_b)
    t = prepare_pair(g.pp_a, g.pp_b)
    ref = engine.align_pairs([t])[0]
    assert_same_result(ref, oracle_align(t), g.name)
    assert int(res["score"]) == ref.score
    edges = [tuple(int(v) for v in e.split(",")) for e in res["edges"].split()]
    assert edges == [tuple(int(v) for v in e) for e in ref.edges]
    gp = GoldenPF("pf90_b")
    resp = _run(exe, tmp_path, gp.pp_a, gp.pp_b)
    assert abs(float(resp["log_z"]) - math.log(gp.Z)) <= 1e-9 * abs(math.log(gp.Z))
    tp = prepare_pair(gp.pp_a, gp.pp_b, min_trace_probability=1e-5, pf_precision=0)
    engine.pf_forward([tp], precision=64)
    r = engine.pf_backward()[0]
    assert abs(float(resp["sum_am"]) - float(np.sum(r["am_prob"]))) <= 1e-9
    assert abs(float(resp["sum_bm"]) - float(np.sum(r["bm_prob"]))) <= 1e-9
