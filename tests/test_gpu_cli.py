"""The locarna / locarna_p command lines on the GPU against the reference's
own binaries' output for the same inputs and options (tests/golden/cli/,
made by tests/golden/make_cli_golden.py from the reference build).

locarna: stdout and every written file equal the reference's text.
locarna_p: the same lines; the printed numbers (6 significant digits) agree
within one unit of the last printed digit, and the probability files list
the same entries (a value within rounding of the output threshold may sit on
either side of it).
"""
import json
import os
import re
import subprocess
import sys
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI_GOLDEN = os.path.join(ROOT, "tests", "golden", "cli")
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))

CASES = sorted(f[:-len(".args.json")] for f in os.listdir(CLI_GOLDEN) if f.endswith(".args.json"))


def _num_close(a, b):
    x, y = float(a), float(b)
    return abs(x - y) <= 1e-5 * max(abs(x), abs(y)) + 1e-12


def _same_numbers_text(got, ref):
    gl, rl = got.strip().splitlines(), ref.strip().splitlines()
    assert len(gl) == len(rl), (len(gl), len(rl))
    for g, r in zip(gl, rl):
        gt, rt = g.split(), r.split()
        assert len(gt) == len(rt), (g, r)
        for x, y in zip(gt, rt):
            if x != y:
                assert re.match(r"^[-+0-9.e]+$", x) and _num_close(x, y), (g, r)


def _prob_entries(text, nkey):
    out = {}
    for line in text.strip().splitlines():
        t = line.split()
        out[tuple(int(v) for v in t[:nkey])] = float(t[nkey])
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES)
def test_cli_matches_reference_binary(case):
    from locarna_gb300.build import OUT, build_cli
    from make_cli_golden import CASES as SPECS, run_case
    build_cli()
    spec = json.load(open(os.path.join(CLI_GOLDEN, case + ".args.json")))
    prog = spec["program"]
    with tempfile.TemporaryDirectory(prefix="cli_run_") as d:
        got = run_case(os.path.join(OUT, prog), case, SPECS[case], d)
    for kind, text in got.items():
        ref = open(os.path.join(CLI_GOLDEN, f"{case}.{kind}")).read()
        if prog == "locarna":
            assert text == ref, (case, kind)
        elif kind == "stdout":
            _same_numbers_text(text, ref)
        else:
            nkey = 4 if kind.startswith("am") else 2
            g, r = _prob_entries(text, nkey), _prob_entries(ref, nkey)
            args = spec["args"]
            opt = "--min-am-prob" if nkey == 4 else "--min-bm-prob"
            thr = float(args[args.index(opt) + 1]) if opt in args else 0.001
            for k in set(g) | set(r):
                if k in g and k in r:
                    assert _num_close(g[k], r[k]), (case, kind, k, g[k], r[k])
                else:  # only a value at the threshold may fall on either side
                    v = g.get(k, r.get(k))
                    assert abs(v - thr) <= 1e-5 * thr, (case, kind, k, v)
