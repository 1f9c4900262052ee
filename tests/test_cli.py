"""The locarna / locarna_p command lines (CPU part).

* option handling without a GPU: --help, --version, options of the reference
  that this build refuses, malformed values;
* the alignment writer (locarna_gb300/cli/lcg_output.hh) on the reference's
  own alignments (golden edges) prints the reference's CLUSTAL / Stockholm
  text (tests/golden/cli/, from the reference's binaries).
The GPU runs of the binaries against the same outputs are in test_gpu_cli.py.
"""
import json
import os
import subprocess

import pytest

from golden_io import Golden

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI_GOLDEN = os.path.join(ROOT, "tests", "golden", "cli")


@pytest.fixture(scope="module")
def cli():
    from locarna_gb300.build import build_cli
    locarna, locarna_p = build_cli()
    return locarna, locarna_p


def test_help_and_version(cli):
    for exe in cli:
        r = subprocess.run([exe, "--help"], capture_output=True, text=True)
        assert r.returncode == 0 and "Usage:" in r.stdout and "--width" in r.stdout or "--pf-scale" in r.stdout
        r = subprocess.run([exe, "--version"], capture_output=True, text=True)
        assert r.returncode == 0 and "LocARNA" in r.stdout


@pytest.mark.parametrize("args,msg", [
    (["--mea-alignment", "a.pp", "b.pp"], "not supported"),
    (["--pp", "x", "a.pp", "b.pp"], "not supported"),
    (["--indel", "abc", "a.pp", "b.pp"], "expects an integer"),
    (["--struct-local", "maybe", "a.pp", "b.pp"], "expects true or false"),
    (["--no-such-option", "a.pp", "b.pp"], "Unknown option"),
    (["a.pp"], "Two input files"),
    (["--normalized", "10", "--penalized", "5", "a.pp", "b.pp"], "simultaneously"),
    (["--sequ-local", "true", "--free-endgaps", "++--", "a.pp", "b.pp"], "Free endgaps"),
    (["--ribosum-file", "RIBOSUM80_60", "a.pp", "b.pp"], "RIBOSUM85_60"),
])
def test_locarna_refuses_before_any_work(cli, args, msg):
    r = subprocess.run([cli[0]] + args, capture_output=True, text=True)
    assert r.returncode != 0
    assert msg in r.stderr, r.stderr


def test_locarna_accepts_extended_pf(cli):
    """--extended-pf is locarna's default envelope precision (always on in
    src/locarna.cc:384): accepted; the run then fails only on the missing
    input file, not on the option."""
    r = subprocess.run([cli[0], "--extended-pf", "no_such_a.pp", "no_such_b.pp"], capture_output=True, text=True)
    assert "not supported" not in r.stderr and "Unknown option" not in r.stderr, r.stderr


def test_locarna_p_refuses_unsupported(cli):
    r = subprocess.run([cli[1], "--fragment-match-probs", "1 2 3 4", "a.pp", "b.pp"], capture_output=True, text=True)
    assert r.returncode != 0 and "not supported" in r.stderr


@pytest.fixture(scope="module")
def writer():
    from locarna_gb300.build import OUT, _run
    exe = os.path.join(OUT, "cli_output_demo")
    _run(["g++", "-O1", "-std=c++17", os.path.join(ROOT, "tests", "cpp", "cli_output_demo.cc"), "-o", exe])
    return exe


def _write(writer, rows_a, rows_b, edges, width, stockholm, anchors=None):
    inp = f"{len(rows_a)} {len(rows_b)} {width} {int(stockholm)}\n"
    inp += "".join(f"{n} {s}\n" for n, s in rows_a + rows_b)
    inp += f"{len(edges)}\n" + "".join(f"{a} {b}\n" for a, b in edges)
    if anchors is not None:
        for lines in anchors:
            inp += f"{len(lines)}\n" + "".join(x + "\n" for x in lines)
    r = subprocess.run([writer], input=inp, capture_output=True, text=True, check=True)
    return r.stdout


def _rows(pp):
    """(name, sequence) rows of a PP text's sequence section."""
    rows, seen = [], {}
    for line in pp.splitlines():
        if line.startswith("#SECTION"):
            break
        if not line or line.startswith("#") or line[0].isspace():
            continue
        name, _, seq = line.partition(" ")
        if name not in seen:
            seen[name] = len(rows)
            rows.append([name, ""])
        rows[seen[name]][1] += seq.strip()
    return [(n, s.upper().replace("T", "U")) for n, s in rows]


def _anchor_lines(pp):
    """The #A<k> lines of a PP text's sequence section, blocks concatenated."""
    lines = {}
    for line in pp.splitlines():
        if line.startswith("#SECTION"):
            break
        if line.startswith("#A") and line[2:3].isdigit():
            k, s = line[2:].split()
            lines[int(k)] = lines.get(int(k), "") + s
    return [lines[k] for k in sorted(lines)]


@pytest.mark.parametrize("case,fname,width,sto", [
    ("locarna_c150_files", "aln.clustal", 70, False),
    ("locarna_c150_files", "aln.sto", 70, True),
    ("locarna_p120_profiles", "aln.clustal", 60, False),
])
def test_writer_prints_the_reference_text(writer, case, fname, width, sto):
    spec = json.load(open(os.path.join(CLI_GOLDEN, case + ".args.json")))
    g = Golden(spec["case"])
    gap = {-1, -2, -3, -4}
    edges = [(a if a > 0 else -1, b if b > 0 else -1) for a, b in g.edges]
    assert all((a > 0 or a in gap) and (b > 0 or b in gap) for a, b in g.edges)
    text = _write(writer, _rows(g.pp_a), _rows(g.pp_b), edges, width, sto)
    ref = open(os.path.join(CLI_GOLDEN, f"{case}.{fname}")).read()
    if sto:
        body = ref.split("\n\n", 1)[1]  # after the header lines
    else:
        body = ref.split("\n\n", 1)[1]  # after the CLUSTAL W title line
        body = "\n".join(l for l in body.splitlines() if l.strip() and not l.startswith(" " * 18) or
                         l.strip() and not set(l.strip()) <= set("().-")) + "\n"
        text = "\n".join(l for l in text.splitlines() if l.strip()) + "\n"
        body = "\n".join(l for l in body.splitlines() if l.strip()) + "\n"
    assert text.replace("\n\n", "\n") == body.replace("\n\n", "\n")


def test_writer_prints_the_consensus_anchor_lines(writer):
    """The anchor lines of both inputs become one consensus line per name
    character, printed after each block's rows ("#A1"; "#=GC cA1" in
    Stockholm); two columns with the same name drop them."""
    spec = json.load(open(os.path.join(CLI_GOLDEN, "locarna_a150_anchors.args.json")))
    g = Golden(spec["case"])
    edges = [(a if a > 0 else -1, b if b > 0 else -1) for a, b in g.edges]
    anch = (_anchor_lines(g.pp_a), _anchor_lines(g.pp_b))
    assert anch[0] and anch[1]
    text = _write(writer, _rows(g.pp_a), _rows(g.pp_b), edges, 120, False, anch)
    ref = open(os.path.join(CLI_GOLDEN, "locarna_a150_anchors.stdout")).read()
    body = [l for l in ref.splitlines()[2:] if l.strip() and not l.startswith(" " * 18)]
    assert [l for l in text.splitlines() if l.strip()] == body
    assert any(l.startswith("#A1 ") for l in body)
    sto = _write(writer, _rows(g.pp_a), _rows(g.pp_b), edges, 120, True, anch)
    assert [l[:8] for l in sto.splitlines() if l.startswith("#")] == ["#=GC cA1"] * 2
    # a name twice in the consensus: no anchor lines
    a2 = [anch[0][0].replace(".", "A", 1)]
    dup = _write(writer, _rows(g.pp_a), _rows(g.pp_b), edges, 120, False, (a2, anch[1]))
    assert not any(l.startswith("#A") for l in dup.splitlines())

