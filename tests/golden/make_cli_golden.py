"""Golden outputs of the reference's own command lines (test infrastructure).

Runs the reference's locarna and locarna_p (oracle/_ref/, built from the
reference sources by oracle/build_ref.sh) on the PP inputs of golden cases
with the option sets below, and stores what they print and write under
tests/golden/cli/: <case>.stdout, and <case>.<file option> for each output
file (the file names in the arguments are placeholders {out}/<name>).

Usage: python tests/golden/make_cli_golden.py   (needs the reference build)
"""
import json
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, ROOT)

OUT = os.path.join(HERE, "cli")

# case: (program, golden case whose PP inputs are used, arguments)
CASES = {
    "locarna_c150_default": ("locarna", "c150_global", []),
    "locarna_c150_files": ("locarna", "c150_global",
                           ["--width", "70", "--write-structure", "--clustal", "{out}/aln.clustal",
                            "--stockholm", "{out}/aln.sto"]),
    "locarna_c90_seqlocal": ("locarna", "c90_seqlocal_b", ["--sequ-local", "true", "--write-structure"]),
    "locarna_p120_profiles": ("locarna", "p120_global", ["--width", "60", "--clustal", "{out}/aln.clustal"]),
    "locarna_h180_structlocal_nolp": ("locarna", "h180_nolp_sl",
                                      ["--struct-local", "true", "--noLP", "--write-structure"]),
    "locarna_c150_kbest": ("locarna", "c150_kbest", ["--sequ-local", "true", "--kbest", "3"]),
    "locarna_c150_unpaired": ("locarna", "c150_global", ["--unpaired-penalty", "40", "--write-structure"]),
    "locarna_c150_bothstack": ("locarna", "c150_bothstack",
                               ["--stacking", "--new-stacking", "--exp-prob", "0.005", "--write-structure"]),
    "locarna_c150_freeleft": ("locarna", "c150_freeleft", ["--free-endgaps", "+-+-", "--pos-output"]),
    "locarna_c150_maxdiff": ("locarna", "c150_maxdiff", ["--max-diff", "20", "--write-structure"]),
    "locarna_c150_normalized": ("locarna", "c150_global", ["--sequ-local", "true", "--normalized", "100"]),
    "locarna_h180_penalized_sl": ("locarna", "h180_penalized_sl",
                                  ["--sequ-local", "true", "--struct-local", "true", "--penalized", "25"]),
    "locarna_a150_anchors": ("locarna", "a150_anchors", ["--write-structure"]),
    "locarna_c150_params": ("locarna", "c150_global",
                            ["--indel", "-200", "--indel-opening", "-500", "--struct-weight", "150", "--tau", "100",
                             "--width", "100"]),
    "locarna_c120_unpaired_noribo": ("locarna", "c120_opening0",
                                     ["--unpaired-penalty", "10", "--use-ribosum", "false", "--write-structure"]),
    "locarna_p_pf90_default": ("locarna_p", "pf90_b_default",
                               ["--write-arcmatch-probs", "{out}/am.txt", "--write-basematch-probs",
                                "{out}/bm.txt"]),
    "locarna_p_pf80_inclam": ("locarna_p", "pf80_default",
                              ["--min-am-prob", "0.01", "--min-bm-prob", "0.005", "--include-am-in-bm",
                               "--write-arcmatch-probs", "{out}/am.txt", "--write-basematch-probs",
                               "{out}/bm.txt"]),
}


def pp_texts(case):
    import numpy as np
    z = np.load(os.path.join(HERE, case + ".npz"))
    return str(z["pp_a"]), str(z["pp_b"])


def run_case(exe, name, spec, workdir):
    """Run `exe` (a locarna-compatible program) on the case in workdir; returns
    {stdout, <file>: text}."""
    prog, case, args = spec
    pa, pb = pp_texts(case)
    fa, fb = os.path.join(workdir, "A.pp"), os.path.join(workdir, "B.pp")
    with open(fa, "w") as f:
        f.write(pa)
    with open(fb, "w") as f:
        f.write(pb)
    argv = [a.replace("{out}", workdir) for a in args]
    r = subprocess.run([exe] + argv + [fa, fb], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"{name}: {exe} exited {r.returncode}: {r.stderr}")
    out = {"stdout": r.stdout}
    for a in args:
        if a.startswith("{out}/"):
            fn = a[len("{out}/"):]
            with open(os.path.join(workdir, fn)) as f:
                out[fn] = f.read()
    return out


def main():
    os.makedirs(OUT, exist_ok=True)
    names = sys.argv[1:] or list(CASES)
    for name in names:
        prog = CASES[name][0]
        exe = os.path.join(ROOT, "oracle", "_ref", prog)
        with tempfile.TemporaryDirectory(prefix="cli_golden_") as d:
            out = run_case(exe, name, CASES[name], d)
        for k, v in out.items():
            with open(os.path.join(OUT, f"{name}.{k}"), "w") as f:
                f.write(v)
        with open(os.path.join(OUT, f"{name}.args.json"), "w") as f:
            json.dump({"program": prog, "case": CASES[name][1], "args": CASES[name][2]}, f)
        print(name, sorted(out))


if __name__ == "__main__":
    main()
