"""Calibration of the CPU port against the reference's own locarna (test
infrastructure; needs oracle/_ref/locarna, built from the reference sources by
oracle/build_ref.sh, and oracle/_build/port_locarna).

bench.py's reference arm times the port (oracle/port_locarna.cc: the host
table preparation + the C restatement of the reference's Aligner) because the
reference's sources, and so its binary, are not available where the bench
runs. This script runs both on the same pairs of the all-pairs workload, one
pair after another on one core, checks that every score is the same, and
prints both rates: the factor by which the port's rate stands in for the
reference's.

Usage: python oracle/calibrate_port.py [pairs]
"""
import os
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)


def main():
    import bench
    npairs = int(sys.argv[1]) if len(sys.argv) > 1 else 32
    ref = os.path.join(HERE, "_ref", "locarna")
    port = os.path.join(HERE, "_build", "port_locarna")
    pp, pairs = bench.workload_pp()
    step = max(1, len(pairs) // npairs)
    sample = pairs[::step][:npairs]
    with tempfile.TemporaryDirectory(prefix="calib_pp_") as d:
        paths = []
        for k, text in enumerate(pp):
            p = os.path.join(d, f"r{k}.pp")
            with open(p, "w") as f:
                f.write(text)
            paths.append(p)
        t0 = time.perf_counter()
        ref_scores = []
        for a, b in sample:
            out = subprocess.run([ref, paths[a], paths[b]], capture_output=True, text=True, check=True).stdout
            ref_scores.append(int(next(l for l in out.splitlines() if l.startswith("Score:")).split()[1]))
        t_ref = time.perf_counter() - t0
        lst = "".join(f"{paths[a]} {paths[b]}\n" for a, b in sample)
        t0 = time.perf_counter()
        out = subprocess.run([port], input=lst, capture_output=True, text=True, check=True).stdout
        t_port = time.perf_counter() - t0
        port_scores = [int(l.split()[0]) for l in out.splitlines()]
    assert port_scores == ref_scores, "the port's scores differ from the reference's"
    print(f"pairs {len(sample)} (every {step}th of the {len(pairs)} workload pairs), one core each")
    print(f"reference locarna (one process per pair): {len(sample) / t_ref:.3f} aligns/s ({t_ref:.1f} s)")
    print(f"port (one process for all pairs):          {len(sample) / t_port:.3f} aligns/s ({t_port:.1f} s)")
    print(f"port / reference rate: {t_ref / t_port:.3f}; scores identical on all {len(sample)} pairs")


if __name__ == "__main__":
    main()
