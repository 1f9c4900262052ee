"""Generate ribosum85_60.inc (the built-in RIBOSUM85_60 tables) from the
reference's data file Data/Matrices/RIBOSUM85_60.

The reference compiles its built-in matrix by printing the parsed values with
the default iostream precision (6 significant digits, src/ribosum2cc.cc and
RibosumFreq::write_CC_matrix, src/LocARNA/ribosum.cc); this script formats the
same values the same way, so the C++ literals denote the same doubles.
The scoring matrices are symmetric and given as lower triangles.

Usage: python gen_ribosum.py path/to/RIBOSUM85_60 > ribosum85_60.inc
(the file lies under Data/Matrices/ of the reference tree)
"""
import sys

if len(sys.argv) != 2:
    raise SystemExit(__doc__)
path = sys.argv[1]
lines = open(path).read().splitlines()


def g6(x):
    return "%.6g" % x


def tri(start, names):
    k = len(names)
    mat = [[0.0] * k for _ in range(k)]
    row = 0
    i = start
    while row < k:
        parts = lines[i].split()
        i += 1
        if not parts or parts[0] != names[row]:
            continue
        vals = [float(v) for v in parts[1:]]
        for c, v in enumerate(vals):
            mat[row][c] = v
            mat[c][row] = v
        row += 1
    return mat, i


def block(header, count):
    i = lines.index(header) + 1
    vals = []
    while len(vals) < count:
        vals += [float(v) for v in lines[i].split()]
        i += 1
    return vals[:count]


bases = ["A", "C", "G", "U"]
pairs = [a + b for a in bases for b in bases]
hdr = next(i for i, l in enumerate(lines) if l.split() == bases)
bm, nxt = tri(hdr + 1, bases)
hdr2 = next(i for i, l in enumerate(lines) if l.split() == pairs)
am, _ = tri(hdr2 + 1, pairs)

out = ["// generated by gen_ribosum.py from the RIBOSUM85_60 data file; do not edit"]


def emit(name, vals):
    out.append(f"static const double {name}[{len(vals)}] = {{")
    for r in range(0, len(vals), 8):
        out.append("    " + ", ".join(g6(v) for v in vals[r:r + 8]) + ",")
    out.append("};")


emit("kBmScore", [v for row in bm for v in row])
emit("kAmScore", [v for row in am for v in row])
emit("kBaseProbs", block("BASE FREQUENCIES", 4))
emit("kBaseNonstructProbs", block("BASE NONSTRUCTURAL FREQUENCIES", 4))
emit("kBasepairProbs", block("BASE PAIR FREQUENCIES", 16))
emit("kBasematchProbs", block("BASE MATCH FREQUENCIES", 16))
emit("kArcmatchProbs", block("BASE PAIR MATCH FREQUENCIES", 256))
print("\n".join(out))
