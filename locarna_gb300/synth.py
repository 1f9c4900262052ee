"""Seeded synthetic RNA inputs in PP 2.0 format.

The reference reads PP 2.0 files (src/LocARNA/rna_data.cc:979-1104): a
clustal-like sequence block ended by ``#END``, then ``#SECTION BASEPAIRS``
with ``i j p`` lines, ended by ``#END``.  Base-pair probability tables
normally come from ViennaRNA folding; here they are synthetic:

* sequence: i.i.d. uniform over ACGU;
* planted stems: nested or disjoint (never crossing), each 4-10 stacked
  canonical/GU pairs whose bases are rewritten to a random canonical pair,
  p ~ U(0.5, 0.99); 3-6 stems per 150 nt (the count scales with length);
* background: every canonical/GU pair with j-i >= 4 is kept with rate
  ``q`` (default 0.05), p ~ Exp(mean 0.02) truncated to <= 0.1 by rejection;
* probabilities are written with 6 decimals and pairs whose written value
  is <= ``min_prob`` (the reference's default --min-prob 0.001,
  src/locarna.cc:183) are dropped, so every reader parses the same value.

Only ``random.Random.random()`` is used, so a seed gives the same file on
every platform.
"""
import math
import random

CANONICAL = {("A", "U"), ("U", "A"), ("C", "G"), ("G", "C"), ("G", "U"), ("U", "G")}
_CANON_LIST = [("A", "U"), ("U", "A"), ("C", "G"), ("G", "C"), ("G", "U"), ("U", "G")]


def _randint(rng, lo, hi):
    """Uniform integer in [lo, hi] from rng.random() only."""
    return lo + min(hi - lo, int(rng.random() * (hi - lo + 1)))


class RnaRecord:
    """One synthetic RNA: name, sequence and sparse base-pair probabilities."""

    def __init__(self, name, seq, pairs, seed=0):
        self.name = name
        self.seq = seq
        self.pairs = pairs  # dict (i, j) -> p, 1-based, i < j
        self.seed = seed

    def stack_probs(self):
        """Joint probabilities p2 of (i,j) and (i+1,j-1) for the pairs whose
        inner pair is listed (the fourth column of a PP base-pair line,
        rna_data.cc:1085-1094): p2 = min(p, p_inner) * U(0.2, 1); one pair in
        ten gets a p2 below the default cutoff (dropped by the reader) and one
        in ten none at all. Drawn from a generator of its own, so the
        sequence and the pairs do not depend on it."""
        rng = random.Random(self.seed * 7919 + 17)
        out = {}
        for (i, j) in sorted(self.pairs):
            pin = self.pairs.get((i + 1, j - 1))
            u = rng.random()
            if pin is None or u < 0.1:
                continue
            if u < 0.2:
                out[(i, j)] = 0.0005
            else:
                out[(i, j)] = round(min(self.pairs[(i, j)], pin) * (0.2 + 0.8 * rng.random()), 6)
        return out

    def to_pp(self, stacking=False, anchors=None):
        """PP 2.0 text; with ``stacking`` the base-pair section carries the
        #STACK keyword and p2 columns (stack_probs); ``anchors`` (a string of
        the sequence's length, '.' for no anchor) becomes an #A1 line."""
        lines = ["#PP 2.0", "", f"{self.name} {self.seq}"]
        if anchors is not None:
            assert len(anchors) == len(self.seq)
            lines.append(f"#A1 {anchors}")
        lines += ["", "#END", "", "#SECTION BASEPAIRS", ""]
        st = self.stack_probs() if stacking else {}
        if stacking:
            lines.append("#STACK")
        for (i, j) in sorted(self.pairs):
            if (i, j) in st:
                lines.append(f"{i} {j} {self.pairs[(i, j)]:.6f} {st[(i, j)]:.6f}")
            else:
                lines.append(f"{i} {j} {self.pairs[(i, j)]:.6f}")
        lines += ["", "#END", ""]
        return "\n".join(lines)


def make_rna(length, seed, name=None, q=0.05, stems=None, min_prob=0.001):
    """Generate one RNA of ``length`` nt from ``seed``."""
    rng = random.Random(seed)
    seq = [("A", "C", "G", "U")[_randint(rng, 0, 3)] for _ in range(length)]
    pairs = {}
    used = [False] * (length + 1)
    planted = []  # list of (i, j) pairs, 1-based
    if stems is None:
        lo = max(1, round(3 * length / 150))
        hi = max(lo, round(6 * length / 150))
        stems = _randint(rng, lo, hi)

    def crosses(i, j):
        for (a, b) in planted:
            if a < i < b < j or i < a < j < b:
                return True
        return False

    for _ in range(stems):
        for _attempt in range(200):
            k = _randint(rng, 4, 10)
            span_min = 2 * k + 2  # hairpin of at least 3 unpaired bases
            if length < span_min + 1:
                break
            i = _randint(rng, 1, length - span_min)
            j = _randint(rng, i + span_min, length)
            ok = True
            for t in range(k):
                a, b = i + t, j - t
                if b - a < 4 or used[a] or used[b] or crosses(a, b):
                    ok = False
                    break
            if not ok:
                continue
            for t in range(k):
                a, b = i + t, j - t
                x, y = _CANON_LIST[_randint(rng, 0, 5)]
                seq[a - 1], seq[b - 1] = x, y
                used[a] = used[b] = True
                planted.append((a, b))
                pairs[(a, b)] = round(0.5 + 0.49 * rng.random(), 6)
            break

    for i in range(1, length + 1):
        for j in range(i + 4, length + 1):
            if (i, j) in pairs or (seq[i - 1], seq[j - 1]) not in CANONICAL:
                continue
            if rng.random() >= q:
                continue
            while True:
                p = -0.02 * math.log(1.0 - rng.random())
                if p <= 0.1:
                    break
            pairs[(i, j)] = round(p, 6)

    pairs = {k: v for k, v in pairs.items() if v > min_prob}
    return RnaRecord(name or f"rna{seed}", "".join(seq), pairs, seed=seed)


def make_homolog(rec, seed, sub_rate=0.1, name=None):
    """A related RNA: ``rec`` with point substitutions (rate ``sub_rate``;
    both bases of a paired position are redrawn as a canonical pair, so the
    structure is kept) and every pair probability scaled by U(0.7, 1.3),
    capped at 0.99. Pairs whose written value drops to <= 0.001 are left out."""
    rng = random.Random(seed)
    seq = list(rec.seq)
    partner = {}
    for (i, j), p in rec.pairs.items():
        if p >= 0.5:
            partner[i], partner[j] = j, i
    for pos in range(1, len(seq) + 1):
        if rng.random() >= sub_rate:
            continue
        if pos in partner:
            a, b = min(pos, partner[pos]), max(pos, partner[pos])
            x, y = _CANON_LIST[_randint(rng, 0, 5)]
            seq[a - 1], seq[b - 1] = x, y
        else:
            seq[pos - 1] = ("A", "C", "G", "U")[_randint(rng, 0, 3)]
    pairs = {}
    for (i, j) in sorted(rec.pairs):
        if (seq[i - 1], seq[j - 1]) not in CANONICAL:
            continue
        p = round(min(0.99, rec.pairs[(i, j)] * (0.7 + 0.6 * rng.random())), 6)
        if p > 0.001:
            pairs[(i, j)] = p
    return RnaRecord(name or f"{rec.name}_h{seed}", "".join(seq), pairs, seed=seed)


class ProfileRecord:
    """A multiple alignment (equal-length rows with '-' gaps) and the base-pair
    probabilities of its columns: the input of progressive alignment."""

    def __init__(self, name, rows, pairs, seed=0):
        self.name = name
        self.rows = rows  # list of (name, aligned row)
        self.pairs = pairs  # dict (i, j) -> p over columns
        self.seed = seed

    def to_pp(self):
        lines = ["#PP 2.0", ""] + [f"{nm} {row}" for nm, row in self.rows] + ["", "#END", "",
                                                                             "#SECTION BASEPAIRS", ""]
        for (i, j) in sorted(self.pairs):
            lines.append(f"{i} {j} {self.pairs[(i, j)]:.6f}")
        lines += ["", "#END", ""]
        return "\n".join(lines)


def make_profile(length, seed, nrows=3, gap_rate=0.08, name=None):
    """A profile of ``nrows`` homologs of one synthetic RNA (make_homolog):
    gaps are placed in each row except the first at unpaired positions (rate
    ``gap_rate``) and in runs; the column pair probabilities are the root's."""
    root = make_rna(length, seed)
    rng = random.Random(seed * 31 + 7)
    paired = set()
    for (i, j), p in root.pairs.items():
        if p >= 0.5:
            paired.update((i, j))
    rows = [(f"{name or 'p' + str(seed)}_0", root.seq)]
    for r in range(1, nrows):
        h = make_homolog(root, seed * 1000 + r, sub_rate=0.1)
        row = list(h.seq)
        pos = 1
        while pos <= length:
            if pos not in paired and rng.random() < gap_rate:
                run = 1 + min(3, int(rng.random() * 4))
                for t in range(pos, min(length, pos + run - 1) + 1):
                    if t not in paired:
                        row[t - 1] = "-"
                pos += run
            else:
                pos += 1
        rows.append((f"{name or 'p' + str(seed)}_{r}", "".join(row)))
    return ProfileRecord(name or f"prof{seed}", rows, dict(root.pairs), seed=seed)


def make_family(count, len_lo, len_hi, seed, q=0.05):
    """``count`` RNAs with lengths uniform in [len_lo, len_hi]."""
    rng = random.Random(seed)
    out = []
    for k in range(count):
        L = _randint(rng, len_lo, len_hi)
        out.append(make_rna(L, seed * 100003 + k, name=f"s{seed}_{k}", q=q))
    return out
