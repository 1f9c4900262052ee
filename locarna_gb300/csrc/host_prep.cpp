// Host-side preparation of the tables the Sankoff engine consumes, restating
// the reference's input and scoring objects for single-sequence PP inputs:
//
//   PP 2.0 reader ............ RnaData::read_pp / read_pp_arc_probabilities
//                              (src/LocARNA/rna_data.cc:979-1104) and the
//                              clustal-like sequence block of
//                              MultipleAlignment::read_clustallike
//                              (multiple_alignment.cc:279-420)
//   arcs ..................... BasePairs::generateBPLists (basepairs.cc:155-205)
//   sigma / gaps / weights ... Scoring (scoring.cc:28-311), arc-match scores
//                              Scoring::arcmatch / riboX_arcmatch_score
//                              (scoring.cc:368-554)
//   band ..................... TraceController (trace_controller.cc:360-597)
//   envelope ................. PFGotoh / PFTraceProbs (edge_probs.icc:7-268)
//                              with StralScore (stral_score.cc:10-100)
//   arc matches .............. ArcMatches ctor + is_valid_arcmatch
//                              (arc_matches.cc:19-48, 130-188)
//
// Floating-point expressions are evaluated in the same order and precision as
// in the reference, so that thresholds (p >= min_prob, envelope >= 1e-4) and
// rounded integer scores come out identical on the same host.
#include <algorithm>
#include <atomic>
#include <cctype>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <string_view>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/locarna_gb300.h"
#include "envelope.hh"

namespace {

#include "ribosum85_60.inc"

struct PrepError {
    lcg_status code;
    std::string msg;
};

[[noreturn]] void perr(lcg_status c, const std::string &m) { throw PrepError{c, m}; }

// ---------------------------------------------------------------- PP reader

struct RnaInput {
    std::string name;
    std::string seq;                  // normalised (upper case, T -> U), 1-based via seq[i-1]; the first row
    // all rows (a multiple alignment: a profile of equal-length rows,
    // MultipleAlignment of the PP sequence section); rows[0] == seq
    std::vector<std::string> rows;
    std::vector<std::string> row_names;  // names of the rows, in order of appearance
    std::map<std::pair<int, int>, double> arc_probs;  // (i,j) -> p, i<j (sparse matrix)
    // joint probabilities of (i,j) and (i+1,j-1) (the p2 column, read only with stacking)
    std::map<std::pair<int, int>, double> arc2_probs;
    std::vector<std::string> anchors;  // the #A<k> lines (k = 1, 2, ...), blocks concatenated
};

// get_nonempty_line (aux.cc:122-145): skip empty lines and lines starting with
// white space; join lines ending in a backslash
bool next_line(std::istream &in, std::string &line) {
    while (std::getline(in, line)) {
        if (!line.empty() && line.back() == '\r') line.pop_back();
        if (!line.empty() && !std::isspace((unsigned char)line[0])) {
            while (!line.empty() && line.back() == '\\') {
                line.pop_back();
                std::string l1;
                if (std::getline(in, l1)) {
                    if (!l1.empty() && l1.back() == '\r') l1.pop_back();
                    line += " " + l1;
                } else {
                    break;
                }
            }
            return true;
        }
    }
    return false;
}

bool has_prefix(const std::string &s, const std::string &p) { return s.compare(0, p.size(), p) == 0; }

RnaInput read_pp(const std::string &text, double p_bpcut, bool stacking) {
    std::istringstream in(text);
    std::string line;
    RnaInput r;
    if (!std::getline(in, line) || !has_prefix(line, "#PP 2")) perr(LCG_ERR_PARSE, "not a PP 2.0 file (header #PP 2.0 missing)");
    // sequence section
    std::vector<std::string> names;
    std::map<std::string, std::string> seqs;
    std::vector<std::string> anchors;
    if (!next_line(in, line)) perr(LCG_ERR_PARSE, "PP file ends before the sequence section");
    do {
        if (line[0] == '#') {
            if (has_prefix(line, "#END")) break;
            if (has_prefix(line, "#A")) {
                std::istringstream a(line.substr(2));
                int idx;
                std::string s;
                a >> idx >> s;
                if (a.fail() || idx < 1) perr(LCG_ERR_PARSE, "invalid anchor line");
                if ((size_t)idx > anchors.size() + 1) perr(LCG_ERR_PARSE, "non-contiguous anchor specification");
                if ((size_t)idx > anchors.size()) anchors.resize(idx);
                anchors[idx - 1] += s;
            }
            // #S / #FS structure annotations and unknown tags are ignored here
        } else {
            std::istringstream ls(line);
            std::string name, s;
            ls >> name;
            if (ls.fail() || name.empty()) perr(LCG_ERR_PARSE, "unexpected line in sequence section");
            ls >> s;
            if (ls.fail()) s = "";
            if (!seqs.count(name)) {
                seqs[name] = "";
                names.push_back(name);
            }
            seqs[name] += s;
        }
    } while (next_line(in, line));
    if (names.empty()) perr(LCG_ERR_PARSE, "PP file without sequence");
    r.anchors = anchors;
    r.name = names[0];
    r.row_names = names;
    // MultipleAlignment::normalize_rna_symbols (multiple_alignment.cc:577-584,
    // aux.cc:65-70) on every row; the rows of an alignment must have equal
    // lengths (MultipleAlignment::is_proper)
    for (auto &nm : names) {
        std::string row = seqs[nm];
        for (auto &c : row) {
            c = (char)std::toupper((unsigned char)c);
            if (c == 'T') c = 'U';
        }
        if (!r.rows.empty() && row.size() != r.rows[0].size())
            perr(LCG_ERR_PARSE, "alignment rows of different lengths in the sequence section");
        r.rows.push_back(row);
    }
    r.seq = r.rows[0];
    if (r.seq.empty()) perr(LCG_ERR_PARSE, "empty sequence");
    // base pair section
    if (!next_line(in, line) || line != "#SECTION BASEPAIRS") perr(LCG_ERR_PARSE, "Expected base pair section header.");
    const size_t len = r.seq.size();
    bool contains_stacking = false;
    while (next_line(in, line)) {
        if (line[0] == '#') {
            if (has_prefix(line, "#END")) break;
            if (has_prefix(line, "#BPCUT")) {
                std::istringstream ls(line);
                std::string dummy;
                double p;
                ls >> dummy >> p;
                if (ls.fail()) perr(LCG_ERR_PARSE, "Cannot parse line \"" + line + "\" in base pairs section.");
                p_bpcut = std::max(p, p_bpcut);
            } else if (has_prefix(line, "#STACK")) {
                contains_stacking = true;
            }
            continue;
        }
        std::istringstream ls(line);
        size_t i, j;
        double p;
        ls >> i >> j >> p;
        if (ls.fail()) perr(LCG_ERR_PARSE, "Cannot parse line \"" + line + "\" in base pairs section.");
        if (!(1 <= i && i < j && j <= len)) perr(LCG_ERR_PARSE, "Invalid indices in PP input line \"" + line + "\".");
        if (p <= p_bpcut) continue;
        r.arc_probs[{(int)i, (int)j}] = p;
        // rna_data.cc:1085-1094: the joint probability of (i,j) and (i+1,j-1)
        double p2;
        if (stacking && (ls >> p2) && p2 > p_bpcut) r.arc2_probs[{(int)i, (int)j}] = p2;
    }
    if (!contains_stacking && !r.arc2_probs.empty())
        perr(LCG_ERR_PARSE, "Stacking probabilties found but stack keyword is missing.");
    return r;
}

// ---------------------------------------------------------------- scoring

int idx_acgu(char c) {
    switch (c) {
    case 'A': return 0;
    case 'C': return 1;
    case 'G': return 2;
    case 'U': return 3;
    default: return -1;
    }
}

long round2score(double d) { return (long)((d < 0) ? (d - 0.5) : (d + 0.5)); }

struct Arc {
    int l, r;
    double p;
};

struct Side {
    RnaInput in;
    int len = 0;
    std::vector<Arc> arcs;        // reference index order
    std::vector<long> weights;    // probToWeight per arc
    // stacking: Scoring::stack_weightsX per arc (scoring.cc:200-237) in the
    // reference's 64-bit arithmetic, and is_stackable_arcX (joint probability > 0)
    std::vector<long> stack_w;
    std::vector<uint8_t> stackable;
    std::vector<double> dsw;      // d weight / d struct_weight per arc, unrounded: 1 - ln p / ln pe
    std::vector<double> p_up, p_down;  // prob_paired_upstream / downstream
    std::vector<int> left_start;  // len+2: arcs with left end l are [left_start[l+1], left_start[l]) (index order)
};

// BasePairs::generateBPLists: i from len-3 down to 1, j ascending from i+3,
// keeping p >= min_prob (the sparse matrix in that order)
void make_arcs(Side &s, double min_prob) {
    s.len = (int)s.in.seq.size();
    for (auto &kv : s.in.arc_probs) {
        const int i = kv.first.first, j = kv.first.second;
        if (i >= 1 && i <= s.len - 3 && j >= i + 3 && j <= s.len && kv.second >= min_prob)
            s.arcs.push_back({i, j, kv.second});
    }
    std::stable_sort(s.arcs.begin(), s.arcs.end(),
                     [](const Arc &x, const Arc &y) { return x.l != y.l ? x.l > y.l : x.r < y.r; });
    // RnaData::prob_paired_upstream / downstream (rna_data.cc:713-732):
    // ascending sums over the sparse probability matrix
    s.p_up.assign(s.len + 1, 0.0);
    s.p_down.assign(s.len + 1, 0.0);
    std::vector<std::vector<std::pair<int, double>>> by_left(s.len + 1), by_right(s.len + 1);
    for (auto &kv : s.in.arc_probs) {
        by_left[kv.first.first].push_back({kv.first.second, kv.second});
        by_right[kv.first.second].push_back({kv.first.first, kv.second});
    }
    for (int i = 1; i <= s.len; ++i) {
        double up = 0.0, down = 0.0;
        for (auto &x : by_left[i]) up += x.second;    // j ascending (map order)
        for (auto &x : by_right[i]) down += x.second; // j ascending
        s.p_up[i] = up;
        s.p_down[i] = down;
    }
}

double basematch_score_corrected(int a, int b) {
    // RibosumFreq::basematch_score_corrected (ribosum.cc:324-331)
    double bi = kBaseNonstructProbs[a], bj = kBaseNonstructProbs[b];
    return log(kBasematchProbs[a * 4 + b] / (bi * bj)) / log(2);
}

long sigma_single(const lcg_prep_opts &o, char ca, char cb) {
    // Scoring::sigma_ for one row in each input (scoring.cc:140-198)
    long score = 0;
    int a = idx_acgu(ca), b = idx_acgu(cb);
    if (o.use_ribosum && a >= 0 && b >= 0) {
        score += round2score(100.0 * basematch_score_corrected(a, b));
    } else if (ca != 'N' && cb != 'N') {
        score += (ca == cb) ? o.match : o.mismatch;
    }
    return round2score((double)(score / (int)(1 * 1)));
}

long riboX_single(char al, char ar, char bl, char br) {
    // Scoring::riboX_arcmatch_score for one row each (scoring.cc:368-438)
    int a1 = idx_acgu(al), a2 = idx_acgu(ar), b1 = idx_acgu(bl), b2 = idx_acgu(br);
    if (al == '-' || ar == '-' || bl == '-' || br == '-') return 0;
    if (a1 < 0 || a2 < 0 || b1 < 0 || b2 < 0) return 0;
    double score = 0;
    score += log(kArcmatchProbs[(a1 * 4 + a2) * 16 + (b1 * 4 + b2)] /
                 (kBasepairProbs[a1 * 4 + a2] * kBasepairProbs[b1 * 4 + b2])) /
             log(2);
    return round2score(100.0 * score / 1);
}

// One row pair's term of Scoring::sigma_ (scoring.cc:155-193): the RIBOSUM
// base-match score for two bases, else match / mismatch unless one is 'N'
long sigma_term(const lcg_prep_opts &o, char ca, char cb) {
    int a = idx_acgu(ca), b = idx_acgu(cb);
    if (o.use_ribosum && a >= 0 && b >= 0) return round2score(100.0 * basematch_score_corrected(a, b));
    if (ca != 'N' && cb != 'N') return (ca == cb) ? o.match : o.mismatch;
    return 0;
}

// Scoring::riboX_arcmatch_score (scoring.cc:368-438) for profiles: the average
// over the row pairs whose four ends are bases
long riboX_profile(const RnaInput &A, int al, int ar, const RnaInput &B, int bl, int br) {
    double score = 0;
    int considered = 0;
    for (const auto &ra : A.rows) {
        for (const auto &rb : B.rows) {
            const char c1 = ra[al - 1], c2 = ra[ar - 1], c3 = rb[bl - 1], c4 = rb[br - 1];
            if (c1 == '-' || c2 == '-' || c3 == '-' || c4 == '-') continue;
            const int a1 = idx_acgu(c1), a2 = idx_acgu(c2), b1 = idx_acgu(c3), b2 = idx_acgu(c4);
            if (a1 < 0 || a2 < 0 || b1 < 0 || b2 < 0) continue;
            considered++;
            score += log(kArcmatchProbs[(a1 * 4 + a2) * 16 + (b1 * 4 + b2)] /
                         (kBasepairProbs[a1 * 4 + a2] * kBasepairProbs[b1 * 4 + b2])) /
                     log(2);
        }
    }
    if (considered == 0) return 0;
    return round2score(100.0 * score / considered);
}

// Scoring::precompute_gapcost (scoring.cc:271-311): the gap cost of a column
// scaled by its fraction of non-gap rows (in float, as the reference)
int32_t column_gapcost(const RnaInput &in, int i, int indel) {
    float gf = 0;
    for (const auto &r : in.rows) gf += (r[i - 1] == '-') ? 1 : 0;
    gf /= (float)in.rows.size();
    return (int32_t)round2score((1 - gf) * indel);
}

long prob_to_weight(double p, double pe, int struct_weight) {
    // Scoring::probToWeight (scoring.cc:250-265)
    return round2score(round(struct_weight * (1 - log(p) / log(pe))));
}

// probToWeight for stack weights, where p may be 0: the weight is then
// -infinity, which the reference converts to its integer score type; both of
// its targets (x86-64 and arm64) give LONG_MIN for that conversion, which is
// what this returns instead of converting -infinity (undefined in C++)
long stack_prob_to_weight(double p, double pe, int struct_weight) {
    const double x = round(struct_weight * (1 - log(p) / log(pe)));
    const double d = x < 0 ? x - 0.5 : x + 0.5;
    if (!(d > -9.2e18)) return LONG_MIN;
    return (long)d;
}

// a + b with 64-bit two's-complement wrap-around, as the reference's sums of
// such weights come out on its targets
long wrap_add(long a, long b) { return (long)((unsigned long)a + (unsigned long)b); }

// ---------------------------------------------------------------- anchors

// AnchorConstraints (anchor_constraints.cc:10-395, strict names unless
// --relaxed-anchors, as the locarna driver constructs it, locarna.cc:553-557):
// the allowed match / deletion / insertion ranges per position and the
// outermost anchors. Positions 1-based.
struct AnchorRanges {
    bool empty = true;
    std::vector<int> match_lo, match_hi, del_lo, del_hi;  // i = 1..lenA (index 0 unused)
    std::vector<int> ins_lo, ins_hi;                      // j = 1..lenB
    int ra_a = 0, ra_b = 0, la_a = 0, la_b = 0;
};

// AnchorConstraints::transform_input (:81-123): the name of every position
// (its characters over all #A lines) for the non-blank positions, names in
// strictly increasing order
std::map<std::string, int> anchor_names(int len, const std::vector<std::string> &rows, bool strict) {
    std::vector<std::string> vec(len);
    for (const auto &x : rows) {
        if ((int)x.size() != len)
            perr(LCG_ERR_PARSE, "Error during parsing of anchor constraints. Anchor specification strings must "
                                "have exactly the same length as the corresponding sequences.");
        for (int i = 0; i < len; ++i) vec[i].push_back(x[i]);
    }
    std::map<std::string, int> tab;
    std::string last;
    for (int i = 1; i <= len; ++i) {
        const std::string &x = vec[i - 1];
        bool dont_care = true;  // only_dont_care (:74-79)
        for (char c : x) dont_care = dont_care && (c == ' ' || c == '.' || c == '-');
        if (dont_care) continue;
        if (strict) {
            if (x <= last)
                perr(LCG_ERR_PARSE, "Error during parsing of constraints. Anchor names not in strict lexicographic "
                                    "order at name \"" + x + "\".");
            last = x;
        } else if (tab.count(x)) {
            perr(LCG_ERR_PARSE, "Error during parsing of constraints. Duplicate constraint name: \"" + x + "\".");
        }
        tab[x] = i;
    }
    return tab;
}

AnchorRanges anchor_ranges(int lenA, const std::vector<std::string> &rowsA, int lenB,
                           const std::vector<std::string> &rowsB, bool strict) {
    AnchorRanges R;
    // the single-string annotations of both inputs, or none (:40-60)
    if (rowsA.empty() || rowsB.empty()) return R;
    if (rowsA.size() != rowsB.size())
        perr(LCG_ERR_PARSE, "Error while setting up consensus anchor constraints. The anchor names in all input "
                            "sequences must have the same length.");
    const auto tabA = anchor_names(lenA, rowsA, strict), tabB = anchor_names(lenB, rowsB, strict);
    // init_anchors (:125-146): partner position, -1 for a name the other lacks
    std::vector<long> anA(lenA + 2, 0), anB(lenB + 2, 0);
    std::vector<std::string> nmA(lenA + 2), nmB(lenB + 2);
    for (const auto &x : tabA) {
        nmA[x.second] = x.first;
        auto it = tabB.find(x.first);
        anA[x.second] = it != tabB.end() ? it->second : -1;
    }
    for (const auto &x : tabB) {
        nmB[x.second] = x.first;
        auto it = tabA.find(x.first);
        anB[x.second] = it != tabA.end() ? it->second : -1;
    }
    anA[lenA + 1] = lenA + 1;
    anB[lenB + 1] = lenB + 1;
    // init_named_tables (:380-395)
    auto named_tables = [](int len, const std::vector<long> &an, std::vector<int> &leq, std::vector<int> &geq) {
        auto named = [&](int i) { return i == 0 || i == len + 1 || an[i] != 0; };
        leq.assign(len + 1, 0);
        for (int i = 1; i <= len; ++i) leq[i] = named(i) ? i : leq[i - 1];
        geq.assign(len + 2, 0);
        geq[len + 1] = len + 1;
        for (int i = len; i > 0; --i) geq[i] = named(i) ? i : geq[i + 1];
    };
    std::vector<int> leqA, geqA, leqB, geqB;
    named_tables(lenA, anA, leqA, geqA);
    named_tables(lenB, anB, leqB, geqB);
    auto anchoredA = [&](int i) { return i == 0 || i == lenA + 1 || anA[i] > 0; };
    auto anchoredB = [&](int j) { return j == 0 || j == lenB + 1 || anB[j] > 0; };
    std::vector<std::pair<long, long>> ar(lenA + 1, {1, lenB}), adr(lenA + 1, {1, lenB}), air(lenB + 1, {1, lenA});
    // relaxed names (:322-357): the match ranges from the anchored positions
    // only; the deletion and insertion ranges keep their initial values
    // (1..lenB, 1..lenA), as in the reference
    if (!strict) {
        long last = 0;
        for (int i = 1; i <= lenA; i++) {
            if (anA[i] > 0) last = anA[i];
            ar[i].first = anA[i] > 0 ? last : last + 1;
        }
        last = lenB + 1;
        for (int i = lenA; i >= 1; i--) {
            if (anA[i] > 0) last = anA[i];
            ar[i].second = anA[i] > 0 ? last : last - 1;
        }
    }
    // match ranges (:186-235)
    long last = 0;
    for (int i = 1; i <= lenA && strict; i++) {
        if (anA[i] > 0) {
            last = anA[i];
            ar[i].first = last;
        } else if (anA[i] == 0) {
            ar[i].first = last + 1;
        } else {
            for (long j = last + 1; j <= lenB && anB[j] <= 0; j++) {
                if (anB[j] == -1) {
                    if (nmB[j] < nmA[i]) last = j;
                    else break;
                }
            }
            ar[i].first = last + 1;
        }
    }
    last = lenB + 1;
    for (int i = lenA; i >= 1 && strict; i--) {
        if (anA[i] > 0) {
            last = anA[i];
            ar[i].second = last;
        } else if (anA[i] == 0) {
            ar[i].second = last - 1;
        } else {
            for (long j = last - 1; j >= 1 && anB[j] <= 0; j--) {
                if (anB[j] == -1) {
                    if (nmB[j] > nmA[i]) last = j;
                    else break;
                }
            }
            ar[i].second = last - 1;
        }
    }
    // deletion and insertion ranges (:237-312)
    nmA[0] = "";
    nmB[0] = "";
    const std::string largest = std::max(nmA[leqA[lenA]], nmB[leqB[lenB]]);
    nmA[lenA + 1] = largest + "X";
    nmB[lenB + 1] = largest + "X";
    for (int i = 1, j1 = 0; i <= lenA && strict; ++i) {
        if (anchoredA(i)) {
            adr[i] = {lenB + 1, 0};
        } else {
            const int i0 = leqA[i], i1 = geqA[i];
            while (nmB[j1] < nmA[i1]) j1 = geqB[j1 + 1];
            int j0 = leqB[j1 - 1];
            while (nmB[j0] > nmA[i0]) j0 = leqB[j0 - 1];
            adr[i] = {j0, j1 - 1};
        }
    }
    for (int j = 1, i1 = 0; j <= lenB && strict; ++j) {
        if (anchoredB(j)) {
            air[j] = {lenA + 1, 0};
        } else {
            const int j0 = leqB[j], j1 = geqB[j];
            while (nmA[i1] < nmB[j1]) i1 = geqA[i1 + 1];
            int i0 = leqA[i1 - 1];
            while (nmA[i0] > nmB[j0]) i0 = leqA[i0 - 1];
            air[j] = {i0, i1 - 1};
        }
    }
    // the ranges clipped to the positions that exist; an empty range as (-1, -2)
    auto clip = [](std::pair<long, long> r, long hi_max, int &lo, int &hi) {
        long a = std::max(r.first, 0L), b = std::min(r.second, hi_max);
        if (a > b) {
            lo = -1;
            hi = -2;
        } else {
            lo = (int)a;
            hi = (int)b;
        }
    };
    R.empty = false;
    R.match_lo.assign(lenA + 1, 0);
    R.match_hi.assign(lenA + 1, 0);
    R.del_lo.assign(lenA + 1, 0);
    R.del_hi.assign(lenA + 1, 0);
    R.ins_lo.assign(lenB + 1, 0);
    R.ins_hi.assign(lenB + 1, 0);
    for (int i = 1; i <= lenA; ++i) {
        clip(ar[i], lenB, R.match_lo[i], R.match_hi[i]);
        clip(adr[i], lenB, R.del_lo[i], R.del_hi[i]);
    }
    for (int j = 1; j <= lenB; ++j) clip(air[j], lenA, R.ins_lo[j], R.ins_hi[j]);
    // rightmost_anchor / leftmost_anchor (anchor_constraints.hh:282-306)
    R.ra_a = R.ra_b = 0;
    for (int i = lenA; i >= 1; --i)
        if (anA[i] > 0) {
            R.ra_a = i;
            R.ra_b = (int)anA[i];
            break;
        }
    R.la_a = lenA + 1;
    R.la_b = lenB + 1;
    for (int i = 0; i <= lenA; ++i)
        if (anA[i] > 0) {
            R.la_a = i;
            R.la_b = (int)anA[i];
            break;
        }
    return R;
}

// ---------------------------------------------------------------- envelope

struct Band {
    std::vector<long> minc, maxc;  // size_t in the reference; all values >= 0
};

// StralScore::sigma (stral_score.cc:29-60) for sequences or profiles; `rev`
// evaluates the reversed object (StralScore::reverse, :78-100), whose
// up/down vectors are swapped and reversed.
struct Stral {
    const Side *A, *B;
    double sw;
    bool rev;
    bool ribosum;
    double match, mismatch;
    double sigma(int i, int j) const {
        int n = A->len, m = B->len;
        int ia = rev ? n + 1 - i : i, jb = rev ? m + 1 - j : j;
        double seq_score = 0;
        int pairs = 0;
        // the average over the row pairs of the two columns whose characters
        // are both in the alphabet (one pair for single sequences)
        for (const auto &ra : A->in.rows) {
            for (const auto &rb : B->in.rows) {
                int a = idx_acgu(ra[ia - 1]), b = idx_acgu(rb[jb - 1]);
                if (a >= 0 && b >= 0) {
                    // sim_mat: ribosum base-match scores, or match/mismatch
                    // (MainHelper::select_basematch_scores, main_helper.icc:281-306)
                    seq_score += ribosum ? kBmScore[a * 4 + b] : (a == b ? match : mismatch);
                    pairs++;
                }
            }
        }
        if (pairs != 0) seq_score /= pairs;
        double dA = rev ? A->p_up[ia] : A->p_down[ia];
        double dB = rev ? B->p_up[jb] : B->p_down[jb];
        double uA = rev ? A->p_down[ia] : A->p_up[ia];
        double uB = rev ? B->p_down[jb] : B->p_up[jb];
        return sw * (sqrt(dA * dB) + sqrt(uA * uB)) + seq_score;
    }
};

template <class T>
struct Mat {
    int rows, cols;
    std::vector<T> v;
    Mat(int r, int c) : rows(r), cols(c), v((size_t)r * c, T(0)) {}
    T &operator()(int i, int j) { return v[(size_t)i * cols + j]; }
    const T &operator()(int i, int j) const { return v[(size_t)i * cols + j]; }
};

// PFGotoh::pf_gotoh (edge_probs.icc:76-162)
template <class T>
void pf_gotoh(Mat<T> &zM, Mat<T> &zA, Mat<T> &zB, const Band &tc, const Stral &score, int fe,
              bool local, double gap_opening, double gap_extension, double temp) {
    const int lenA = zM.rows - 1, lenB = zM.cols - 1;
    double g_open = exp(gap_opening / temp);
    double g_ext = exp(gap_extension / temp);
    auto valid = [&](int i, int j) { return tc.minc[i] <= j && j <= tc.maxc[i]; };
    if (valid(0, 0)) zM(0, 0) = local ? 0 : 1;
    if (lenA > 0 && valid(1, 0)) zA(1, 0) = g_open * g_ext;
    if (lenB > 0 && valid(0, 1)) zB(0, 1) = g_open * g_ext;
    for (int i = 2; i <= lenA; i++) {
        if (tc.minc[i] > 0) break;
        zA(i, 0) = zA(i - 1, 0) * g_ext;
    }
    for (long j = std::max(tc.minc[0], 2L); j <= std::min(tc.maxc[0], (long)lenB); j++) zB(0, j) = zB(0, j - 1) * g_ext;
    if (fe & LCG_FREE_LEFT_2)
        for (int i = 1; i <= lenA; i++) zA(i, 0) += 1;
    if (fe & LCG_FREE_LEFT_1)
        for (int j = 1; j <= lenB; j++) zB(0, j) += 1;
    for (int i = 1; i <= lenA; i++) {
        for (long j = std::max(tc.minc[i], 1L); j <= std::min(tc.maxc[i], (long)lenB); j++) {
            double match_score_ij = score.sigma(i, (int)j);
            double match_ij = exp(match_score_ij / temp);
            zM(i, j) = zM(i - 1, j - 1) * match_ij + zA(i - 1, j - 1) * match_ij + zB(i - 1, j - 1) * match_ij +
                       (local ? match_ij : 0);
            zA(i, j) = zA(i - 1, j) * g_ext + zM(i - 1, j) * g_open * g_ext + zB(i - 1, j) * g_open * g_ext;
            zB(i, j) = zB(i, j - 1) * g_ext + zM(i, j - 1) * g_open * g_ext + zA(i, j - 1) * g_open * g_ext;
        }
    }
}

int reverse_fe(int fe) {
    // FreeEndgaps::reverse (free_endgaps.hh:74-79): swap left/right per sequence
    int r = 0;
    if (fe & LCG_FREE_LEFT_1) r |= LCG_FREE_RIGHT_1;
    if (fe & LCG_FREE_RIGHT_1) r |= LCG_FREE_LEFT_1;
    if (fe & LCG_FREE_LEFT_2) r |= LCG_FREE_RIGHT_2;
    if (fe & LCG_FREE_RIGHT_2) r |= LCG_FREE_LEFT_2;
    return r;
}

template <class I>
void apply_envelope_rows(Band &tc, const I *nmin, const I *nmax);

// PFTraceProbs (edge_probs.icc:212-268) followed by
// TraceController::restrict_by_trace_probabilities (trace_controller.cc:565-597)
template <class T>
bool restrict_by_envelope(Band &tc, const Side &A, const Side &B, const lcg_prep_opts &o) {
    const int n = A.len, m = B.len;
    const double gap_opening = o.indel_opening / 100.0, gap_ext = o.indel / 100.0;
    const double sw = o.struct_weight / 100.0, temp = o.temperature_alipf / 100.0;
    const bool local = o.sequ_local != 0;
    const int fe = o.free_endgaps & 15;
    Mat<T> zM(n + 1, m + 1), zA(n + 1, m + 1), zB(n + 1, m + 1);
    Mat<T> zMr(n + 1, m + 1), zAr(n + 1, m + 1), zBr(n + 1, m + 1);
    Stral fwd{&A, &B, sw, false, o.use_ribosum != 0, (double)o.match, (double)o.mismatch};
    Stral rev{&A, &B, sw, true, o.use_ribosum != 0, (double)o.match, (double)o.mismatch};
    pf_gotoh(zM, zA, zB, tc, fwd, fe, local, gap_opening, gap_ext, temp);
    // TraceRange::reverse (trace_controller.cc:319-338)
    Band rtc;
    rtc.minc.resize(n + 1);
    rtc.maxc.resize(n + 1);
    for (int i = 0; i <= n; ++i) {
        rtc.maxc[n - i] = m - tc.minc[i];
        rtc.minc[n - i] = m - tc.maxc[i];
    }
    pf_gotoh(zMr, zAr, zBr, rtc, rev, reverse_fe(fe), local, gap_opening, gap_ext, temp);
    T z;
    if (local) {
        z = 1;
        for (int i = 0; i <= n; i++)
            for (int j = 0; j <= m; j++) z += zM(i, j);
    } else {
        z = zM(n, m) + zA(n, m) + zB(n, m);
        if (fe & LCG_FREE_LEFT_2)
            for (int i = 0; i <= n; i++) z += zA(i, m);
        if (fe & LCG_FREE_LEFT_1)
            for (int j = 0; j <= m; j++) z += zB(n, j);
    }
    bool failed = z == (T)0 || std::isnan((long double)z) || std::isinf((long double)z);
    double locality_add = local ? 1 : 0;
    double g_open = exp(gap_opening / temp);
    Mat<double> probs(n + 1, m + 1);
    for (int i = 0; i <= n; i++) {
        for (long j = std::max(tc.minc[i], 0L); j <= std::min(tc.maxc[i], (long)m); j++) {
            T z_ij = zM(i, j) * (zMr(n - i, m - j) + zAr(n - i, m - j) + zBr(n - i, m - j) + locality_add) +
                     zA(i, j) * (zMr(n - i, m - j) + zAr(n - i, m - j) / g_open + zBr(n - i, m - j)) +
                     zB(i, j) * (zMr(n - i, m - j) + zAr(n - i, m - j) + zBr(n - i, m - j) / g_open);
            probs(i, j) = z_ij / z;
        }
    }
    const double min_prob = o.min_trace_probability;
    std::vector<long> nmin(n + 1), nmax(n + 1);
    for (int i = 0; i <= n; ++i) {
        long new_min = tc.maxc[i], new_max = tc.minc[i];
        for (long j = tc.minc[i]; j <= tc.maxc[i]; ++j) {
            if (probs(i, j) >= min_prob) {
                new_min = std::min(new_min, j);
                new_max = std::max(new_max, j);
            }
        }
        nmin[i] = new_min;
        nmax[i] = new_max;
    }
    apply_envelope_rows(tc, nmin.data(), nmax.data());
    return !failed;
}

// the band update of TraceController::restrict_by_trace_probabilities
// (trace_controller.cc:576-597) from each row's first and last kept column
template <class I>
void apply_envelope_rows(Band &tc, const I *nmin, const I *nmax) {
    const int n = (int)tc.minc.size() - 1;
    for (int i = 0; i <= n; ++i) {
        tc.minc[i] = std::max(tc.minc[i], (long)nmin[i]);
        tc.maxc[i] = std::min(tc.maxc[i], (long)nmax[i]);
    }
    long mx = 0;
    for (int i = 0; i <= n; ++i) {
        tc.maxc[i] = std::max(tc.maxc[i], mx);
        mx = tc.maxc[i];
    }
    long mn = tc.maxc[n];
    for (int i = n + 1; i > 0;) {
        --i;
        tc.minc[i] = std::min(tc.minc[i], mn);
        mn = tc.minc[i];
    }
}

// TraceController::constrain_wo_ref (trace_controller.cc:360-390)
void constrain_wo_ref(Band &tc, size_t lenA, size_t lenB, size_t delta) {
    if (lenA == 0 || lenB == 0) return;
    for (size_t i = 0; i <= lenA; i++) {
        size_t x = i * lenB * (lenA + lenB);
        size_t y = 2 * delta * lenA * lenB;
        size_t z = lenA * (lenA + lenB);
        if (lenA > lenB) y = std::max(y, (lenA + lenB) * lenA / 2);
        else if (lenB > lenA) y = std::max(y, (lenA + lenB) * lenB / 2);
        tc.minc[i] = x > y ? (long)((x - y + z - 1) / z) : 0;
        tc.maxc[i] = (long)std::min((x + y) / z, lenB);
    }
}

}  // namespace

// ---------------------------------------------------------------- prepared pair

struct lcg_prepared_s {
    int n = 0, m = 0;
    std::string seq_a, seq_b, name_a, name_b;
    std::vector<std::string> rows_a, rows_b, row_names_a, row_names_b;  // all rows of profile inputs
    std::vector<std::string> anchor_rows_a, anchor_rows_b;              // the #A<k> lines of the inputs
    std::vector<int32_t> sigma, gap_a, gap_b, arcs_a, arcs_b, am_arcs, am_score, min_col, max_col;
    std::vector<double> arc_p_a, arc_p_b;
    std::vector<int8_t> code_a, code_b;  // 0..3 for A,C,G,U, -1 otherwise; index 1..len
    std::vector<double> am_dsw;          // d am_score / d struct_weight, unrounded
    std::vector<int32_t> am_stack_score; // stacking: Scoring::arcmatch(am, true) (LCG_STACK_NONE: out of range)
    std::vector<uint8_t> am_stackable;   // stacking: Scoring::is_stackable_am
    int32_t indel_opening = 0, exclusion = 0;
    int envelope_ok = 1;
    bool stacking = false;
    AnchorRanges anchors;  // empty unless both inputs carry #A lines
};

extern "C" {

void lcg_prep_opts_default(lcg_prep_opts *o) {
    std::memset(o, 0, sizeof *o);
    o->min_prob = 0.001;
    o->indel = -150;
    o->indel_opening = -750;
    o->struct_weight = 200;
    o->tau = 50;
    o->exclusion = 0;
    o->match = 50;
    o->mismatch = 0;
    o->use_ribosum = 1;
    o->min_trace_probability = 1e-4;
    o->max_diff = -1;
    o->max_diff_am = -1;
    o->max_diff_at_am = -1;
    o->temperature_alipf = 300;
    o->sequ_local = 0;
    o->free_endgaps = 0;
    o->pf_precision = 1;
    o->exp_prob = -1.0;
}

lcg_status lcg_prepare_pair(const char *pp_a, const char *pp_b, const lcg_prep_opts *opts,
                            lcg_prepared *out);
lcg_status lcg_prepared_tables(lcg_prepared p, lcg_pair_tables *t);
const char *lcg_prepared_sequence(lcg_prepared p, int32_t which);
lcg_status lcg_prepared_free(lcg_prepared p);
int32_t lcg_prepared_envelope_ok(lcg_prepared p);

}  // extern "C"

namespace lcg_host {
void set_error(const std::string &msg);
}

namespace {

// One pair between the stages of the preparation: inputs read, band before
// the envelope, then the tables.
struct Staged {
    lcg_prep_opts o;
    std::shared_ptr<const Side> pa, pb;  // shared by the pairs of a batch that use the same input
    Band tc;
    std::unique_ptr<lcg_prepared_s> P;
    lcg_status code = LCG_OK;
    std::string err;
};

// One input: PP reading, arcs (basepairs.cc:155-205), pairing probabilities,
// arc weights Scoring::probToWeight (scoring.cc:250-265) with
// pe = prob_exp_f(len) (aux.hh:216-220), and the arcs by left end.
std::shared_ptr<const Side> make_side(const char *pp, const lcg_prep_opts &o) {
    auto s = std::make_shared<Side>();
    // locarna turns the (old) stacking off unless --exp-prob is given
    // (src/locarna.cc:407-414); the PP reader reads the joint probabilities
    // when either stacking is on (locarna.cc:462)
    const bool old_stacking = o.stacking && o.exp_prob > 0;
    const bool stacking = old_stacking || o.new_stacking;
    s->in = read_pp(pp, o.min_prob, stacking);
    make_arcs(*s, o.min_prob);
    const double pe = o.exp_prob > 0 ? o.exp_prob : 1.0 / (2.0 * s->len);
    for (auto &a : s->arcs) {
        s->weights.push_back(prob_to_weight(a.p, pe, o.struct_weight));
        s->dsw.push_back(1 - log(a.p) / log(pe));
    }
    if (stacking) {
        // Scoring::precompute_weights (scoring.cc:200-237)
        auto prob = [](const std::map<std::pair<int, int>, double> &mp, int i, int j) {
            auto it = mp.find({i, j});
            return it == mp.end() ? 0.0 : it->second;
        };
        for (size_t k = 0; k < s->arcs.size(); ++k) {
            const Arc &a = s->arcs[k];
            const double p_in = prob(s->in.arc_probs, a.l + 1, a.r - 1);
            const double joint = prob(s->in.arc2_probs, a.l, a.r);
            long w = 0;
            if (old_stacking && p_in > 0) w = stack_prob_to_weight(joint / p_in, pe, o.struct_weight);
            if (o.new_stacking) {
                if (!old_stacking) w = s->weights[k];
                if (p_in > 0) w = wrap_add(w, stack_prob_to_weight(joint, pe, o.struct_weight));
            }
            s->stack_w.push_back(w);
            s->stackable.push_back(joint > 0 ? 1 : 0);
        }
    }
    // arcs are ordered by left end descending: [left_start[l+1], left_start[l])
    s->left_start.assign(s->len + 2, 0);
    size_t k = s->arcs.size();
    for (int l = 0; l <= s->len + 1; ++l) {
        while (k > 0 && s->arcs[k - 1].l < l) --k;
        s->left_start[l] = (int)k;
    }
    return s;
}

// the pair's record and the max-diff band (locarna.cc:398-560)
void stage_inputs(std::shared_ptr<const Side> A, std::shared_ptr<const Side> B, Staged &S) {
    const lcg_prep_opts &o = S.o;
    S.P = std::make_unique<lcg_prepared_s>();
    S.pa = std::move(A);
    S.pb = std::move(B);
    const Side &sa = *S.pa, &sb = *S.pb;
    const int n = sa.len, m = sb.len;
    lcg_prepared_s *P = S.P.get();
    P->n = n;
    P->m = m;
    P->seq_a = sa.in.seq;
    P->seq_b = sb.in.seq;
    P->name_a = sa.in.name;
    P->name_b = sb.in.name;
    P->rows_a = sa.in.rows;
    P->rows_b = sb.in.rows;
    P->row_names_a = sa.in.row_names;
    P->row_names_b = sb.in.row_names;
    P->anchor_rows_a = sa.in.anchors;
    P->anchor_rows_b = sb.in.anchors;
    // trace controller (no reference alignment, no anchors)
    S.tc.minc.assign(n + 1, 0);
    S.tc.maxc.assign(n + 1, m);
    if (o.max_diff >= 0) constrain_wo_ref(S.tc, n, m, (size_t)o.max_diff);
    // anchor constraints (strict names) and TraceController::restrict_by_anchors
    // (trace_controller.cc:542-563)
    P->anchors = anchor_ranges(n, sa.in.anchors, m, sb.in.anchors, !o.relaxed_anchors);
    const AnchorRanges &R = P->anchors;
    if (!R.empty) {
        for (int i = 1; i <= n; ++i) {
            long cmin = S.tc.maxc[i], cmax = S.tc.minc[i];
            for (long j = S.tc.minc[i]; j <= S.tc.maxc[i]; ++j) {
                const bool ok = (R.match_lo[i] <= j && j <= R.match_hi[i]) ||
                                (j > 0 && R.ins_lo[j] <= i && i <= R.ins_hi[j]) ||
                                (R.del_lo[i] <= j && j <= R.del_hi[i]);
                if (ok) {
                    cmin = std::min(cmin, j);
                    cmax = std::max(cmax, j);
                }
            }
            S.tc.minc[i] = std::max(S.tc.minc[i], cmin);
            S.tc.maxc[i] = std::min(S.tc.maxc[i], cmax);
        }
    }
}

// the envelope in the reference's precision (edge_probs.icc, trace_controller.cc:565-597)
void stage_envelope_host(Staged &S) {
    bool ok;
    if (S.o.pf_precision == 0) ok = restrict_by_envelope<double>(S.tc, *S.pa, *S.pb, S.o);
    else ok = restrict_by_envelope<long double>(S.tc, *S.pa, *S.pb, S.o);
    S.P->envelope_ok = ok ? 1 : 0;
}

// scoring tables and arc matches on the final band (locarna.cc:560-703)
void stage_tables(Staged &S) {
    const lcg_prep_opts &o = S.o;
    const Side &A = *S.pa, &B = *S.pb;
    const Band &tc = S.tc;
    lcg_prepared_s *P = S.P.get();
    const int n = A.len, m = B.len;
    P->stacking = (o.stacking && o.exp_prob > 0) || o.new_stacking;
    // scoring tables
    P->sigma.assign((size_t)(n + 1) * (m + 1), 0);
    const bool profiles = A.in.rows.size() > 1 || B.in.rows.size() > 1;
    long tab[256][256];
    bool have[256][256];
    std::memset(have, 0, sizeof have);
    if (profiles) {
        // Scoring::sigma_ (scoring.cc:140-198): the sum over the row pairs of
        // the two columns, divided (in integers) by their number; summed per
        // column by the counts of its distinct characters
        auto hist = [](const RnaInput &in, int len) {
            std::vector<std::vector<std::pair<unsigned char, long>>> h(len + 1);
            for (int i = 1; i <= len; ++i) {
                for (const auto &r : in.rows) {
                    const unsigned char c = (unsigned char)r[i - 1];
                    bool found = false;
                    for (auto &x : h[i])
                        if (x.first == c) {
                            x.second++;
                            found = true;
                        }
                    if (!found) h[i].push_back({c, 1});
                }
            }
            return h;
        };
        const auto hA = hist(A.in, n), hB = hist(B.in, m);
        const long npairs_rows = (long)(A.in.rows.size() * B.in.rows.size());
        for (int i = 1; i <= n; ++i) {
            for (int j = 1; j <= m; ++j) {
                long score = 0;
                for (const auto &x : hA[i]) {
                    for (const auto &y : hB[j]) {
                        if (!have[x.first][y.first]) {
                            tab[x.first][y.first] = sigma_term(o, (char)x.first, (char)y.first);
                            have[x.first][y.first] = true;
                        }
                        score += x.second * y.second * tab[x.first][y.first];
                    }
                }
                P->sigma[(size_t)i * (m + 1) + j] = (int32_t)round2score((double)(score / (int)npairs_rows));
            }
        }
    }
    for (int i = 1; i <= n && !profiles; ++i) {
        unsigned char ca = (unsigned char)A.in.seq[i - 1];
        for (int j = 1; j <= m; ++j) {
            unsigned char cb = (unsigned char)B.in.seq[j - 1];
            if (!have[ca][cb]) {
                tab[ca][cb] = sigma_single(o, (char)ca, (char)cb);
                have[ca][cb] = true;
            }
            P->sigma[(size_t)i * (m + 1) + j] = (int32_t)tab[ca][cb];
        }
    }
    // Scoring::precompute_gapcost (scoring.cc:271-311) for gap-free rows
    P->gap_a.assign(n + 1, 0);
    P->gap_b.assign(m + 1, 0);
    for (int i = 1; i <= n; ++i) P->gap_a[i] = column_gapcost(A.in, i, o.indel);
    for (int j = 1; j <= m; ++j) P->gap_b[j] = column_gapcost(B.in, j, o.indel);
    P->indel_opening = o.indel_opening;
    P->exclusion = o.exclusion;
    // Scoring::apply_unpaired_penalty (scoring.cc:65-74): done when the
    // Scoring is constructed, so the arc-match scores below (which read σ
    // without RIBOSUM) see the penalised table
    if (o.unpaired_penalty != 0) {
        const int32_t up = o.unpaired_penalty;
        for (auto &v : P->sigma) v -= 2 * up;
        for (auto &v : P->gap_a) v -= up;
        for (auto &v : P->gap_b) v -= up;
    }

    // arc matches (arc_matches.cc:130-188), A index outer, B index inner;
    // for arc a only the B arcs whose left end b.l passes
    // is_valid_match(a.l, b.l) are visited (by left end descending = B index
    // ascending)
    const size_t mdam = o.max_diff_am != -1 ? (size_t)o.max_diff_am : (size_t)std::max(n, m);
    const size_t mdaam = o.max_diff_at_am != -1 ? (size_t)o.max_diff_at_am : (size_t)std::max(n, m);
    auto valid = [&](long i, long j) { return i >= 0 && i <= n && tc.minc[i] <= j && j <= tc.maxc[i]; };
    auto valid_match = [&](long i, long j) { return valid(i, j) && valid(i - 1, j - 1); };
    long ribo_cache[4][4][4][4];
    bool ribo_have[4][4][4][4];
    std::memset(ribo_have, 0, sizeof ribo_have);
    for (size_t ia = 0; ia < A.arcs.size(); ++ia) {
        const Arc &a = A.arcs[ia];
        const long llo = std::max({tc.minc[a.l], tc.minc[a.l - 1] + 1, 1L});
        const long lhi = std::min({tc.maxc[a.l], tc.maxc[a.l - 1] + 1, (long)m});
        const size_t ib0 = lhi >= llo ? (size_t)B.left_start[lhi + 1] : 0;
        const size_t ib1 = lhi >= llo ? (size_t)B.left_start[llo] : 0;
        for (size_t ib = ib0; ib < ib1; ++ib) {
            const Arc &b = B.arcs[ib];
            const AnchorRanges &R = P->anchors;
            bool ok = valid_match(a.l, b.l) && valid_match(a.r, b.r) &&
                      (R.empty || (R.match_lo[a.l] <= b.l && b.l <= R.match_hi[a.l] && R.match_lo[a.r] <= b.r &&
                                   b.r <= R.match_hi[a.r])) &&
                      (size_t)std::abs((a.r - a.l) - (b.r - b.l)) <= mdam &&
                      (size_t)a.l <= b.l + mdaam && (size_t)b.l <= a.l + mdaam &&
                      (size_t)a.r <= b.r + mdaam && (size_t)b.r <= a.r + mdaam;
            if (!ok) continue;
            long seqc = 0;
            if (o.tau != 0) {
                if (o.use_ribosum && profiles) {
                    seqc = riboX_profile(A.in, a.l, a.r, B.in, b.l, b.r);
                } else if (o.use_ribosum) {
                    char c1 = A.in.seq[a.l - 1], c2 = A.in.seq[a.r - 1];
                    char c3 = B.in.seq[b.l - 1], c4 = B.in.seq[b.r - 1];
                    int x1 = idx_acgu(c1), x2 = idx_acgu(c2), x3 = idx_acgu(c3), x4 = idx_acgu(c4);
                    if (x1 >= 0 && x2 >= 0 && x3 >= 0 && x4 >= 0) {
                        if (!ribo_have[x1][x2][x3][x4]) {
                            ribo_cache[x1][x2][x3][x4] = riboX_single(c1, c2, c3, c4);
                            ribo_have[x1][x2][x3][x4] = true;
                        }
                        seqc = ribo_cache[x1][x2][x3][x4];
                    } else {
                        seqc = riboX_single(c1, c2, c3, c4);
                    }
                } else {
                    seqc = P->sigma[(size_t)a.l * (m + 1) + b.l] + P->sigma[(size_t)a.r * (m + 1) + b.r];
                }
            }
            long s = ((long)o.tau * seqc) / 100 + (A.weights[ia] + B.weights[ib]);
            P->am_arcs.push_back((int32_t)ia);
            P->am_arcs.push_back((int32_t)ib);
            P->am_score.push_back((int32_t)s);
            P->am_dsw.push_back(A.dsw[ia] + B.dsw[ib]);
            if (!A.stack_w.empty()) {
                // Scoring::arcmatch(am, true) (scoring.cc:440-480) in the
                // reference's 64-bit arithmetic; values that leave the int32
                // tables' range only arise from undefined (zero-probability)
                // stack weights and never explain an alignment
                const long st = wrap_add(((long)o.tau * seqc) / 100, wrap_add(A.stack_w[ia], B.stack_w[ib]));
                P->am_stack_score.push_back(st > -(1L << 29) && st < (1L << 29) ? (int32_t)st : LCG_STACK_NONE);
                P->am_stackable.push_back(A.stackable[ia] && B.stackable[ib]);
            }
        }
    }
    for (auto &a : A.arcs) {
        P->arcs_a.push_back(a.l);
        P->arcs_a.push_back(a.r);
        P->arc_p_a.push_back(a.p);
    }
    for (auto &b : B.arcs) {
        P->arcs_b.push_back(b.l);
        P->arcs_b.push_back(b.r);
        P->arc_p_b.push_back(b.p);
    }
    P->code_a.assign(n + 1, -1);
    P->code_b.assign(m + 1, -1);
    // base codes for the base-match gradients of LocARNA-P: single sequences
    // only (a profile column is no single base)
    for (int i = 1; i <= n && A.in.rows.size() == 1; ++i) P->code_a[i] = (int8_t)idx_acgu(A.in.seq[i - 1]);
    for (int j = 1; j <= m && B.in.rows.size() == 1; ++j) P->code_b[j] = (int8_t)idx_acgu(B.in.seq[j - 1]);
    P->min_col.resize(n + 1);
    P->max_col.resize(n + 1);
    for (int i = 0; i <= n; ++i) {
        P->min_col[i] = (int32_t)tc.minc[i];
        P->max_col[i] = (int32_t)tc.maxc[i];
    }
}

}  // namespace

lcg_status lcg_prepare_pair(const char *pp_a, const char *pp_b, const lcg_prep_opts *opts,
                            lcg_prepared *out) {
    if (!pp_a || !pp_b || !out) {
        lcg_host::set_error("NULL argument");
        return LCG_ERR_ARG;
    }
    *out = nullptr;
    Staged S;
    if (opts) S.o = *opts;
    else lcg_prep_opts_default(&S.o);
    try {
        stage_inputs(make_side(pp_a, S.o), make_side(pp_b, S.o), S);
        if (S.o.min_trace_probability > 0.0) stage_envelope_host(S);
        stage_tables(S);
        *out = S.P.release();
        return LCG_OK;
    } catch (const PrepError &e) {
        lcg_host::set_error(e.msg);
        return e.code;
    } catch (const std::exception &e) {
        lcg_host::set_error(e.what());
        return LCG_ERR_NOMEM;
    }
}

namespace {

// fn(q) for q in [0, n) on the host's threads
template <typename F>
void host_parallel(int n, F &&fn) {
    if (n <= 0) return;
    std::atomic<int> next(0);
    const int nth = (int)std::min<unsigned>(std::max(1u, std::thread::hardware_concurrency()), (unsigned)std::min(n, 64));
    auto work = [&]() {
        for (int q; (q = next.fetch_add(1)) < n;) fn(q);
    };
    std::vector<std::thread> th;
    for (int t = 1; t < nth; ++t) th.emplace_back(work);
    work();
    for (auto &t : th) t.join();
}

template <typename F>
void guarded(Staged &S, F &&fn) {
    if (S.code != LCG_OK) return;
    try {
        fn();
    } catch (const PrepError &e) {
        S.code = e.code;
        S.err = e.msg;
    } catch (const std::exception &e) {
        S.code = LCG_ERR_NOMEM;
        S.err = e.what();
    }
}

}  // namespace

namespace lcg_host {

// A batch of pairs between the two stages of lcg_prepare_pairs: inputs read,
// bands and envelopes done for every pair (stage_batch); the tables built for
// a range of pairs at a time (finish_tables), so that a caller can build the
// tables of one chunk while the device aligns the previous one. With
// first < npairs, stage_batch finishes the GPU envelopes of pairs [0, first)
// only and leaves those of the other pairs enqueued on the engine's stream
// (they run while the host builds the first pairs' tables); the first
// finish_tables past `first` waits for them.
struct EnvBuf {
    std::vector<int8_t> ca, cb;
    std::vector<double> sdA, suA, sdB, suB;
    std::vector<int32_t> minc, maxc, nmin, nmax;
};
struct StagedBatch {
    std::vector<Staged> st;
    lcg_engine eng = nullptr;
    std::vector<EnvBuf> buf;               // per pair
    std::vector<lcg_env::PairIn> in;       // per GPU pair
    std::vector<lcg_env::PairOut> res;     // per GPU pair
    std::vector<int> kof;                  // per pair: its GPU index, or -1 (host envelope)
    int first = 0;                         // pairs whose envelopes stage_batch finished
    lcg_env::Pending *pending = nullptr;   // the GPU envelopes of the other pairs
    int host_envelopes = 0;
    ~StagedBatch() {
        std::string err;
        if (pending) lcg_env::compute_end(eng, pending, err);  // nothing of a batch stays in flight
    }
};

// the envelope of pairs [q0, q1): the GPU result, or the host path for the
// pairs the kernel does not take or flagged
static void apply_envelopes(StagedBatch &B, int q0, int q1) {
    std::atomic<int> host{0};
    host_parallel(q1 - q0, [&](int k) {
        const int q = q0 + k;
        guarded(B.st[q], [&]() {
            const int g = B.kof[q];
            if (g >= 0 && B.res[g].flag == 0) {
                apply_envelope_rows(B.st[q].tc, B.buf[q].nmin.data(), B.buf[q].nmax.data());
                B.st[q].P->envelope_ok = 1;
            } else {
                ++host;
                stage_envelope_host(B.st[q]);
            }
        });
    });
    B.host_envelopes += host.load();
}

// the pending GPU envelopes (pairs [first, npairs)), once
static lcg_status finish_envelopes(StagedBatch &B) {
    if (B.first >= (int)B.st.size()) return LCG_OK;
    std::string err;
    lcg_env::Pending *p = B.pending;
    B.pending = nullptr;
    lcg_status rc = lcg_env::compute_end(B.eng, p, err);
    if (rc != LCG_OK) {
        lcg_host::set_error(err);
        return rc;
    }
    apply_envelopes(B, B.first, (int)B.st.size());
    B.first = (int)B.st.size();
    return LCG_OK;
}

lcg_status stage_batch(lcg_engine eng, const char *const *pp_a, const char *const *pp_b, int32_t npairs,
                       const lcg_prep_opts *opts, StagedBatch **out, int32_t *host_envelopes, int32_t first) {
    if (!eng || !pp_a || !pp_b || !out || npairs < 0) {
        lcg_host::set_error("NULL argument");
        return LCG_ERR_ARG;
    }
    *out = nullptr;
    if (host_envelopes) *host_envelopes = 0;
    lcg_env::reset_transfer(eng);
    auto B = std::make_unique<StagedBatch>();
    B->eng = eng;
    B->first = npairs;
    if (npairs == 0) {
        *out = B.release();
        return LCG_OK;
    }
    lcg_prep_opts o;
    if (opts) o = *opts;
    else lcg_prep_opts_default(&o);
    std::vector<Staged> &st = B->st;
    st.resize(npairs);
    for (auto &S : st) S.o = o;
    for (int q = 0; q < npairs; ++q)
        if (!pp_a[q] || !pp_b[q]) {
            lcg_host::set_error("pair " + std::to_string(q) + ": NULL PP text");
            return LCG_ERR_ARG;
        }
    // every distinct input is read once (all-pairs batches repeat each input)
    std::unordered_map<std::string_view, int> text_id;
    std::vector<const char *> texts;
    std::vector<int> ida(npairs), idb(npairs);
    for (int q = 0; q < npairs; ++q)
        for (int w = 0; w < 2; ++w) {
            const char *t = w ? pp_b[q] : pp_a[q];
            auto it = text_id.emplace(std::string_view(t), (int)texts.size());
            if (it.second) texts.push_back(t);
            (w ? idb : ida)[q] = it.first->second;
        }
    std::vector<std::shared_ptr<const Side>> sides(texts.size());
    std::vector<Staged> side_err(texts.size());
    host_parallel((int)texts.size(), [&](int k) { guarded(side_err[k], [&]() { sides[k] = make_side(texts[k], o); }); });
    for (int q = 0; q < npairs; ++q) {
        const Staged &ea = side_err[ida[q]], &eb = side_err[idb[q]];
        if (ea.code != LCG_OK || eb.code != LCG_OK) {
            const Staged &e = ea.code != LCG_OK ? ea : eb;
            lcg_host::set_error("pair " + std::to_string(q) + ": " + e.err);
            return e.code;
        }
    }
    host_parallel(npairs, [&](int q) { guarded(st[q], [&]() { stage_inputs(sides[ida[q]], sides[idb[q]], st[q]); }); });
    for (int q = 0; q < npairs; ++q)
        if (st[q].code != LCG_OK) {
            lcg_host::set_error("pair " + std::to_string(q) + ": " + st[q].err);
            return st[q].code;
        }
    if (o.min_trace_probability > 0.0) {
        // per-position inputs of the GPU envelope
        lcg_env::Params ep;
        ep.sw = o.struct_weight / 100.0;
        ep.temp = o.temperature_alipf / 100.0;
        ep.g_open = exp((o.indel_opening / 100.0) / ep.temp);
        ep.g_ext = exp((o.indel / 100.0) / ep.temp);
        ep.min_prob = o.min_trace_probability;
        for (int a = 0; a < 4; ++a)
            for (int b = 0; b < 4; ++b)
                ep.score[a * 4 + b] = o.use_ribosum ? kBmScore[a * 4 + b] : (a == b ? (double)o.match : (double)o.mismatch);
        ep.local = o.sequ_local != 0;
        ep.fe = o.free_endgaps & 15;
        // |log2| range of the reference's float type, and the sequence
        // lengths up to which no value of the recursions comes near its
        // subnormal range; longer pairs take the host path
        const bool dbl = o.pf_precision == 0;
        ep.exp_limit = dbl ? 1000 : 16000;
        const int max_len_sum = dbl ? 1000 : 16000;
        std::vector<EnvBuf> &buf = B->buf;
        buf.resize(npairs);
        std::vector<lcg_env::PairIn> &in = B->in;
        std::vector<lcg_env::PairOut> &res = B->res;
        std::vector<int> gpu_q;
        B->kof.assign(npairs, -1);
        // the kernel scores single sequences; profiles take the host path
        for (int q = 0; q < npairs; ++q)
            if (st[q].pa->len + st[q].pb->len <= max_len_sum && st[q].pa->in.rows.size() == 1 &&
                st[q].pb->in.rows.size() == 1) {
                B->kof[q] = (int)gpu_q.size();
                gpu_q.push_back(q);
            }
        in.resize(gpu_q.size());
        res.resize(gpu_q.size());
        host_parallel((int)gpu_q.size(), [&](int k) {
            const int q = gpu_q[k];
            const Side &SA = *st[q].pa, &SB = *st[q].pb;
            const Staged &S = st[q];
            EnvBuf &b = buf[q];
            const int n = SA.len, m = SB.len;
            b.ca.assign(n + 1, -1);
            b.cb.assign(m + 1, -1);
            b.sdA.assign(n + 1, 0.0);
            b.suA.assign(n + 1, 0.0);
            b.sdB.assign(m + 1, 0.0);
            b.suB.assign(m + 1, 0.0);
            for (int i = 1; i <= n; ++i) {
                b.ca[i] = (int8_t)idx_acgu(SA.in.seq[i - 1]);
                b.sdA[i] = std::sqrt(SA.p_down[i]);
                b.suA[i] = std::sqrt(SA.p_up[i]);
            }
            for (int j = 1; j <= m; ++j) {
                b.cb[j] = (int8_t)idx_acgu(SB.in.seq[j - 1]);
                b.sdB[j] = std::sqrt(SB.p_down[j]);
                b.suB[j] = std::sqrt(SB.p_up[j]);
            }
            b.minc.assign(S.tc.minc.begin(), S.tc.minc.end());
            b.maxc.assign(S.tc.maxc.begin(), S.tc.maxc.end());
            b.nmin.assign(n + 1, 0);
            b.nmax.assign(n + 1, 0);
            in[k] = lcg_env::PairIn{n, m, b.ca.data(), b.cb.data(), b.sdA.data(), b.suA.data(),
                                   b.sdB.data(), b.suB.data(), b.minc.data(), b.maxc.data()};
            res[k] = lcg_env::PairOut{b.nmin.data(), b.nmax.data(), 0};
        });
        // the first pairs' envelopes now; the others enqueued behind them
        const int f = std::max(0, std::min<int>(first, npairs));
        const int kf = (int)(std::lower_bound(gpu_q.begin(), gpu_q.end(), f) - gpu_q.begin());
        std::string err;
        lcg_status rc = lcg_env::compute(eng, ep, kf, in.data(), res.data(), err);
        if (rc == LCG_OK && kf < (int)gpu_q.size())
            rc = lcg_env::compute_begin(eng, ep, (int)gpu_q.size() - kf, in.data() + kf, res.data() + kf,
                                        &B->pending, err);
        if (rc != LCG_OK) {
            lcg_host::set_error(err);
            return rc;
        }
        B->first = f;
        apply_envelopes(*B, 0, f);
        if (f >= npairs) B->first = npairs;
    } else {
        B->first = npairs;
    }
    if (host_envelopes) *host_envelopes = B->host_envelopes;
    *out = B.release();
    return LCG_OK;
}

lcg_status finish_tables(StagedBatch *B, int q0, int nq, lcg_prepared *out) {
    std::vector<Staged> &st = B->st;
    if (q0 + nq > B->first) {
        lcg_status rc = finish_envelopes(*B);
        if (rc != LCG_OK) return rc;
    }
    host_parallel(nq, [&](int k) { guarded(st[q0 + k], [&]() { stage_tables(st[q0 + k]); }); });
    for (int k = 0; k < nq; ++k)
        if (st[q0 + k].code != LCG_OK) {
            lcg_host::set_error("pair " + std::to_string(q0 + k) + ": " + st[q0 + k].err);
            return st[q0 + k].code;
        }
    for (int k = 0; k < nq; ++k) out[k] = st[q0 + k].P.release();
    return LCG_OK;
}

void free_batch(StagedBatch *B) { delete B; }

int batch_host_envelopes(const StagedBatch *B) { return B ? B->host_envelopes : 0; }

}  // namespace lcg_host

lcg_status lcg_prepare_pairs(lcg_engine eng, const char *const *pp_a, const char *const *pp_b, int32_t npairs,
                             const lcg_prep_opts *opts, lcg_prepared *out, int32_t *host_envelopes) {
    if (!eng || !pp_a || !pp_b || !out || npairs < 0) {
        lcg_host::set_error("NULL argument");
        return LCG_ERR_ARG;
    }
    for (int q = 0; q < npairs; ++q) out[q] = nullptr;
    lcg_host::StagedBatch *B = nullptr;
    lcg_status rc = lcg_host::stage_batch(eng, pp_a, pp_b, npairs, opts, &B, host_envelopes, npairs);
    if (rc == LCG_OK) rc = lcg_host::finish_tables(B, 0, npairs, out);
    lcg_host::free_batch(B);
    return rc;
}

lcg_status lcg_prepared_tables(lcg_prepared p, lcg_pair_tables *t) {
    if (!p || !t) {
        lcg_host::set_error("NULL argument");
        return LCG_ERR_ARG;
    }
    std::memset(t, 0, sizeof *t);
    t->len_a = p->n;
    t->len_b = p->m;
    t->sigma = p->sigma.data();
    t->gap_a = p->gap_a.data();
    t->gap_b = p->gap_b.data();
    t->indel_opening = p->indel_opening;
    t->exclusion = p->exclusion;
    t->num_arcs_a = (int32_t)(p->arcs_a.size() / 2);
    t->num_arcs_b = (int32_t)(p->arcs_b.size() / 2);
    t->arcs_a = p->arcs_a.data();
    t->arcs_b = p->arcs_b.data();
    t->num_arcmatches = (int32_t)p->am_score.size();
    t->am_arcs = p->am_arcs.data();
    t->am_score = p->am_score.data();
    t->min_col = p->min_col.data();
    t->max_col = p->max_col.data();
    if (p->stacking) {
        t->am_stack_score = p->am_stack_score.data();
        t->am_stackable = p->am_stackable.data();
    }
    t->right_anchor_a = 0;
    t->right_anchor_b = 0;
    t->left_anchor_a = p->n + 1;
    t->left_anchor_b = p->m + 1;
    if (!p->anchors.empty) {
        const AnchorRanges &R = p->anchors;
        t->match_lo = R.match_lo.data();
        t->match_hi = R.match_hi.data();
        t->del_lo = R.del_lo.data();
        t->del_hi = R.del_hi.data();
        t->ins_lo = R.ins_lo.data();
        t->ins_hi = R.ins_hi.data();
        t->right_anchor_a = R.ra_a;
        t->right_anchor_b = R.ra_b;
        t->left_anchor_a = R.la_a;
        t->left_anchor_b = R.la_b;
    }
    return LCG_OK;
}

const char *lcg_prepared_sequence(lcg_prepared p, int32_t which) {
    if (!p) return "";
    switch (which) {
    case 0: return p->seq_a.c_str();
    case 1: return p->seq_b.c_str();
    case 2: return p->name_a.c_str();
    case 3: return p->name_b.c_str();
    default: return "";
    }
}

const char *lcg_prepared_row(lcg_prepared p, int32_t which, int32_t k) {
    if (!p || k < 0) return nullptr;
    const std::vector<std::string> *v = nullptr;
    switch (which) {
    case 0: v = &p->rows_a; break;
    case 1: v = &p->rows_b; break;
    case 2: v = &p->row_names_a; break;
    case 3: v = &p->row_names_b; break;
    case 4: v = &p->anchor_rows_a; break;
    case 5: v = &p->anchor_rows_b; break;
    default: return nullptr;
    }
    return (size_t)k < v->size() ? (*v)[k].c_str() : nullptr;
}

int32_t lcg_prepared_envelope_ok(lcg_prepared p) { return p ? p->envelope_ok : 0; }

lcg_status lcg_prepared_grad_spec(lcg_prepared p, lcg_pf_grad_spec *out) {
    if (!p || !out) {
        lcg_host::set_error("NULL argument");
        return LCG_ERR_ARG;
    }
    out->code_a = p->code_a.data();
    out->code_b = p->code_b.data();
    out->am_dscore_dsw = p->am_dsw.data();
    return LCG_OK;
}

lcg_status lcg_prepared_free(lcg_prepared p) {
    delete p;
    return LCG_OK;
}
