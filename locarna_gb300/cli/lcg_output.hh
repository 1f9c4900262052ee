// Alignment output of the locarna / locarna_p command lines: the traced edges
// expanded to the full alignment, the structure strings, and the CLUSTAL and
// Stockholm writers, as the reference prints them.
//
//   alignment_edges   Alignment::alignment_edges        (src/LocARNA/alignment.cc:120-167)
//   structure         Alignment::dot_bracket_structureA/B (alignment.cc:215-239)
//                     with add_basepairA/B               (alignment.cc:97-107)
//   rows              MultipleAlignment(const Alignment&) (multiple_alignment.cc:153-245)
//   anchor_consensus  SequenceAnnotation(edges, A, B)     (sequence_annotation.cc:15-51)
//                     kept unless duplicate_names()       (multiple_alignment.cc:157-165,
//                                                          sequence_annotation.cc:103-120)
//   write_blocks      MultipleAlignment::write            (multiple_alignment.cc:995-1085)
//
// Edge ends are ints: a position p >= 1, or a gap -1 - code with the
// reference's Gap codes (aux.hh:132-137): regular 0, loop 1, locality 2; a
// gap prints as the simplified gap symbol of its code (aux.cc:24-38).
#pragma once
#include <algorithm>
#include <ostream>
#include <set>
#include <string>
#include <utility>
#include <vector>

namespace lcg_cli {

constexpr int GAP_REGULAR = -1;
constexpr int GAP_LOCALITY = -3;

inline char gap_char(int code) {
    static const char simplified[] = "---.";
    return simplified[-1 - code];
}

using Edges = std::vector<std::pair<int, int>>;

// raw: the edges in the order the traceback appends them, -1 for a gap
inline Edges alignment_edges(const Edges &raw, int len_a, int len_b, bool only_local = false) {
    Edges res;
    int last_a = 1, last_b = 1;
    for (const auto &e : raw) {
        if (e.first > 0) {
            for (int j = last_a; j < e.first; ++j) {
                if (!only_local) res.emplace_back(j, GAP_LOCALITY);
                ++last_a;
            }
        }
        if (e.second > 0) {
            for (int j = last_b; j < e.second; ++j) {
                if (!only_local) res.emplace_back(GAP_LOCALITY, j);
                ++last_b;
            }
        }
        if (e.first > 0) ++last_a;
        if (e.second > 0) ++last_b;
        res.emplace_back(e.first > 0 ? e.first : GAP_REGULAR, e.second > 0 ? e.second : GAP_REGULAR);
    }
    if (!only_local) {
        for (int j = last_a; j <= len_a; ++j) res.emplace_back(j, GAP_LOCALITY);
        for (int j = last_b; j <= len_b; ++j) res.emplace_back(GAP_LOCALITY, j);
    }
    return res;
}

// dot-bracket strings of both sides along the edges; arcs: the traced arc
// matches as ((a.l, a.r), (b.l, b.r))
inline std::pair<std::string, std::string> structure(const Edges &edges, int len_a, int len_b,
                                                     const std::vector<std::pair<std::pair<int, int>, std::pair<int, int>>> &arcs) {
    std::string sa((size_t)len_a + 1, '.'), sb((size_t)len_b + 1, '.');
    for (const auto &am : arcs) {
        sa[am.first.first] = '(';
        sa[am.first.second] = ')';
        sb[am.second.first] = '(';
        sb[am.second.second] = ')';
    }
    std::string a, b;
    for (const auto &e : edges) {
        a += e.first > 0 ? sa[e.first] : gap_char(e.first);
        b += e.second > 0 ? sb[e.second] : gap_char(e.second);
    }
    return {a, b};
}

struct Row {
    std::string name, seq;
};

// the alignment rows: every row of A, then every row of B, along the edges;
// names present on both sides get the prefixes "A." / "B."
inline std::vector<Row> rows(const Edges &edges, const std::vector<Row> &in_a, const std::vector<Row> &in_b) {
    bool clash = false;
    for (const auto &ra : in_a)
        for (const auto &rb : in_b) clash = clash || ra.name == rb.name;
    std::vector<Row> out;
    for (const auto &r : in_a) {
        std::string s;
        for (const auto &e : edges) s += e.first > 0 ? r.seq[e.first - 1] : gap_char(e.first);
        out.push_back({clash ? "A." + r.name : r.name, s});
    }
    for (const auto &r : in_b) {
        std::string s;
        for (const auto &e : edges) s += e.second > 0 ? r.seq[e.second - 1] : gap_char(e.second);
        out.push_back({clash ? "B." + r.name : r.name, s});
    }
    return out;
}

// Consensus of the inputs' anchor lines along the edges: one string per
// character of the anchor names (line k holds character k of every column's
// name). A column aligned to a gap takes the other side's name; a match
// takes the non-neutral name, or the smaller of two (a name is neutral when
// it holds only ' ' and '.'). Empty when either input has no anchor lines,
// or when two non-neutral columns share a name (the reference then sets no
// anchor annotation).
inline std::vector<std::string> anchor_consensus(const Edges &edges, const std::vector<std::string> &in_a,
                                                 const std::vector<std::string> &in_b) {
    if (in_a.empty() || in_b.empty() || in_a[0].empty() || in_b[0].empty()) return {};
    const size_t nl = in_a.size();
    auto name_of = [](const std::vector<std::string> &lines, int pos) {
        std::string nm;
        for (const auto &l : lines) nm += (size_t)pos <= l.size() ? l[pos - 1] : ' ';
        return nm;
    };
    auto neutral = [](const std::string &nm) {
        return std::all_of(nm.begin(), nm.end(), [](char c) { return c == ' ' || c == '.'; });
    };
    std::vector<std::string> out(nl);
    std::set<std::string> seen;
    for (const auto &e : edges) {
        std::string nm;
        if (e.first <= 0) {
            nm = name_of(in_b, e.second);
        } else if (e.second <= 0) {
            nm = name_of(in_a, e.first);
        } else {
            const std::string na = name_of(in_a, e.first), nb = name_of(in_b, e.second);
            nm = neutral(na) ? nb : neutral(nb) ? na : std::min(na, nb);
        }
        if (!neutral(nm) && !seen.insert(nm).second) return {};
        for (size_t k = 0; k < nl; ++k) out[k] += k < nm.size() ? nm[k] : ' ';
    }
    return out;
}

// blocks of `width` columns, "name sequence" lines with the name padded to
// max(18, longest row name), then per block the anchor lines tagged "#A<k>"
// ("#=GC cA<k>" in Stockholm), a blank line between blocks; Stockholm ends
// with "//"
inline void write_blocks(std::ostream &out, const std::vector<Row> &rs, size_t width, bool stockholm,
                         const std::vector<std::string> &anchors = {}) {
    size_t namew = 18, len = 0;
    for (const auto &r : rs) {
        namew = std::max(namew, r.name.size());
        len = std::max(len, r.seq.size());
    }
    if (width == 0) width = len;
    auto line = [&](std::string name, const std::string &seq, size_t start, size_t end) {
        if (name.size() < namew) name.append(namew - name.size(), ' ');
        out << name << " " << seq.substr(std::min(start, seq.size()), end - start) << "\n";
    };
    size_t start = 0;
    do {
        const size_t end = std::min(len, start + width);
        for (const auto &r : rs) line(r.name, r.seq, start, end);
        for (size_t k = 0; k < anchors.size(); ++k)
            line(std::string(stockholm ? "#=GC cA" : "#A") + std::to_string(k + 1), anchors[k], start, end);
        start = end;
        if (start < len) out << "\n";
    } while (start < len);
    if (stockholm) out << "//\n";
}

}  // namespace lcg_cli
