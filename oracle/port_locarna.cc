// ORACLE — test infrastructure only: the CPU port of `locarna A.pp B.pp`
// (default flags: global alignment, RIBOSUM85_60 scoring, envelope 1e-4) that
// bench.py's reference arm times. It reads pairs of PP file names from
// standard input (one pair per line), and for each pair runs the same steps
// as the reference's locarna driver (src/locarna.cc:398-785): PP reading,
// scoring tables and sequence envelope (the host table preparation,
// lcg_prepare_pair, in long double as locarna computes it), then Aligner::align
// + Aligner::trace (the plain-C restatement, oracle/sankoff_oracle.c). Prints
// one line "<score> <edges>" per pair. Nothing here runs on a GPU and nothing
// of the GPU engine is linked in.
#include <cstdio>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "../include/locarna_gb300.h"

extern "C" int lcg_oracle_align(const lcg_pair_tables *t, const lcg_align_opts *o, lcg_align_result *r,
                                lcg_work_counts *cnt);

static bool slurp(const std::string &path, std::string &out) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    std::stringstream ss;
    ss << f.rdbuf();
    out = ss.str();
    return true;
}

int main() {
    std::string a, b;
    lcg_prep_opts po;
    lcg_prep_opts_default(&po);
    lcg_align_opts ao{};
    ao.do_trace = 1;
    int rc_all = 0;
    while (std::cin >> a >> b) {
        std::string ta, tb;
        if (!slurp(a, ta) || !slurp(b, tb)) {
            std::fprintf(stderr, "cannot read %s / %s\n", a.c_str(), b.c_str());
            return 2;
        }
        lcg_prepared p = nullptr;
        if (lcg_prepare_pair(ta.c_str(), tb.c_str(), &po, &p) != LCG_OK) {
            std::fprintf(stderr, "%s %s: %s\n", a.c_str(), b.c_str(), lcg_last_error());
            return 3;
        }
        lcg_pair_tables t;
        lcg_prepared_tables(p, &t);
        std::vector<int32_t> edges(2 * (t.len_a + t.len_b) + 2), tam(std::min(t.len_a, t.len_b) + 1);
        lcg_align_result r{};
        r.edges = edges.data();
        r.traced_am = tam.data();
        if (lcg_oracle_align(&t, &ao, &r, nullptr) != 0) rc_all = 4;
        std::printf("%lld %d\n", (long long)r.score, r.num_edges);
        lcg_prepared_free(p);
    }
    return rc_all;
}
