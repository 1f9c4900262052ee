// Drives the C++ facade (include/locarna_gb300.hpp) the way src/locarna.cc
// and src/locarna_p.cc drive LocARNA::Aligner / LocARNA::AlignerP: prepare a
// pair from two PP files, align + trace, then the partition function and its
// probabilities. Prints one line per result for the test that runs it.
// Usage: facade_demo A.pp B.pp [free_endgaps] [struct_local 0/1] [sequ_local 0/1]
#include <cstdio>
#include <fstream>
#include <sstream>
#include <string>

#include "locarna_gb300.hpp"

static std::string slurp(const char *path) {
    std::ifstream f(path);
    std::stringstream s;
    s << f.rdbuf();
    return s.str();
}

int main(int argc, char **argv) {
    if (argc < 3) {
        std::fprintf(stderr, "usage: %s A.pp B.pp [free_endgaps] [struct_local] [sequ_local]\n", argv[0]);
        return 2;
    }
    try {
        namespace lg = locarna_gb300;
        lg::Engine engine(0);
        lg::PreparedPair pair(slurp(argv[1]), slurp(argv[2]));
        const lcg_pair_tables t = pair.tables();
        lg::AlignerParams ap;
        ap.with_tables(&t)
            .with_free_endgaps(argc > 3 ? argv[3] : "----")
            .with_struct_local(argc > 4 && argv[4][0] == '1')
            .with_sequ_local(argc > 5 && argv[5][0] == '1');
        lg::Aligner aligner(ap, engine);
        const int64_t score = aligner.align();
        aligner.trace();
        const lg::Alignment &a = aligner.get_alignment();
        std::printf("score %lld\n", (long long)score);
        std::printf("edges");
        for (auto &e : a.edges) std::printf(" %d,%d", e.first, e.second);
        std::printf("\ntraced");
        for (int k : a.traced_arcmatches) std::printf(" %d", k);
        std::printf("\n");
        if (argc <= 3) {
            lcg_prep_opts po;
            lcg_prep_opts_default(&po);
            po.min_trace_probability = 1e-5;
            po.pf_precision = 0;
            lg::PreparedPair pp(slurp(argv[1]), slurp(argv[2]), &po);
            const lcg_pair_tables tp = pp.tables();
            lg::AlignerPParams pap;
            pap.tables = &tp;
            lg::AlignerP ap2(pap, engine);
            const double lz = ap2.align_inside();
            ap2.align_outside();
            const auto &am = ap2.compute_arcmatch_probabilities();
            const auto bm = ap2.compute_basematch_probabilities(false);
            double sam = 0, sbm = 0;
            for (double x : am) sam += x;
            for (double x : bm) sbm += x;
            std::printf("log_z %.12f\nsum_am %.12f\nsum_bm %.12f\n", lz, sam, sbm);
        }
    } catch (const locarna_gb300::failure &e) {
        std::fprintf(stderr, "failure: %s\n", e.what());
        return 1;
    }
    return 0;
}
