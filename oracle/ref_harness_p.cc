// Test infrastructure only (oracle). In-process harness over the REFERENCE's
// own LocARNA-P (AlignerP, src/LocARNA/aligner_p.icc) built from the
// reference sources by oracle/build_ref.sh, following src/locarna_p.cc:298-531
// for PP inputs. Prints the prepared tables (as oracle/ref_harness.cc does),
// the partition function, and every arc-match and base-match probability
// with 17 significant digits, plus the time of inside+outside+probabilities.
//
// Usage: ref_harness_p A.pp B.pp [key=value ...]
//   min_trace_prob=1e-5 min_am_prob=0 include_am=0 extended=0 pf_scale=1
//   temperature=300 min_prob=0.001 dump_tables=1 repeat=1
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <memory>
#include <string>

#include "LocARNA/aligner_p.hh"
#include "LocARNA/aligner_params.hh"
#include "LocARNA/anchor_constraints.hh"
#include "LocARNA/arc_matches.hh"
#include "LocARNA/basepairs.hh"
#include "LocARNA/edge_probs.hh"
#include "LocARNA/free_endgaps.hh"
#include "LocARNA/multiple_alignment.hh"
#include "LocARNA/pfold_params.hh"
#include "LocARNA/ribosum.hh"
#include "LocARNA/rna_data.hh"
#include "LocARNA/scoring.hh"
#include "LocARNA/sequence.hh"
#include "LocARNA/trace_controller.hh"
#include "LocARNA/ribosum85_60.icc"

using namespace LocARNA;

struct Opts {
    double min_trace_prob = 1e-5, min_am_prob = 0.0, min_prob = 0.001, pf_scale = 1.0;
    int include_am = 0, extended = 0, temperature = 300, dump_tables = 1, repeat = 1;
};

template <class T>
int run(const Opts &o, const char *fa, const char *fb) {
    auto ribosum = std::make_unique<Ribosum85_60>();
    PFoldParams pfoldparams(PFoldParams::args::noLP(false), PFoldParams::args::stacking(false),
                            PFoldParams::args::max_bp_span(-1));
    RnaData rnaA(fa, o.min_prob, 0.0, pfoldparams);
    RnaData rnaB(fb, o.min_prob, 0.0, pfoldparams);
    const Sequence &seqA = rnaA.sequence();
    const Sequence &seqB = rnaB.sequence();
    size_t lenA = seqA.length(), lenB = seqB.length();
    AnchorConstraints anchors(
        lenA, seqA.annotation(MultipleAlignment::AnnoType::anchors).single_string(), lenB,
        seqB.annotation(MultipleAlignment::AnnoType::anchors).single_string(), true);
    TraceController tc(seqA, seqB, nullptr, -1, false);
    tc.restrict_by_anchors(anchors);
    if (o.min_trace_prob > 0.0) {
        PFTraceProbs<T> tp(rnaA, rnaB, tc, ribosum->get_basematch_scores(), ribosum->alphabet(),
                           -750 / 100.0, -150 / 100.0, 200 / 100.0, o.temperature / 100.0,
                           FreeEndgaps("----"), false);
        tc.restrict_by_trace_probabilities(tp, o.min_trace_prob);
    }
    ArcMatches am(rnaA, rnaB, o.min_prob, std::max(lenA, lenB), std::max(lenA, lenB), tc, anchors);
    ScoringParams sp(ScoringParams::match(50), ScoringParams::mismatch(0), ScoringParams::indel(-150),
                     ScoringParams::indel_opening(-750), ScoringParams::ribosum(ribosum.get()),
                     ScoringParams::ribofit(nullptr), ScoringParams::struct_weight(200),
                     ScoringParams::tau_factor(50), ScoringParams::exp_probA(prob_exp_f(lenA)),
                     ScoringParams::exp_probB(prob_exp_f(lenB)),
                     ScoringParams::temperature_alipf(o.temperature));
    PFScoring<T> scoring(seqA, seqB, rnaA, rnaB, am, nullptr, sp);
    const BasePairs &bpsA = am.get_base_pairsA();
    const BasePairs &bpsB = am.get_base_pairsB();
    std::printf("LCGREFP 1\nlens %zu %zu\n", lenA, lenB);
    std::printf("band");
    for (size_t i = 0; i <= lenA; ++i) std::printf(" %zu:%zu", tc.min_col(i), tc.max_col(i));
    std::printf("\nnarcs %zu %zu\nnam %zu\n", bpsA.num_bps(), bpsB.num_bps(), am.num_arc_matches());
    if (o.dump_tables) {
        std::printf("params %ld %ld\n", (long)scoring.indel_opening(), (long)scoring.exclusion());
        std::printf("seqA %s\nseqB %s\n", seqA.seqentry(0).seq().str().c_str(), seqB.seqentry(0).seq().str().c_str());
        std::printf("gapA");
        for (size_t i = 0; i <= lenA; ++i) std::printf(" %ld", (long)(i ? scoring.gapA(i) : 0));
        std::printf("\ngapB");
        for (size_t j = 0; j <= lenB; ++j) std::printf(" %ld", (long)(j ? scoring.gapB(j) : 0));
        std::printf("\nsigma");
        for (size_t i = 1; i <= lenA; ++i)
            for (size_t j = 1; j <= lenB; ++j) std::printf(" %ld", (long)scoring.basematch(i, j));
        std::printf("\narcsA");
        for (size_t k = 0; k < bpsA.num_bps(); ++k) std::printf(" %zu:%zu", bpsA.arc(k).left(), bpsA.arc(k).right());
        std::printf("\narcsB");
        for (size_t k = 0; k < bpsB.num_bps(); ++k) std::printf(" %zu:%zu", bpsB.arc(k).left(), bpsB.arc(k).right());
        std::printf("\nam");
        for (size_t k = 0; k < am.num_arc_matches(); ++k) {
            const ArcMatch &x = am.arcmatch(k);
            std::printf(" %zu:%zu:%ld", x.arcA().idx(), x.arcB().idx(), (long)scoring.arcmatch(x));
        }
        std::printf("\n");
    }
    double best = 1e30;
    std::unique_ptr<AlignerP<T>> keep;
    T Z = 0;
    for (int r = 0; r < std::max(1, o.repeat); ++r) {
        auto t0 = std::chrono::steady_clock::now();
        using apparams_t = AlignerPParams<T>;
        auto al = std::make_unique<AlignerP<T>>(apparams_t(
            AlignerParams::seqA(&seqA), AlignerParams::seqB(&seqB), AlignerParams::scoring(&scoring),
            AlignerParams::max_diff_am(-1), AlignerParams::max_diff_at_am(-1),
            AlignerParams::trace_controller(&tc), AlignerParams::constraints(&anchors),
            typename apparams_t::min_am_prob(o.min_am_prob), typename apparams_t::min_bm_prob(0.0),
            typename apparams_t::pf_scale((T)o.pf_scale)));
        Z = al->align_inside();
        al->align_outside();
        al->compute_arcmatch_probabilities();
        al->compute_basematch_probabilities(o.include_am);
        auto t1 = std::chrono::steady_clock::now();
        best = std::min(best, std::chrono::duration<double>(t1 - t0).count());
        keep = std::move(al);
    }
    std::printf("Z %.17g\n", (double)Z);
    // probabilities through the reference writers are rounded to 6 digits;
    // recompute them at full precision through the same objects
    std::ostringstream amo, bmo;
    amo.precision(17);
    bmo.precision(17);
    keep->write_arcmatch_probabilities(amo);
    keep->write_basematch_probabilities(bmo);
    std::string line;
    std::istringstream ami(amo.str()), bmi(bmo.str());
    std::printf("amprobs");
    while (std::getline(ami, line)) {
        std::istringstream l(line);
        size_t a, b, c, d;
        double p;
        l >> a >> b >> c >> d >> p;
        std::printf(" %zu:%zu:%zu:%zu:%.17g", a, b, c, d, p);
    }
    std::printf("\nbmprobs");
    while (std::getline(bmi, line)) {
        std::istringstream l(line);
        size_t i, j;
        double p;
        l >> i >> j >> p;
        std::printf(" %zu:%zu:%.17g", i, j, p);
    }
    std::printf("\npf_seconds %.6f\n", best);
    return 0;
}

int main(int argc, char **argv) {
    if (argc < 3) return 2;
    Opts o;
    for (int k = 3; k < argc; ++k) {
        std::string s(argv[k]);
        auto p = s.find('=');
        std::string key = s.substr(0, p), v = s.substr(p + 1);
        if (key == "min_trace_prob") o.min_trace_prob = std::atof(v.c_str());
        else if (key == "min_am_prob") o.min_am_prob = std::atof(v.c_str());
        else if (key == "min_prob") o.min_prob = std::atof(v.c_str());
        else if (key == "pf_scale") o.pf_scale = std::atof(v.c_str());
        else if (key == "include_am") o.include_am = std::atoi(v.c_str());
        else if (key == "extended") o.extended = std::atoi(v.c_str());
        else if (key == "temperature") o.temperature = std::atoi(v.c_str());
        else if (key == "dump_tables") o.dump_tables = std::atoi(v.c_str());
        else if (key == "repeat") o.repeat = std::atoi(v.c_str());
        else { std::fprintf(stderr, "unknown option %s\n", key.c_str()); return 2; }
    }
    if (o.extended) return run<long double>(o, argv[1], argv[2]);
    return run<double>(o, argv[1], argv[2]);
}
