// Test infrastructure only (oracle). Not shipped, never on the product path.
//
// In-process harness over the REFERENCE's own LocARNA library objects (built
// from the reference sources by oracle/build_ref.sh into oracle/_ref/). It runs
// the pipeline of src/locarna.cc:398-785 for PP inputs with the options used by
// the parity tests, and prints, in one text block:
//   * the prepared tables the Sankoff DP consumes (sigma, gap costs, arcs in
//     reference index order, arc matches with Scoring::arcmatch scores, the
//     TraceController band, anchor ranges);
//   * the results: score, max_i/max_j, raw traceback edges, structure strings;
//   * the wall time of Aligner::align()+trace() alone.
// The test suite turns this output into golden fixtures (tests/golden/) and the
// bench uses the timing line as the reference's own CPU baseline.
//
// Usage: ref_harness A.pp B.pp [key=value ...]
//   struct_local=0|1 sequ_local=0|1 no_lonely_pairs=0|1 free_endgaps=---- min_trace_prob=1e-4
//   max_diff=-1 min_prob=0.001 indel=-150 indel_opening=-750 struct_weight=200
//   tau=50 exclusion=0 stacking=0|1 new_stacking=0|1 exp_prob=P normalized=L penalized=PP
//   dump_tables=1 repeat=1
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <memory>
#include <queue>
#include <string>
#include <vector>

#include "LocARNA/aligner.hh"
#include "LocARNA/aligner_restriction.hh"
#include "LocARNA/aligner_params.hh"
#include "LocARNA/alignment.hh"
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
    bool struct_local = false, sequ_local = false, no_lonely_pairs = false;
    std::string free_endgaps = "----";
    double min_trace_prob = 1e-4, min_prob = 0.001;
    int max_diff = -1, indel = -150, indel_opening = -750, struct_weight = 200,
        tau = 50, exclusion = 0, max_diff_am = -1, max_diff_at_am = -1;
    bool stacking = false, new_stacking = false;
    double exp_prob = -1;  // --exp-prob; < 0: not given
    int normalized = -1, penalized = -1;  // --normalized L / --penalized PP (-1: off)
    int kbest = 0;                          // --kbest k (0: off)
    bool relaxed_anchors = false;           // --relaxed-anchors
    long better = -1000000;                 // --better t
    bool dump_tables = true;
    int repeat = 1;
};

static void parse(Opts &o, const char *kv) {
    std::string s(kv);
    auto p = s.find('=');
    if (p == std::string::npos) { std::cerr << "bad option " << s << "\n"; std::exit(2); }
    std::string k = s.substr(0, p), v = s.substr(p + 1);
    if (k == "struct_local") o.struct_local = std::atoi(v.c_str());
    else if (k == "sequ_local") o.sequ_local = std::atoi(v.c_str());
    else if (k == "no_lonely_pairs") o.no_lonely_pairs = std::atoi(v.c_str());
    else if (k == "free_endgaps") o.free_endgaps = v;
    else if (k == "min_trace_prob") o.min_trace_prob = std::atof(v.c_str());
    else if (k == "min_prob") o.min_prob = std::atof(v.c_str());
    else if (k == "max_diff") o.max_diff = std::atoi(v.c_str());
    else if (k == "max_diff_am") o.max_diff_am = std::atoi(v.c_str());
    else if (k == "max_diff_at_am") o.max_diff_at_am = std::atoi(v.c_str());
    else if (k == "indel") o.indel = std::atoi(v.c_str());
    else if (k == "indel_opening") o.indel_opening = std::atoi(v.c_str());
    else if (k == "struct_weight") o.struct_weight = std::atoi(v.c_str());
    else if (k == "tau") o.tau = std::atoi(v.c_str());
    else if (k == "exclusion") o.exclusion = std::atoi(v.c_str());
    else if (k == "dump_tables") o.dump_tables = std::atoi(v.c_str());
    else if (k == "stacking") o.stacking = std::atoi(v.c_str());
    else if (k == "new_stacking") o.new_stacking = std::atoi(v.c_str());
    else if (k == "exp_prob") o.exp_prob = std::atof(v.c_str());
    else if (k == "normalized") o.normalized = std::atoi(v.c_str());
    else if (k == "penalized") o.penalized = std::atoi(v.c_str());
    else if (k == "kbest") o.kbest = std::atoi(v.c_str());
    else if (k == "relaxed_anchors") o.relaxed_anchors = std::atoi(v.c_str());
    else if (k == "better") o.better = std::atol(v.c_str());
    else if (k == "repeat") o.repeat = std::atoi(v.c_str());
    else { std::cerr << "unknown option " << k << "\n"; std::exit(2); }
}

static long score_val(const infty_score_t &s) {
    if (s.is_neg_infty()) return -(1L << 40);
    return s.finite_value();
}

int main(int argc, char **argv) {
    if (argc < 3) { std::cerr << "usage: ref_harness A.pp B.pp [k=v...]\n"; return 2; }
    Opts o;
    for (int k = 3; k < argc; ++k) parse(o, argv[k]);

    // ribosum as in MainHelper::init_ribo_matrix (main_helper.icc:251-279)
    auto ribosum = std::make_unique<Ribosum85_60>();
    // locarna turns the (old) stacking off unless --exp-prob is given
    // (src/locarna.cc:407-414)
    if (o.stacking && o.exp_prob < 0) o.stacking = false;
    const bool stacking = o.stacking || o.new_stacking;
    PFoldParams pfoldparams(PFoldParams::args::noLP(false),
                            PFoldParams::args::stacking(stacking),
                            PFoldParams::args::max_bp_span(-1));
    RnaData rnaA(argv[1], o.min_prob, 0.0, pfoldparams);
    RnaData rnaB(argv[2], o.min_prob, 0.0, pfoldparams);
    const Sequence &seqA = rnaA.sequence();
    const Sequence &seqB = rnaB.sequence();
    size_t lenA = seqA.length(), lenB = seqB.length();

    AnchorConstraints anchors(
        lenA, seqA.annotation(MultipleAlignment::AnnoType::anchors).single_string(),
        lenB, seqB.annotation(MultipleAlignment::AnnoType::anchors).single_string(),
        !o.relaxed_anchors);
    TraceController tc(seqA, seqB, nullptr, o.max_diff, false);
    tc.restrict_by_anchors(anchors);

    // envelope as in MainHelper::make_trace_probs (main_helper.icc:356-400),
    // extended (long double) precision as forced by src/locarna.cc:384
    if (o.min_trace_prob > 0.0) {
        PFTraceProbs<long double> tp(rnaA, rnaB, tc, ribosum->get_basematch_scores(),
                                     ribosum->alphabet(), o.indel_opening / 100.0,
                                     o.indel / 100.0, o.struct_weight / 100.0,
                                     300 / 100.0, FreeEndgaps(o.free_endgaps),
                                     o.sequ_local);
        tc.restrict_by_trace_probabilities(tp, o.min_trace_prob);
    }

    size_t mdam = o.max_diff_am != -1 ? (size_t)o.max_diff_am : std::max(lenA, lenB);
    size_t mdaam = o.max_diff_at_am != -1 ? (size_t)o.max_diff_at_am : std::max(lenA, lenB);
    ArcMatches am(rnaA, rnaB, o.min_prob, mdam, mdaam, tc, anchors);

    auto sp = ScoringParams(
        ScoringParams::match(50), ScoringParams::mismatch(0),
        ScoringParams::indel(o.indel), ScoringParams::indel_opening(o.indel_opening),
        ScoringParams::ribosum(ribosum.get()), ScoringParams::ribofit(nullptr),
        ScoringParams::unpaired_penalty(0), ScoringParams::struct_weight(o.struct_weight),
        ScoringParams::tau_factor(o.tau), ScoringParams::exclusion(o.exclusion),
        ScoringParams::exp_probA(o.exp_prob >= 0 ? o.exp_prob : prob_exp_f(lenA)),
        ScoringParams::exp_probB(o.exp_prob >= 0 ? o.exp_prob : prob_exp_f(lenB)),
        ScoringParams::temperature_alipf(300), ScoringParams::stacking(o.stacking),
        ScoringParams::new_stacking(o.new_stacking), ScoringParams::mea_scoring(false),
        ScoringParams::mea_alpha(0), ScoringParams::mea_beta(200),
        ScoringParams::mea_gamma(100), ScoringParams::probability_scale(10000));
    Scoring scoring(seqA, seqB, rnaA, rnaB, am, nullptr, sp);

    const BasePairs &bpsA = am.get_base_pairsA();
    const BasePairs &bpsB = am.get_base_pairsB();

    std::printf("LCGREF 1\n");
    std::printf("lens %zu %zu\n", lenA, lenB);
    std::printf("seqA %s\n", seqA.seqentry(0).seq().str().c_str());
    std::printf("seqB %s\n", seqB.seqentry(0).seq().str().c_str());
    std::printf("params %ld %ld\n", (long)scoring.indel_opening(), (long)scoring.exclusion());
    std::printf("band");
    for (size_t i = 0; i <= lenA; ++i) std::printf(" %zu:%zu", tc.min_col(i), tc.max_col(i));
    std::printf("\n");
    std::printf("narcs %zu %zu\n", bpsA.num_bps(), bpsB.num_bps());
    std::printf("nam %zu\n", am.num_arc_matches());
    if (o.dump_tables) {
        std::printf("gapA");
        for (size_t i = 0; i <= lenA; ++i) std::printf(" %ld", (long)(i ? scoring.gapA(i) : 0));
        std::printf("\ngapB");
        for (size_t j = 0; j <= lenB; ++j) std::printf(" %ld", (long)(j ? scoring.gapB(j) : 0));
        std::printf("\nsigma");
        for (size_t i = 1; i <= lenA; ++i)
            for (size_t j = 1; j <= lenB; ++j) std::printf(" %ld", (long)scoring.basematch(i, j));
        std::printf("\narcsA");
        for (size_t k = 0; k < bpsA.num_bps(); ++k)
            std::printf(" %zu:%zu", bpsA.arc(k).left(), bpsA.arc(k).right());
        std::printf("\narcsB");
        for (size_t k = 0; k < bpsB.num_bps(); ++k)
            std::printf(" %zu:%zu", bpsB.arc(k).left(), bpsB.arc(k).right());
        std::printf("\nam");
        for (size_t k = 0; k < am.num_arc_matches(); ++k) {
            const ArcMatch &x = am.arcmatch(k);
            std::printf(" %zu:%zu:%ld", x.arcA().idx(), x.arcB().idx(), (long)scoring.arcmatch(x));
        }
        if (stacking) {
            // Scoring::arcmatch(am, true) and Scoring::is_stackable_am per arc match
            std::printf("\namstack");
            for (size_t k = 0; k < am.num_arc_matches(); ++k) {
                const ArcMatch &x = am.arcmatch(k);
                std::printf(" %ld:%d", (long)scoring.arcmatch(x, true), (int)scoring.is_stackable_am(x));
            }
        }
        std::printf("\nanchor_match");
        for (size_t i = 1; i <= lenA; ++i) {
            long lo = -1, hi = -2;
            for (size_t j = 0; j <= lenB; ++j)
                if (anchors.allowed_match(i, j)) { if (lo < 0) lo = j; hi = j; }
            std::printf(" %ld:%ld", lo, hi);
        }
        // the deletion and insertion ranges (AnchorConstraints::allowed_del /
        // allowed_ins, anchor_constraints.hh:160-253), checked to be intervals
        bool intervals = true;
        std::printf("\nanchor_del");
        for (size_t i = 1; i <= lenA; ++i) {
            long lo = -1, hi = -2;
            for (size_t j = 0; j <= lenB; ++j)
                if (anchors.allowed_del(i, j)) {
                    if (lo < 0) lo = j;
                    else if (hi != (long)j - 1) intervals = false;
                    hi = j;
                }
            std::printf(" %ld:%ld", lo, hi);
        }
        std::printf("\nanchor_ins");
        for (size_t j = 1; j <= lenB; ++j) {
            long lo = -1, hi = -2;
            for (size_t i = 0; i <= lenA; ++i)
                if (anchors.allowed_ins(i, j)) {
                    if (lo < 0) lo = i;
                    else if (hi != (long)i - 1) intervals = false;
                    hi = i;
                }
            std::printf(" %ld:%ld", lo, hi);
        }
        auto ra = anchors.rightmost_anchor(), la = anchors.leftmost_anchor();
        std::printf("\nanchor_ends %zu %zu %zu %zu %d %d\n", ra.first, ra.second, la.first, la.second,
                    (int)anchors.empty(), (int)intervals);
    }

    auto make_aligner = [&]() {
        return std::make_unique<Aligner>(AlignerParams(
            AlignerParams::seqA(&seqA), AlignerParams::seqB(&seqB),
            AlignerParams::scoring(&scoring), AlignerParams::no_lonely_pairs(o.no_lonely_pairs),
            AlignerParams::struct_local(o.struct_local), AlignerParams::sequ_local(o.sequ_local),
            AlignerParams::free_endgaps(FreeEndgaps(o.free_endgaps)),
            AlignerParams::max_diff_am(o.max_diff_am), AlignerParams::max_diff_at_am(o.max_diff_at_am),
            AlignerParams::trace_controller(&tc), AlignerParams::stacking(stacking),
            AlignerParams::constraints(&anchors)));
    };
    if (o.kbest > 0) {
        // (1) the reference's own enumeration (Aligner::suboptimal), which
        // prints "HIT score startA startA endB endB" per hit
        std::fflush(stdout);
        make_aligner()->suboptimal(o.kbest, o.better, o.normalized >= 0, std::max(o.normalized, 0), 120, false,
                                   false, true, false);
        std::cout.flush();
        // (2) the same enumeration through the public Aligner API
        // (aligner.cc:1384-1512), printing each hit's full alignment
        auto a = make_aligner();
        typedef std::pair<AlignerRestriction, infty_score_t> task_t;
        std::priority_queue<task_t, std::vector<task_t>, greater_second<task_t>> tasks;
        const bool norm = o.normalized >= 0;
        infty_score_t s0 = norm ? a->normalized_align(o.normalized, false) : a->align();
        tasks.push(task_t(a->get_restriction(), s0));
        for (size_t i = 1; i <= (size_t)o.kbest && !tasks.empty();) {
            task_t task = tasks.top();
            tasks.pop();
            AlignerRestriction r = task.first;
            if (task.second < (infty_score_t)o.better + 1) break;
            a->set_restriction(r);
            if (norm) {
                a->normalized_align(o.normalized, false);
            } else {
                a->align();
                a->trace();
            }
            Alignment alignment = a->get_alignment();
            if (alignment.empty()) continue;
            std::printf("khit %ld", score_val(task.second));
            for (auto &e : alignment.alignment_edges(false)) {
                int x = e.first.is_pos() ? (int)(size_t)e.first : -1 - (int)e.first.gap();
                int y = e.second.is_pos() ? (int)(size_t)e.second : -1 - (int)e.second.gap();
                std::printf(" %d:%d", x, y);
            }
            std::printf("\nklocal");
            for (auto &e : alignment.alignment_edges(true)) {
                int x = e.first.is_pos() ? (int)(size_t)e.first : -1 - (int)e.first.gap();
                int y = e.second.is_pos() ? (int)(size_t)e.second : -1 - (int)e.second.gap();
                std::printf(" %d:%d", x, y);
            }
            std::printf("\nkstruct %s %s\n", alignment.dot_bracket_structureA(false).c_str(),
                        alignment.dot_bracket_structureB(false).c_str());
            if (i == (size_t)o.kbest) break;
            size_t lenA = r.endA() - r.startA(), lenB = r.endB() - r.startB();
            AlignerRestriction r1(r), r2(r);
            if (lenA > lenB) {
                int split = (alignment.start_positions().first + alignment.end_positions().first) / 2;
                r1.set_endA(split);
                r2.set_startA(split);
            } else {
                int split = (alignment.start_positions().second + alignment.end_positions().second) / 2;
                r1.set_endB(split);
                r2.set_startB(split);
            }
            a->set_restriction(r1);
            infty_score_t s1 = norm ? a->normalized_align(o.normalized, false) : a->align();
            a->set_restriction(r2);
            infty_score_t s2 = norm ? a->normalized_align(o.normalized, false) : a->align();
            tasks.push(task_t(r1, s1));
            tasks.push(task_t(r2, s2));
            ++i;
        }
    }

    double best = 1e30;
    infty_score_t score;
    std::unique_ptr<Alignment> aln;
    for (int r = 0; r < std::max(1, o.repeat); ++r) {
        auto t0 = std::chrono::steady_clock::now();
        Aligner aligner(AlignerParams(
            AlignerParams::seqA(&seqA), AlignerParams::seqB(&seqB),
            AlignerParams::scoring(&scoring), AlignerParams::no_lonely_pairs(o.no_lonely_pairs),
            AlignerParams::struct_local(o.struct_local), AlignerParams::sequ_local(o.sequ_local),
            AlignerParams::free_endgaps(FreeEndgaps(o.free_endgaps)),
            AlignerParams::max_diff_am(o.max_diff_am), AlignerParams::max_diff_at_am(o.max_diff_at_am),
            AlignerParams::trace_controller(&tc), AlignerParams::stacking(stacking),
            AlignerParams::constraints(&anchors)));
        // src/locarna.cc:751-783: normalized and penalized alignment trace
        // inside their own calls
        if (o.normalized >= 0) {
            score = aligner.normalized_align(o.normalized, false);
        } else if (o.penalized >= 0) {
            score = aligner.penalized_align(o.penalized);
        } else {
            score = aligner.align();
            aligner.trace();
        }
        auto t1 = std::chrono::steady_clock::now();
        best = std::min(best, std::chrono::duration<double>(t1 - t0).count());
        aln = std::make_unique<Alignment>(aligner.get_alignment());
    }
    std::printf("score %ld\n", score_val(score));
    auto edges = aln->alignment_edges(false);
    std::printf("edges");
    for (auto &e : edges) {
        int a = e.first.is_pos() ? (int)(size_t)e.first : -1 - (int)e.first.gap();
        int b = e.second.is_pos() ? (int)(size_t)e.second : -1 - (int)e.second.gap();
        std::printf(" %d:%d", a, b);
    }
    std::printf("\nstructA %s\n", aln->dot_bracket_structureA(false).c_str());
    std::printf("structB %s\n", aln->dot_bracket_structureB(false).c_str());
    std::printf("align_seconds %.6f\n", best);
    return 0;
}
