// locarna_p — the reference's partition-function command line
// (src/locarna_p.cc:40-201 options, :466-531 flow) on the GB300 engine: PP
// inputs prepared by lcg_prepare_pairs (envelope 1e-5 in double, as locarna_p
// computes it), the inside pass (lcg_pf_forward) and its adjoint
// (lcg_pf_backward) in double, the partition function printed, and the
// arc-match / base-match probabilities written in the reference's format
// (AlignerP::write_arcmatch_probabilities / write_basematch_probabilities,
// aligner_p.icc:1404-1435) with its --min-am-prob / --min-bm-prob semantics.
// Options of the reference that this build does not implement are refused.
#include <cmath>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/locarna_gb300.hpp"
#include "lcg_cli_opts.hh"

using namespace lcg_cli;

namespace {

struct Clp {
    bool help = false, version = false, verbose = false, quiet = false;
    int indel = -150, indel_opening = -750, match = 50, mismatch = 0, struct_weight = 200, tau = 50;
    std::string ribosum_file = "RIBOSUM85_60";
    bool use_ribosum = true;
    double exp_prob = 0;
    bool exp_prob_given = false;
    int temperature_alipf = 300;
    double pf_scale = 1.0;
    bool write_am = false, write_bm = false, include_am_in_bm = false;
    std::string am_file, bm_file;
    double min_am_prob = 0.001, min_bm_prob = 0.001;
    double min_prob = 0.001, min_trace_probability = 1e-5;
    int max_diff_am = -1, max_diff = -1, max_diff_at_am = -1, max_bp_span = -1;
    bool relaxed_anchors = false;
    std::vector<std::string> files;
};

std::string read_file(const std::string &path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw locarna_gb300::failure("Cannot read input file " + path);
    std::stringstream ss;
    ss << f.rdbuf();
    return ss.str();
}

int run(const Clp &c) {
    lcg_prep_opts po;
    lcg_prep_opts_default(&po);
    po.min_prob = c.min_prob;
    po.indel = c.indel;
    po.indel_opening = c.indel_opening;
    po.struct_weight = c.struct_weight;
    po.tau = c.tau;
    po.match = c.match;
    po.mismatch = c.mismatch;
    po.use_ribosum = c.use_ribosum;
    po.min_trace_probability = c.min_trace_probability;
    po.max_diff = c.max_diff;
    po.max_diff_am = c.max_diff_am;
    po.max_diff_at_am = c.max_diff_at_am;
    po.temperature_alipf = c.temperature_alipf;
    po.pf_precision = 0;  // locarna_p's envelope is computed in pf_score_t = double
    po.exp_prob = c.exp_prob_given ? c.exp_prob : -1.0;
    po.relaxed_anchors = c.relaxed_anchors;

    const std::string pa = read_file(c.files[0]), pb = read_file(c.files[1]);
    locarna_gb300::Engine eng(0);
    const char *ta[1] = {pa.c_str()}, *tb[1] = {pb.c_str()};
    lcg_prepared prep = nullptr;
    locarna_gb300::check(lcg_prepare_pairs(eng.get(), ta, tb, 1, &po, &prep, nullptr));
    struct Free {
        lcg_prepared p;
        ~Free() { lcg_prepared_free(p); }
    } free_prep{prep};
    lcg_pair_tables t;
    locarna_gb300::check(lcg_prepared_tables(prep, &t));
    if (t.match_lo) throw locarna_gb300::failure("LocARNA-P does not take anchor constraints");

    lcg_pf_opts o;
    lcg_pf_opts_default(&o);
    o.temperature = c.temperature_alipf;
    o.pf_scale = c.pf_scale;
    o.precision = 64;
    o.min_am_prob = c.min_am_prob;
    o.min_bm_prob = c.min_bm_prob;
    o.gap_gradients = 0;  // probabilities only
    if (c.verbose) std::cout << "Run inside algorithm." << std::endl;
    double log_z = 0;
    locarna_gb300::check(lcg_pf_forward(eng.get(), &t, 1, &o, nullptr, &log_z));
    if (!c.quiet) std::cout << "Partition function: " << std::exp(log_z) << std::endl;
    if (c.verbose) std::cout << "Run outside algorithm." << std::endl;
    std::vector<double> am((size_t)std::max(t.num_arcmatches, 1)), bm((size_t)(t.len_a + 1) * (t.len_b + 1));
    lcg_pf_result r{};
    r.am_prob = am.data();
    r.bm_prob = bm.data();
    locarna_gb300::check(lcg_pf_backward(eng.get(), nullptr, &r));
    if (c.verbose) std::cout << "Compute probabilities." << std::endl;
    if (c.write_am) {
        std::ofstream out(c.am_file);
        if (!out.good()) {
            std::cerr << "Cannot write to " << c.am_file << "! Exit." << std::endl;
            return -1;
        }
        for (int k = 0; k < t.num_arcmatches; ++k) {
            if (!(am[k] >= c.min_am_prob)) continue;
            const int a = t.am_arcs[2 * k], b = t.am_arcs[2 * k + 1];
            out << t.arcs_a[2 * a] << " " << t.arcs_a[2 * a + 1] << " " << t.arcs_b[2 * b] << " "
                << t.arcs_b[2 * b + 1] << " " << am[k] << std::endl;
        }
    }
    if (c.include_am_in_bm) {
        // compute_basematch_probabilities(true): the arc-match probabilities
        // added at both arc ends (aligner_p.icc:1382-1398)
        const int m1 = t.len_b + 1;
        for (int k = 0; k < t.num_arcmatches; ++k) {
            const int a = t.am_arcs[2 * k], b = t.am_arcs[2 * k + 1];
            bm[(size_t)t.arcs_a[2 * a] * m1 + t.arcs_b[2 * b]] += am[k];
            bm[(size_t)t.arcs_a[2 * a + 1] * m1 + t.arcs_b[2 * b + 1]] += am[k];
        }
    }
    if (c.write_bm) {
        std::ofstream out(c.bm_file);
        if (!out.good()) {
            std::cerr << "Cannot write to " << c.bm_file << "! Exit." << std::endl;
            return -1;
        }
        for (int i = 1; i <= t.len_a; ++i)
            for (int j = 1; j <= t.len_b; ++j) {
                const double p = bm[(size_t)i * (t.len_b + 1) + j];
                if (p >= c.min_bm_prob) out << i << " " << j << " " << p << std::endl;
            }
    }
    return 0;
}

}  // namespace

int main(int argc, char **argv) {
    Clp c;
    OptionTable tab("locarna_p", "partition function and match probabilities of two RNAs (PP inputs)");
    tab.flag("help", 'h', &c.help);
    tab.flag("version", 'V', &c.version);
    tab.flag("verbose", 'v', &c.verbose);
    tab.flag("quiet", 'q', &c.quiet);
    tab.integer("indel", 'i', &c.indel);
    tab.integer("indel-opening", 0, &c.indel_opening);
    tab.string("ribosum-file", 0, &c.ribosum_file);
    tab.boolean("use-ribosum", 0, &c.use_ribosum);
    tab.integer("match", 'm', &c.match);
    tab.integer("mismatch", 'M', &c.mismatch);
    tab.integer("struct-weight", 's', &c.struct_weight);
    tab.real("exp-prob", 'e', &c.exp_prob, &c.exp_prob_given);
    tab.integer("tau", 't', &c.tau);
    tab.integer("temperature-alipf", 0, &c.temperature_alipf);
    tab.real("pf-scale", 0, &c.pf_scale);
    tab.string("write-arcmatch-probs", 0, &c.am_file, &c.write_am);
    tab.string("write-basematch-probs", 0, &c.bm_file, &c.write_bm);
    tab.real("min-am-prob", 'a', &c.min_am_prob);
    tab.real("min-bm-prob", 'b', &c.min_bm_prob);
    tab.flag("include-am-in-bm", 0, &c.include_am_in_bm);
    tab.real("min-prob", 'p', &c.min_prob);
    tab.integer("max-diff-am", 'D', &c.max_diff_am);
    tab.integer("max-diff", 'd', &c.max_diff);
    tab.integer("max-diff-at-am", 0, &c.max_diff_at_am);
    tab.real("min-trace-probability", 0, &c.min_trace_probability);
    tab.integer("maxBPspan", 0, &c.max_bp_span);
    tab.flag("relaxed-anchors", 0, &c.relaxed_anchors);
    for (const char *o : {"extended-pf", "quad-pf", "stopwatch", "max-bps-length-ratio", "max-diff-aln",
                          "max-diff-pw-aln", "max-diff-relax", "fragment-match-probs", "ribofit"})
        tab.unsupported(o);
    std::string err;
    if (!tab.parse(argc, argv, c.files, err)) {
        std::cerr << err << std::endl << tab.usage();
        return -1;
    }
    if (c.help) {
        std::cout << tab.usage();
        return 0;
    }
    if (c.version) {
        std::cout << "locarna_p (" << LCG_CLI_PACKAGE_STRING << ")" << std::endl;
        return 0;
    }
    if (c.files.size() != 2) {
        std::cerr << "Two input files are required." << std::endl << tab.usage();
        return -1;
    }
    const char *why = nullptr;
    if (c.ribosum_file != "RIBOSUM85_60") why = "--ribosum-file: only the built-in RIBOSUM85_60 is available";
    else if (c.max_bp_span != -1) why = "--maxBPspan applies to folding, which this build does not do";
    else if (!(c.pf_scale > 0)) why = "--pf-scale must be positive";
    if (why) {
        std::cerr << "ERROR: " << why << std::endl;
        return -1;
    }
    try {
        return run(c);
    } catch (const std::exception &e) {
        std::cerr << "ERROR: " << e.what() << std::endl;
        return -1;
    }
}
