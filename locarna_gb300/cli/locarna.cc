// locarna — the reference's pairwise alignment command line
// (src/locarna.cc:83-272 options, :398-785 flow, :890-935 output) on the
// GB300 engine: PP inputs are prepared by lcg_prepare_pairs (scoring, arc
// matches, sequence envelope on the GPU), aligned by lcg_align_pairs /
// lcg_align_kbest, and printed as the reference prints them (score line,
// CLUSTAL block output, --clustal / --stockholm files). Options keep the
// reference's names and defaults; options of the reference that this build
// does not implement (folding, MEA, consensus structures, ...) are refused
// with an error. Inputs must be PP files (the reference folds FASTA inputs
// with ViennaRNA, which is not part of this path).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/locarna_gb300.hpp"
#include "lcg_cli_opts.hh"
#include "lcg_output.hh"

using namespace lcg_cli;

namespace {

struct Clp {
    bool help = false, version = false, verbose = false, quiet = false;
    int indel = -150, indel_opening = -750, match = 50, mismatch = 0, unpaired_penalty = 0;
    int struct_weight = 200, tau = 50, exclusion = 0;
    std::string ribosum_file = "RIBOSUM85_60";
    bool use_ribosum = true;
    double exp_prob = 0;
    bool exp_prob_given = false;
    bool stacking = false, new_stacking = false;
    bool struct_local = false, sequ_local = false, struct_local_given = false, sequ_local_given = false;
    std::string free_endgaps = "----";
    bool normalized = false, penalized = false;
    int normalized_L = 0, position_penalty = 0;
    int width = 120;
    std::string clustal, stockholm;
    bool clustal_given = false, stockholm_given = false;
    bool local_output = false, local_file_output = false, pos_output = false, write_structure = false;
    double min_prob = 0.001, min_trace_probability = 1e-4;
    int max_diff_am = -1, max_diff = -1, max_diff_at_am = -1;
    bool subopt = false;
    int kbest_k = -1, subopt_threshold = -1000000;
    int temperature_alipf = 300;
    bool no_lonely_pairs = false, relaxed_anchors = false, extended_pf = false;
    int max_bp_span = -1;
    std::vector<std::string> files;
};

std::string read_file(const std::string &path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw locarna_gb300::failure("Cannot read input file " + path);
    std::stringstream ss;
    ss << f.rdbuf();
    return ss.str();
}

std::string score_str(int64_t s) { return s == LCG_NEG_INF ? std::string("-inf") : std::to_string(s); }

std::vector<Row> input_rows(lcg_prepared p, int side) {
    std::vector<Row> out;
    for (int k = 0;; ++k) {
        const char *seq = lcg_prepared_row(p, side, k), *name = lcg_prepared_row(p, side + 2, k);
        if (!seq) break;
        out.push_back({name ? name : "", seq});
    }
    return out;
}

// pos_output positions: the first / last edge ends that are positions
// (Alignment::start_positions / end_positions, alignment.cc:170-200)
std::pair<int, int> start_positions(const Edges &raw, int n, int m) {
    int a = n, b = m;
    for (const auto &e : raw)
        if (e.first > 0) { a = e.first; break; }
    for (const auto &e : raw)
        if (e.second > 0) { b = e.second; break; }
    return {a, b};
}
std::pair<int, int> end_positions(const Edges &raw) {
    int a = 0, b = 0;
    for (auto it = raw.rbegin(); it != raw.rend(); ++it)
        if (it->first > 0) { a = it->first; break; }
    for (auto it = raw.rbegin(); it != raw.rend(); ++it)
        if (it->second > 0) { b = it->second; break; }
    return {a, b};
}

struct Traced {
    Edges raw;
    std::vector<std::pair<std::pair<int, int>, std::pair<int, int>>> arcs;
};

Traced traced(const lcg_pair_tables &t, const locarna_gb300::Alignment &al) {
    Traced tr;
    tr.raw = al.edges;
    for (int k : al.traced_arcmatches) {
        const int a = t.am_arcs[2 * k], b = t.am_arcs[2 * k + 1];
        tr.arcs.push_back({{t.arcs_a[2 * a], t.arcs_a[2 * a + 1]}, {t.arcs_b[2 * b], t.arcs_b[2 * b + 1]}});
    }
    return tr;
}

// the #A<k> lines of input `side` (0 A, 1 B)
std::vector<std::string> input_anchors(lcg_prepared p, int side) {
    std::vector<std::string> out;
    for (int k = 0;; ++k) {
        const char *l = lcg_prepared_row(p, side + 4, k);
        if (!l) break;
        out.push_back(l);
    }
    return out;
}

// the consensus anchor lines the reference's MultipleAlignment of the
// alignment carries (multiple_alignment.cc:153-165)
std::vector<std::string> alignment_anchors(const lcg_pair_tables &t, lcg_prepared p, const Traced &tr,
                                           bool only_local) {
    return anchor_consensus(alignment_edges(tr.raw, t.len_a, t.len_b, only_local), input_anchors(p, 0),
                            input_anchors(p, 1));
}

std::vector<Row> alignment_rows(const lcg_pair_tables &t, lcg_prepared p, const Traced &tr, bool only_local,
                                bool with_structure) {
    const Edges edges = alignment_edges(tr.raw, t.len_a, t.len_b, only_local);
    std::vector<Row> rs = rows(edges, input_rows(p, 0), input_rows(p, 1));
    if (with_structure) {
        auto st = structure(edges, t.len_a, t.len_b, tr.arcs);
        rs.insert(rs.begin(), Row{"", st.first});
        rs.push_back(Row{"", st.second});
    }
    return rs;
}

int run(const Clp &c) {
    lcg_prep_opts po;
    lcg_prep_opts_default(&po);
    po.min_prob = c.min_prob;
    po.indel = c.indel;
    po.indel_opening = c.indel_opening;
    po.struct_weight = c.struct_weight;
    po.tau = c.tau;
    po.exclusion = c.exclusion;
    po.match = c.match;
    po.mismatch = c.mismatch;
    po.use_ribosum = c.use_ribosum;
    po.min_trace_probability = c.min_trace_probability;
    po.max_diff = c.max_diff;
    po.max_diff_am = c.max_diff_am;
    po.max_diff_at_am = c.max_diff_at_am;
    po.temperature_alipf = c.temperature_alipf;
    po.sequ_local = c.sequ_local;
    int fe = 0;
    for (int k = 0; k < 4 && k < (int)c.free_endgaps.size(); ++k)
        if (c.free_endgaps[k] == '+') fe |= 1 << k;
    po.free_endgaps = fe;
    po.exp_prob = c.exp_prob_given ? c.exp_prob : -1.0;
    po.stacking = c.stacking;
    po.new_stacking = c.new_stacking;
    po.unpaired_penalty = c.unpaired_penalty;
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

    locarna_gb300::AlignerParams ap;
    ap.with_tables(&t).with_struct_local(c.struct_local).with_sequ_local(c.sequ_local)
        .with_free_endgaps(c.free_endgaps).with_no_lonely_pairs(c.no_lonely_pairs);
    if (c.normalized) ap.with_normalized(c.normalized_L);
    if (c.penalized) ap.with_penalized(c.position_penalty);
    locarna_gb300::Aligner aligner(ap, eng);

    if (c.subopt) {
        // Aligner::suboptimal's printing (aligner.cc:1447-1463)
        auto hits = aligner.suboptimal(c.kbest_k, c.subopt_threshold);
        for (const auto &h : hits) {
            const Traced tr = traced(t, h.second);
            if (c.pos_output) {
                auto s = start_positions(tr.raw, t.len_a, t.len_b);
                auto e = end_positions(tr.raw);
                std::cout << "HIT " << score_str(h.first) << " " << s.first << " " << s.first << " " << e.second
                          << " " << e.second << " " << std::endl;
            } else {
                std::cout << "Score: " << score_str(h.first) << std::endl;
                write_blocks(std::cout, alignment_rows(t, prep, tr, true, false), 120, false,
                             alignment_anchors(t, prep, tr, true));
                std::cout << std::endl << std::endl;
            }
        }
        return 0;
    }

    const int64_t score = aligner.align();
    if (!c.quiet) std::cout << "Score: " << score_str(score) << std::endl << std::endl;
    const Traced tr = traced(t, aligner.get_alignment());
    int rc = 0;
    if (c.clustal_given) {
        std::ofstream out(c.clustal);
        if (out.good()) {
            out << "CLUSTAL W --- " << LCG_CLI_PACKAGE_STRING;
            if (input_rows(prep, 0).size() == 1 && input_rows(prep, 1).size() == 1)
                out << " --- Score: " << score_str(score);
            out << std::endl << std::endl;
            write_blocks(out, alignment_rows(t, prep, tr, c.local_file_output, c.write_structure), c.width, false,
                         alignment_anchors(t, prep, tr, c.local_file_output));
        } else {
            std::cerr << "ERROR: Cannot write to " << c.clustal << "." << std::endl;
            rc = -1;
        }
    }
    if (c.stockholm_given) {
        std::ofstream out(c.stockholm);
        if (out.good()) {
            const auto rs = alignment_rows(t, prep, tr, c.local_file_output, false);
            out << "# STOCKHOLM 1.0" << std::endl;
            out << "#=GF CC Generated by " << LCG_CLI_PACKAGE_STRING << std::endl;
            out << "#=GF SQ " << rs.size() << std::endl << std::endl;
            write_blocks(out, rs, c.width, true, alignment_anchors(t, prep, tr, c.local_file_output));
        } else {
            std::cerr << "ERROR: Cannot write to " << c.stockholm << "." << std::endl;
            rc = -1;
        }
    }
    if (c.pos_output) {
        auto s = start_positions(tr.raw, t.len_a, t.len_b);
        auto e = end_positions(tr.raw);
        std::cout << "HIT " << score_str(score) << " " << s.first << " " << s.second << " " << e.first << " "
                  << e.second << " " << std::endl
                  << std::endl;
    }
    if ((!c.pos_output && !c.quiet) || c.local_output) {
        if (c.pos_output) {
            auto s = start_positions(tr.raw, t.len_a, t.len_b);
            std::cout << "\t+" << s.first << std::endl << "\t+" << s.second << std::endl << std::endl << std::endl;
        }
        write_blocks(std::cout, alignment_rows(t, prep, tr, c.local_output, c.write_structure), c.width, false,
                     alignment_anchors(t, prep, tr, c.local_output));
        if (c.pos_output) {
            auto e = end_positions(tr.raw);
            std::cout << std::endl << "\t+" << e.first << std::endl << "\t+" << e.second << std::endl << std::endl;
        }
    }
    if (!c.quiet) std::cout << std::endl;
    return rc;
}

}  // namespace

int main(int argc, char **argv) {
    Clp c;
    OptionTable tab("locarna", "pairwise sequence-structure alignment of two RNAs (PP inputs)");
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
    tab.integer("unpaired-penalty", 0, &c.unpaired_penalty);
    tab.integer("struct-weight", 's', &c.struct_weight);
    tab.real("exp-prob", 'e', &c.exp_prob, &c.exp_prob_given);
    tab.integer("tau", 't', &c.tau);
    tab.integer("exclusion", 'E', &c.exclusion);
    tab.flag("stacking", 0, &c.stacking);
    tab.flag("new-stacking", 0, &c.new_stacking);
    tab.boolean("struct-local", 0, &c.struct_local, &c.struct_local_given);
    tab.boolean("sequ-local", 0, &c.sequ_local, &c.sequ_local_given);
    tab.string("free-endgaps", 0, &c.free_endgaps);
    tab.integer("normalized", 0, &c.normalized_L, &c.normalized);
    tab.integer("penalized", 0, &c.position_penalty, &c.penalized);
    tab.integer("width", 'w', &c.width);
    tab.string("clustal", 0, &c.clustal, &c.clustal_given);
    tab.string("stockholm", 0, &c.stockholm, &c.stockholm_given);
    tab.flag("local-output", 'L', &c.local_output);
    tab.flag("local-file-output", 0, &c.local_file_output);
    tab.flag("pos-output", 'P', &c.pos_output);
    tab.flag("write-structure", 0, &c.write_structure);
    tab.real("min-prob", 'p', &c.min_prob);
    tab.integer("max-diff-am", 'D', &c.max_diff_am);
    tab.integer("max-diff", 'd', &c.max_diff);
    tab.integer("max-diff-at-am", 0, &c.max_diff_at_am);
    tab.real("min-trace-probability", 0, &c.min_trace_probability);
    tab.integer("kbest", 0, &c.kbest_k, &c.subopt);
    tab.integer("better", 0, &c.subopt_threshold, &c.subopt);
    tab.integer("temperature-alipf", 0, &c.temperature_alipf);
    tab.flag("noLP", 0, &c.no_lonely_pairs);
    tab.integer("maxBPspan", 0, &c.max_bp_span);
    tab.flag("relaxed-anchors", 0, &c.relaxed_anchors);
    // the envelope in long double is locarna's only mode without
    // --quad-pf (src/locarna.cc:384 sets extended_pf unconditionally)
    tab.flag("extended-pf", 0, &c.extended_pf);
    // options of the reference outside this build's scope
    for (const char *o : {"galaxy-xml", "quad-pf", "pp", "alifold-consensus-dp", "consensus-structure",
                          "consensus-gamma", "score-components", "stopwatch", "max-bps-length-ratio", "max-diff-aln",
                          "max-diff-pw-aln", "max-diff-relax", "mea-alignment", "match-prob-method", "probcons-file",
                          "pf-struct-weight", "mea-gapcost", "mea-alpha", "mea-beta", "mea-gamma", "probability-scale",
                          "write-match-probs", "write-trace-probs", "read-match-probs", "write-arcmatch-scores",
                          "read-arcmatch-scores", "read-arcmatch-probs", "ribofit"})
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
        std::cout << "locarna (" << LCG_CLI_PACKAGE_STRING << ")" << std::endl;
        return 0;
    }
    if (c.files.size() != 2) {
        std::cerr << "Two input files are required." << std::endl << tab.usage();
        return -1;
    }
    // the reference's checks (src/locarna.cc:364-446)
    if (c.struct_weight < 0) {
        std::cerr << "Structure weight must be greater equal 0." << std::endl;
        return -1;
    }
    if (c.normalized && c.penalized) {
        std::cerr << "One cannot specify penalized and normalized simultaneously." << std::endl;
        return -1;
    }
    if (c.sequ_local && c.free_endgaps != "----") {
        std::cerr << "Free endgaps cannot be combined with local alignment." << std::endl;
        return -1;
    }
    if (c.normalized) {
        if (!c.sequ_local_given) {
            c.sequ_local = true;
        } else if (!c.sequ_local) {
            std::cerr << "ERROR: Cannot run normalized alignment without --sequ_local on." << std::endl;
            return -1;
        }
        if (c.struct_local_given && c.struct_local) {
            std::cerr << "ERROR: Normalized structure local alignment not supported." << std::endl;
            return -1;
        }
        c.struct_local = false;
    }
    // restrictions of this build, checked before any work
    const char *why = nullptr;
    if (c.ribosum_file != "RIBOSUM85_60") why = "--ribosum-file: only the built-in RIBOSUM85_60 is available";
    else if (c.max_bp_span != -1) why = "--maxBPspan applies to folding, which this build does not do";
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
