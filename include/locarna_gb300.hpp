/*
 * locarna_gb300.hpp — C++ facade over the C ABI of locarna_gb300.h.
 *
 * Mirrors the shape of the reference's aligner classes so that a caller of
 * LocARNA::Aligner / LocARNA::AlignerP can switch with few changes:
 *   Aligner  (src/LocARNA/aligner.hh:67-189):     align(), trace(), get_alignment()
 *   AlignerP (src/LocARNA/aligner_p.hh:53-622):   align_inside(), align_outside(),
 *            compute_arcmatch_probabilities(), compute_basematch_probabilities(bool)
 *   AlignerParams / AlignerPParams (aligner_params.hh:49-156): the options
 * Errors become exceptions of type locarna_gb300::failure, as the reference
 * raises LocARNA::failure (aux.hh:160). The tables stand for the reference's
 * Sequence / Scoring / TraceController / AnchorConstraints objects
 * (lcg_prepare_pair builds them from PP files, as src/locarna.cc does).
 * Header-only; link against liblocarna_gb300.so.
 */
#ifndef LOCARNA_GB300_HPP
#define LOCARNA_GB300_HPP

#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "locarna_gb300.h"

namespace locarna_gb300 {

class failure : public std::runtime_error {
public:
    explicit failure(const std::string &msg) : std::runtime_error(msg) {}
};

inline void check(lcg_status s) {
    if (s != LCG_OK) throw failure(std::string("locarna_gb300: ") + lcg_last_error());
}

// One GPU engine (device buffers and a stream); share it between aligners of
// one host thread.
class Engine {
    lcg_engine e_ = nullptr;

public:
    explicit Engine(int device = 0, void *stream = nullptr) {
        // the structures of this header must be the library's
        if (lcg_abi_version() != LCG_ABI_VERSION)
            throw failure("locarna_gb300: the library's ABI version differs from the header's");
        check(lcg_engine_create(device, stream, &e_));
    }
    ~Engine() {
        if (e_) lcg_engine_destroy(e_);
    }
    Engine(const Engine &) = delete;
    Engine &operator=(const Engine &) = delete;
    lcg_engine get() const { return e_; }
    // pairs per chunk of the batched call's host/device pipeline (0: automatic)
    void set_chunk_pairs(int n) { check(lcg_engine_set_chunk_pairs(e_, n)); }
};

// Tables of one pair built from two PP 2.0 texts (lcg_prepare_pair).
class PreparedPair {
    lcg_prepared p_ = nullptr;

public:
    PreparedPair(const std::string &pp_a, const std::string &pp_b, const lcg_prep_opts *opts = nullptr) {
        check(lcg_prepare_pair(pp_a.c_str(), pp_b.c_str(), opts, &p_));
    }
    ~PreparedPair() {
        if (p_) lcg_prepared_free(p_);
    }
    PreparedPair(const PreparedPair &) = delete;
    PreparedPair &operator=(const PreparedPair &) = delete;
    lcg_pair_tables tables() const {
        lcg_pair_tables t;
        check(lcg_prepared_tables(p_, &t));
        return t;
    }
    lcg_pf_grad_spec grad_spec() const {
        lcg_pf_grad_spec g;
        check(lcg_prepared_grad_spec(p_, &g));
        return g;
    }
    std::string sequence(int which) const { return lcg_prepared_sequence(p_, which); }
};

// AlignerParams (aligner_params.hh:49-64): the tables plus the mode flags.
struct AlignerParams {
    const lcg_pair_tables *tables = nullptr;  // seqA, seqB, scoring, trace_controller, constraints
    bool struct_local = false;
    bool sequ_local = false;
    std::string free_endgaps = "----";  // FreeEndgaps("abcd")
    bool do_trace = true;               // DO_TRACE
    bool no_lonely_pairs = false;       // no_lonely_pairs (locarna --noLP)
    int normalized = -1;                // locarna --normalized L (-1 = off)
    int penalized = -1;                 // locarna --penalized PP (-1 = off)
    AlignerParams &with_tables(const lcg_pair_tables *t) { tables = t; return *this; }
    AlignerParams &with_struct_local(bool v) { struct_local = v; return *this; }
    AlignerParams &with_sequ_local(bool v) { sequ_local = v; return *this; }
    AlignerParams &with_free_endgaps(const std::string &v) { free_endgaps = v; return *this; }
    AlignerParams &with_do_trace(bool v) { do_trace = v; return *this; }
    AlignerParams &with_no_lonely_pairs(bool v) { no_lonely_pairs = v; return *this; }
    AlignerParams &with_normalized(int L) { normalized = L; return *this; }
    AlignerParams &with_penalized(int pp) { penalized = pp; return *this; }
    lcg_align_opts opts() const {
        int fe = 0;
        for (int k = 0; k < 4 && k < (int)free_endgaps.size(); ++k)
            if (free_endgaps[k] == '+') fe |= 1 << k;
        return lcg_align_opts{struct_local, sequ_local, fe, do_trace, no_lonely_pairs,
                              normalized >= 0, normalized >= 0 ? normalized : 0,
                              penalized >= 0, penalized >= 0 ? penalized : 0};
    }
};

// The traced alignment: the edges in the order Alignment::append receives
// them ((pos_a, pos_b), -1 for a gap) and the traced arc matches.
struct Alignment {
    std::vector<std::pair<int, int>> edges;
    std::vector<int> traced_arcmatches;
    int max_i = 0, max_j = 0, min_i = 1, min_j = 1;
};

class Aligner {
    Engine *eng_;
    AlignerParams ap_;
    Alignment alignment_;
    int64_t score_ = LCG_NEG_INF;
    bool aligned_ = false;

public:
    Aligner(const AlignerParams &ap, Engine &engine) : eng_(&engine), ap_(ap) {
        if (!ap_.tables) throw failure("locarna_gb300: AlignerParams without tables");
    }
    // align(): the optimal score; LCG_NEG_INF for negative infinity. With
    // do_trace the traceback runs in the same launch.
    int64_t align() {
        const lcg_pair_tables &t = *ap_.tables;
        std::vector<int32_t> edges(2 * (size_t)(t.len_a + t.len_b) + 2), tam((size_t)std::min(t.len_a, t.len_b) + 1);
        lcg_align_result r{};
        r.edges = edges.data();
        r.traced_am = tam.data();
        const lcg_align_opts o = ap_.opts();
        check(lcg_align_pairs(eng_->get(), &t, 1, &o, &r));
        score_ = r.score;
        alignment_ = Alignment{};
        alignment_.max_i = r.max_i;
        alignment_.max_j = r.max_j;
        alignment_.min_i = r.min_i;
        alignment_.min_j = r.min_j;
        for (int k = 0; k < r.num_edges; ++k) alignment_.edges.emplace_back(edges[2 * k], edges[2 * k + 1]);
        alignment_.traced_arcmatches.assign(tam.begin(), tam.begin() + r.num_traced_am);
        aligned_ = true;
        return score_;
    }
    // trace(): the traceback of align() (computed by the same call)
    void trace() {
        if (!aligned_) align();
        if (!ap_.do_trace) throw failure("locarna_gb300: trace() needs do_trace");
    }
    // Aligner::normalized_align(L) (aligner.cc:1521-1588): the normalized
    // score; the alignment is traced by the same call
    int64_t normalized_align(int L) {
        AlignerParams keep = ap_;
        ap_.normalized = L;
        ap_.penalized = -1;
        int64_t s = align();
        ap_ = keep;
        return s;
    }
    // Aligner::penalized_align(PP) (aligner.cc:1590-1617): the penalised
    // score; the alignment is traced by the same call
    int64_t penalized_align(int position_penalty) {
        AlignerParams keep = ap_;
        ap_.penalized = position_penalty;
        ap_.normalized = -1;
        int64_t s = align();
        ap_ = keep;
        return s;
    }
    // Aligner::suboptimal (aligner.cc:1384-1512): up to k alignments by
    // interval splitting with their scores (normalized when the parameters
    // ask for it), ending below threshold + 1
    std::vector<std::pair<int64_t, Alignment>> suboptimal(int k, int64_t threshold) {
        const lcg_pair_tables &t = *ap_.tables;
        const size_t ne = 2 * (size_t)(t.len_a + t.len_b) + 2, nt = (size_t)std::min(t.len_a, t.len_b) + 1;
        std::vector<int32_t> edges(ne * (size_t)k), tam(nt * (size_t)k);
        std::vector<lcg_align_result> r((size_t)k);
        for (int h = 0; h < k; ++h) {
            r[h] = lcg_align_result{};
            r[h].edges = edges.data() + ne * h;
            r[h].traced_am = tam.data() + nt * h;
        }
        const lcg_align_opts o = ap_.opts();
        int32_t hits = 0;
        check(lcg_align_kbest(eng_->get(), &t, 1, &o, k, threshold, r.data(), &hits));
        std::vector<std::pair<int64_t, Alignment>> out;
        for (int h = 0; h < hits; ++h) {
            Alignment a;
            a.max_i = r[h].max_i;
            a.max_j = r[h].max_j;
            a.min_i = r[h].min_i;
            a.min_j = r[h].min_j;
            for (int q = 0; q < r[h].num_edges; ++q)
                a.edges.emplace_back(r[h].edges[2 * q], r[h].edges[2 * q + 1]);
            a.traced_arcmatches.assign(r[h].traced_am, r[h].traced_am + r[h].num_traced_am);
            out.emplace_back(r[h].score, std::move(a));
        }
        return out;
    }
    const Alignment &get_alignment() const { return alignment_; }
    static bool is_neg_inf(int64_t score) { return score == LCG_NEG_INF; }
};

// AlignerPParams (aligner_params.hh:122-156)
struct AlignerPParams {
    const lcg_pair_tables *tables = nullptr;
    const lcg_pf_grad_spec *grad_spec = nullptr;  // for the parameter gradients
    double temperature = 300.0;                   // temperature_alipf
    double pf_scale = 1.0;
    int precision = 64;                           // 64, or 32 with per-position scaling
};

class AlignerP {
    Engine *eng_;
    AlignerPParams ap_;
    double log_z_ = 0.0;
    std::vector<double> am_, bm_;
    lcg_pf_result res_{};
    bool inside_ = false, outside_ = false;

public:
    AlignerP(const AlignerPParams &ap, Engine &engine) : eng_(&engine), ap_(ap) {
        if (!ap_.tables) throw failure("locarna_gb300: AlignerPParams without tables");
    }
    // align_inside(): the partition function (as log Z: Z itself overflows
    // double for long sequences)
    double align_inside() {
        lcg_pf_opts o;
        lcg_pf_opts_default(&o);
        o.temperature = ap_.temperature;
        o.pf_scale = ap_.pf_scale;
        o.precision = ap_.precision;
        check(lcg_pf_forward(eng_->get(), ap_.tables, 1, &o, ap_.grad_spec, &log_z_));
        inside_ = true;
        outside_ = false;
        return log_z_;
    }
    // align_outside(): the adjoint pass, which yields every probability and
    // the derivatives of log Z
    void align_outside() {
        if (!inside_) throw failure("locarna_gb300: align_outside() needs align_inside()");
        am_.assign((size_t)std::max(ap_.tables->num_arcmatches, 1), 0.0);
        bm_.assign((size_t)(ap_.tables->len_a + 1) * (ap_.tables->len_b + 1), 0.0);
        res_ = lcg_pf_result{};
        res_.am_prob = am_.data();
        res_.bm_prob = bm_.data();
        check(lcg_pf_backward(eng_->get(), ap_.grad_spec, &res_));
        outside_ = true;
        inside_ = false;
    }
    // arc-match probabilities, reference arc-match order
    const std::vector<double> &compute_arcmatch_probabilities() {
        if (!outside_) align_outside();
        am_.resize((size_t)ap_.tables->num_arcmatches);
        return am_;
    }
    // base-match probabilities, (len_a+1) x (len_b+1) row-major; with
    // include_am, the arc-match probabilities are added at both arc ends
    // (compute_basematch_probabilities(true), aligner_p.icc:1382-1398)
    std::vector<double> compute_basematch_probabilities(bool include_am = false) {
        if (!outside_) align_outside();
        std::vector<double> bm = bm_;
        if (include_am) {
            const lcg_pair_tables &t = *ap_.tables;
            const int m1 = t.len_b + 1;
            for (int k = 0; k < t.num_arcmatches; ++k) {
                const int a = t.am_arcs[2 * k], b = t.am_arcs[2 * k + 1];
                bm[(size_t)t.arcs_a[2 * a] * m1 + t.arcs_b[2 * b]] += am_[k];
                bm[(size_t)t.arcs_a[2 * a + 1] * m1 + t.arcs_b[2 * b + 1]] += am_[k];
            }
        }
        return bm;
    }
    const lcg_pf_result &gradients() const { return res_; }
    double log_z() const { return log_z_; }
};

}  // namespace locarna_gb300

#endif  // LOCARNA_GB300_HPP
