// Per-pair host preparation shared by the entry points of engine.cu and
// noalloc.cu: validation of the prepared tables and the derived index
// structures the kernels read (band offsets, candidate lists by right-end
// cell, left-end groups in dependency order, D-write lists).
#pragma once
#include <algorithm>
#include <cstdlib>
#include <atomic>
#include <string>
#include <thread>
#include <vector>

#include "../../include/locarna_gb300.h"
#include "lcg_device.cuh"

namespace lcg_host {

struct Prep {
    int n = 0, m = 0;
    int flags = 0, fe = 0;
    int bandcells = 0;
    std::vector<int> min_col, max_col, bandoff;  // n+2
    std::vector<int4> rowinfo;                   // n+2
    int maxband = 0;
    int span = 2;  // max over i of max_col[i+1] - min_col[i] + 3 (ring rows of the kernels)
    std::vector<int> cre_start;                  // bandcells+1
    std::vector<int> cre;                        // 4 per entry: D position, a.l-1, b.l-1, am
    std::vector<int> crow;                       // 2 per entry by row a.r, a.l desc, b.l desc:
                                                 //   (a.l-1) | (b.l-1) << 16, b.r
    std::vector<int> rowarc;                     // 2 per row 0..n+1: [start, end) in crow
    std::vector<int> am_pos;                     // per am: its crow position = D index (-1: right ends off the band)
    int num_pos = 0;                             // crow entries = D entries
    std::vector<int> am_ends;                    // 4 per am
    std::vector<int> Dinit;                      // per D position
    // sigma as a class table when rows and columns fall into <= 16 classes
    // each (single sequences: one class per base): sigma(i,j) =
    // scls[rcls[i]*16 + ccls[j]]
    bool use_cls = false;
    std::vector<int> scls, rcls, ccls;
    std::vector<int> gbc;  // m+1: gapB(j) * 16 + sigma column class (0 without classes)
    std::vector<lcg::GroupItem> groups;          // pair field filled later
    std::vector<int4> dw;                        // dw_start relative to this pair
    std::vector<int2> dwn;                       // no lonely pairs / stacking: parallel to dw (PairDev::dwn)
    std::vector<int2> inner;                     // no lonely pairs / stacking: per am (PairDev::inner)
    std::vector<int> sscore;                     // stacking: per am (PairDev::am_sscore)
    int rows_max = 0, width_max = 0;             // over groups
    // kept group rectangles: (ar-al) x (br-bl) ints per group, in group order
    // (GroupItem::rect_off, pitch br - bl); per arc match its group's
    // (rect_off, pitch) or (-1, 0); rect_cells = -1: too large to keep
    long long rect_cells = 0;
    std::vector<int2> am_rect;
    int token_cap = 0, tq_cap = 0;
    long long cells = 0;                         // M cells of all groups + top level
    std::string err;
    lcg_status code = LCG_OK;
};

// Validate one pair's tables and build its derived structures; on error
// p.code / p.err describe it.
lcg_status prep_pair(const lcg_pair_tables &t, const lcg_align_opts &o, Prep &p);

void set_error(const std::string &msg);

// the two stages of lcg_prepare_pairs (host_prep.cpp): inputs, bands and
// envelopes of every pair; then the tables of pairs [q0, q0 + nq)
struct StagedBatch;
// first: the pairs whose GPU envelopes are finished before it returns; the
// others' are enqueued and finished by the first finish_tables that needs
// them. host_envelopes: the host-path envelopes so far (batch_host_envelopes
// gives the final count).
lcg_status stage_batch(lcg_engine eng, const char *const *pp_a, const char *const *pp_b, int32_t npairs,
                       const lcg_prep_opts *opts, StagedBatch **out, int32_t *host_envelopes, int32_t first);
int batch_host_envelopes(const StagedBatch *B);
lcg_status finish_tables(StagedBatch *B, int q0, int nq, lcg_prepared *out);
void free_batch(StagedBatch *B);

// ring size of the kernels' shared-memory rows for a set of pairs: the
// smallest multiple of 32 >= every pair's span
inline int ring_size(int span) { return (std::max(span, 32) + 31) / 32 * 32; }

// Bytes of per-pair tables one wave of pairs in the work queue may keep hot
// (default 8 MB of the 126 MB L2); LCG_WAVE_MB overrides it for tuning runs
// (0 = one wave).
inline double wave_budget_bytes() {
    const char *v = std::getenv("LCG_WAVE_MB");
    const double mb = v ? std::atof(v) : 8.0;
    return (mb > 0 ? mb : 1e9) * 1048576.0;
}

// Work-queue order of the groups of a batch: pairs in waves whose tables
// (bytes(q)) fit wave_budget_bytes(); inside a wave, the pairs' lists are
// interleaved by progress, quantised to 4096 steps; each pair's own order is
// kept. Writes (pair, group index) in queue order to out[0 .. total); one
// counting sort per wave, waves in parallel.
template <typename BytesOf, typename ParallelFor>
void queue_order(const std::vector<size_t> &ngroups, BytesOf bytes, int2 *out, ParallelFor pfor,
                 double budget_bytes = 0.0) {
    const int npairs = (int)ngroups.size();
    constexpr size_t NB = 4096;
    const double budget = budget_bytes > 0.0 ? budget_bytes : wave_budget_bytes();
    std::vector<int> wave_first;  // first pair of each wave
    std::vector<size_t> wave_off;  // first output slot of each wave
    double acc = 0.0;
    size_t items = 0;
    for (int q = 0; q < npairs; ++q) {
        const double fp = bytes(q);
        if (q == 0 || (acc > 0.0 && acc + fp > budget)) {
            wave_first.push_back(q);
            wave_off.push_back(items);
            acc = 0.0;
        }
        acc += fp;
        items += ngroups[q];
    }
    wave_first.push_back(npairs);
    const int nw = (int)wave_first.size() - 1;
    pfor(nw, [&](int w) {
        std::vector<size_t> start(NB + 1, 0);
        auto key = [&](int q, size_t g) { return ((g + 1) * NB - 1) / ngroups[q]; };  // nondecreasing in g
        for (int q = wave_first[w]; q < wave_first[w + 1]; ++q)
            for (size_t g = 0; g < ngroups[q]; ++g) ++start[key(q, g) + 1];
        for (size_t k = 0; k < NB; ++k) start[k + 1] += start[k];
        int2 *o = out + wave_off[w];
        for (int q = wave_first[w]; q < wave_first[w + 1]; ++q)
            for (size_t g = 0; g < ngroups[q]; ++g) o[start[key(q, g)]++] = make_int2(q, (int)g);
    });
}

// fn(q) for q in [0, n) on up to 64 host threads (dynamic assignment)
template <typename F>
void parallel_for(int n, F &&fn) {
    if (n <= 0) return;
    std::atomic<int> next(0);
    int nth = (int)std::min<unsigned>(std::max(1u, std::thread::hardware_concurrency()), (unsigned)n);
    nth = std::min(nth, 64);
    auto work = [&]() {
        for (int q; (q = next.fetch_add(1)) < n;) fn(q);
    };
    std::vector<std::thread> th;
    for (int t = 1; t < nth; ++t) th.emplace_back(work);
    work();
    for (auto &t : th) t.join();
}

}  // namespace lcg_host
