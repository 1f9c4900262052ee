// ORACLE — test infrastructure only. Only tests/, __graft_entry__.smoke() and
// bench.py's CPU-baseline leg may load this file's library, and only as the
// checker, never as the product path.
//
// Restatement of Aligner::suboptimal (src/LocARNA/aligner.cc:1384-1512): k
// best alignments by interval splitting, scored by align() or, normalized,
// by normalized_align(). The tasks are
// kept in a std::priority_queue ordered by score with the reference's
// comparator (greater_second, aligner.hh:32-44), so that equal scores leave
// the queue in the same order as in the reference.
#include <queue>
#include <vector>

#include "../include/locarna_gb300.h"

extern "C" {
void *lcg_oracle_ctx_new(const lcg_pair_tables *t, const lcg_align_opts *o);
long long lcg_oracle_ctx_top(void *ctx, int sA, int sB, int eA, int eB);
void lcg_oracle_ctx_trace(void *ctx, lcg_align_result *r);
void lcg_oracle_ctx_free(void *ctx);
int lcg_oracle_ctx_stale(void *ctx);
int lcg_oracle_ctx_normalized(void *ctx, int sA, int sB, int eA, int eB, lcg_align_result *r, long long *score);
}

namespace {

struct Restriction {
    int sA, sB, eA, eB;
};
typedef std::pair<Restriction, long long> task_t;

struct score_less {
    bool operator()(const task_t &a, const task_t &b) const { return a.second < b.second; }
};

// Alignment::start_positions / end_positions (alignment.cc:169-195) of raw
// edges: the first / last non-gap position in each sequence
void ends_of(const lcg_align_result &r, int n, int m, int *sa, int *sb, int *ea, int *eb) {
    *sa = n;
    *sb = m;
    *ea = 0;
    *eb = 0;
    for (int k = 0; k < r.num_edges; ++k)
        if (r.edges[2 * k] >= 0) { *sa = r.edges[2 * k]; break; }
    for (int k = 0; k < r.num_edges; ++k)
        if (r.edges[2 * k + 1] >= 0) { *sb = r.edges[2 * k + 1]; break; }
    for (int k = r.num_edges - 1; k >= 0; --k)
        if (r.edges[2 * k] >= 0) { *ea = r.edges[2 * k]; break; }
    for (int k = r.num_edges - 1; k >= 0; --k)
        if (r.edges[2 * k + 1] >= 0) { *eb = r.edges[2 * k + 1]; break; }
}

}  // namespace

// Up to k hits into results[0..k) (edge / arc-match buffers provided as for
// lcg_oracle_align); each hit's score is its task's score. Returns the number
// of hits, or -1 on allocation failure. threshold: tasks scoring below
// threshold + 1 end the enumeration (--better). *stale (may be NULL): the
// number of interval top levels whose result the reference would have taken
// from a cell outside the band (the hits then follow the defined rule and
// may differ from the reference's).
extern "C" int lcg_oracle_kbest(const lcg_pair_tables *t, const lcg_align_opts *o, int k, long long threshold,
                                lcg_align_result *results, int *stale) {
    void *ctx = lcg_oracle_ctx_new(t, o);
    if (!ctx) return -1;
    const int n = t->len_a, m = t->len_b;
    const bool norm = o->normalized != 0;
    // the score of an interval: Aligner::align() or normalized_align() (whose
    // last trace goes to res when given)
    auto eval = [&](const Restriction &r, lcg_align_result *res) -> long long {
        if (!norm) return lcg_oracle_ctx_top(ctx, r.sA, r.sB, r.eA, r.eB);
        long long sc = LCG_NEG_INF;
        if (lcg_oracle_ctx_normalized(ctx, r.sA, r.sB, r.eA, r.eB, res, &sc) != 0) return LCG_NEG_INF;
        return sc;
    };
    std::priority_queue<task_t, std::vector<task_t>, score_less> tasks;
    Restriction full{1, 1, n, m};
    tasks.push(task_t(full, eval(full, nullptr)));
    int hits = 0;
    for (int i = 1; k < 0 || i <= k;) {
        // the reference reads top() of an empty queue here (undefined); the
        // enumeration ends instead
        if (tasks.empty()) break;
        task_t task = tasks.top();
        tasks.pop();
        const Restriction r = task.first;
        // InftyInt comparison: -inf is below every threshold
        if (task.second == LCG_NEG_INF || task.second < threshold + 1) break;
        lcg_align_result &res = results[hits];
        if (norm) {
            eval(r, &res);
        } else {
            lcg_oracle_ctx_top(ctx, r.sA, r.sB, r.eA, r.eB);
            lcg_oracle_ctx_trace(ctx, &res);
        }
        if (res.num_edges == 0) continue;  // empty alignment: no hit, i unchanged
        res.score = task.second;
        ++hits;
        if (k >= 0 && i == k) break;
        int sa, sb, ea, eb;
        ends_of(res, n, m, &sa, &sb, &ea, &eb);
        Restriction r1 = r, r2 = r;
        // the reference's restriction lengths are size_t differences
        if ((unsigned long)(long)(r.eA - r.sA) > (unsigned long)(long)(r.eB - r.sB)) {
            const int split = (sa + ea) / 2;
            r1.eA = split;
            r2.sA = split;
        } else {
            const int split = (sb + eb) / 2;
            r1.eB = split;
            r2.sB = split;
        }
        const long long s1 = eval(r1, nullptr);
        const long long s2 = eval(r2, nullptr);
        tasks.push(task_t(r1, s1));
        tasks.push(task_t(r2, s2));
        ++i;
    }
    if (stale) *stale = lcg_oracle_ctx_stale(ctx);
    lcg_oracle_ctx_free(ctx);
    return hits;
}
