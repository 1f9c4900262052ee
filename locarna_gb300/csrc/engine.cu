// Host side of the GB300 Sankoff engine: validation of the prepared tables,
// derived index structures, one packed host->device upload per batch, the two
// kernel launches, one device->host download, and assembly of the traceback
// tokens into the reference's edge order. Exposes the C ABI of
// include/locarna_gb300.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <functional>
#include <atomic>
#include <cstdio>
#include <chrono>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <queue>
#include <string>
#include <thread>
#include <vector>

#include "../../include/locarna_gb300.h"
#include "lcg_device.cuh"
#include "engine_prep.hh"
#include "engine_state.hh"

#include "sankoff_launch.hh"

using namespace lcg;
using lcg_host::Prep;
using lcg_host::prep_pair;

static thread_local std::string g_last_error;

namespace lcg_host {
void set_error(const std::string &msg) { g_last_error = msg; }
}  // namespace lcg_host

static lcg_status fail(lcg_status code, const std::string &msg) {
    g_last_error = msg;
    return code;
}

#define CUDA_TRY(call)                                                                  \
    do {                                                                                \
        cudaError_t _e = (call);                                                        \
        if (_e != cudaSuccess)                                                          \
            return fail(LCG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e)); \
    } while (0)

// ------------------------------------------------------------------ per-pair prep

namespace lcg_host {

inline bool allowed_match(const lcg_pair_tables &t, int i, int j) {
    return !t.match_lo || (t.match_lo[i] <= j && j <= t.match_hi[i]);
}

lcg_status prep_pair(const lcg_pair_tables &t, const lcg_align_opts &o, Prep &p) {
    auto bad = [&](lcg_status c, const std::string &s) {
        p.code = c;
        p.err = s;
        return c;
    };
    const int n = t.len_a, m = t.len_b;
    if (n < 1 || m < 1) return bad(LCG_ERR_UNSUPPORTED, "empty sequence");
    if (n > 32000 || m > 32000) return bad(LCG_ERR_UNSUPPORTED, "sequence longer than 32000");
    if (!t.sigma || !t.gap_a || !t.gap_b || !t.min_col || !t.max_col)
        return bad(LCG_ERR_ARG, "NULL table pointer");
    if (t.num_arcs_a < 0 || t.num_arcs_b < 0 || t.num_arcmatches < 0)
        return bad(LCG_ERR_ARG, "negative count");
    if ((t.num_arcs_a && !t.arcs_a) || (t.num_arcs_b && !t.arcs_b) ||
        (t.num_arcmatches && (!t.am_arcs || !t.am_score)))
        return bad(LCG_ERR_ARG, "NULL arc table");
    const bool anchors = t.match_lo != nullptr;
    if (anchors && (!t.match_hi || !t.del_lo || !t.del_hi || !t.ins_lo || !t.ins_hi))
        return bad(LCG_ERR_ARG, "anchor ranges must be all set or all NULL");
    p.n = n;
    p.m = m;
    p.fe = o.free_endgaps & 15;
    const bool nolp = o.no_lonely_pairs != 0;
    const bool stack = t.am_stack_score != nullptr;
    if (stack != (t.am_stackable != nullptr))
        return bad(LCG_ERR_ARG, "am_stack_score and am_stackable must be both set or both NULL");
    // normalized and penalized alignment always trace (aligner.cc:1564,1614)
    const bool traced = o.do_trace || o.normalized || o.penalized;
    p.flags = (o.sequ_local ? PF_SEQU_LOCAL : 0) | (anchors ? PF_ANCHORS : 0) |
              (traced ? PF_TRACE : 0) | (o.struct_local ? PF_STRUCT_LOCAL : 0) | (nolp ? PF_NOLP : 0) |
              (stack ? PF_STACK : 0);
    // src/locarna.cc:369-373, 428-446
    if (o.normalized && o.penalized) return bad(LCG_ERR_ARG, "normalized and penalized alignment cannot be combined");
    if (o.normalized && (!o.sequ_local || o.struct_local))
        return bad(LCG_ERR_ARG, "normalized alignment needs sequ_local and no struct_local");
    if (o.normalized && o.normalized_L < 0) return bad(LCG_ERR_ARG, "normalized alignment needs L >= 0");
    if (o.penalized && (long long)std::llabs(o.position_penalty) * (n + m) >= (1ll << 26))
        return bad(LCG_ERR_RANGE, "position penalty times (lenA + lenB) exceeds the device range");
    if (o.sequ_local && p.fe) return bad(LCG_ERR_ARG, "free end gaps cannot be combined with local alignment");

    // band: monotone, inside [0,m], rows non-empty and connected
    // (trace_controller.cc:320-339 asserts the same invariants)
    p.min_col.resize(n + 2);
    p.max_col.resize(n + 2);
    p.bandoff.resize(n + 2);
    long long cells = 0;
    for (int i = 0; i <= n; ++i) {
        int lo = t.min_col[i], hi = t.max_col[i];
        if (lo < 0 || hi > m || lo > hi) return bad(LCG_ERR_ARG, "band row " + std::to_string(i) + " out of range");
        if (i > 0 && (lo < t.min_col[i - 1] || hi < t.max_col[i - 1] || t.max_col[i - 1] + 1 < lo))
            return bad(LCG_ERR_ARG, "band not monotone/connected at row " + std::to_string(i));
        p.min_col[i] = lo;
        p.max_col[i] = hi;
        p.bandoff[i] = (int)cells;
        cells += hi - lo + 1;
    }
    p.min_col[n + 1] = m + 1;
    p.max_col[n + 1] = m;
    p.bandoff[n + 1] = (int)cells;
    p.rowinfo.resize(n + 2);
    for (int i = 0; i <= n + 1; ++i) {
        p.rowinfo[i] = make_int4(p.min_col[i], p.max_col[i], i <= n ? t.gap_a[i] : 0, p.bandoff[i]);
        if (i <= n) p.maxband = std::max(p.maxband, p.max_col[i] - p.min_col[i] + 1);
    }
    for (int i = 0; i < n; ++i) p.span = std::max(p.span, p.max_col[i + 1] - p.min_col[i] + 3);

    // sigma classes: identical rows share a row class, identical columns a
    // column class; with at most 16 of each, sigma is a 16x16 table lookup
    {
        const size_t m1 = (size_t)m + 1;
        std::vector<int> rep_row, rep_col;
        p.rcls.assign(n + 2, 0);
        p.ccls.assign(m + 1, 0);
        bool ok = true;
        for (int i = 1; i <= n && ok; ++i) {
            int c = -1;
            for (size_t k = 0; k < rep_row.size() && c < 0; ++k)
                if (std::memcmp(t.sigma + (size_t)i * m1 + 1, t.sigma + (size_t)rep_row[k] * m1 + 1, 4 * (size_t)m) == 0)
                    c = (int)k;
            if (c < 0) {
                if (rep_row.size() == 16) ok = false;
                c = (int)rep_row.size();
                rep_row.push_back(i);
            }
            p.rcls[i] = c;
        }
        for (int j = 1; j <= m && ok; ++j) {
            int c = -1;
            for (size_t k = 0; k < rep_col.size() && c < 0; ++k) {
                bool same = true;
                for (size_t r = 0; r < rep_row.size() && same; ++r)
                    same = t.sigma[(size_t)rep_row[r] * m1 + j] == t.sigma[(size_t)rep_row[r] * m1 + rep_col[k]];
                if (same) c = (int)k;
            }
            if (c < 0) {
                if (rep_col.size() == 16) ok = false;
                c = (int)rep_col.size();
                rep_col.push_back(j);
            }
            p.ccls[j] = c;
        }
        if (ok) {
            p.scls.assign(256, 0);
            for (size_t r = 0; r < rep_row.size(); ++r)
                for (size_t k = 0; k < rep_col.size(); ++k)
                    p.scls[r * 16 + k] = t.sigma[(size_t)rep_row[r] * m1 + rep_col[k]];
            p.use_cls = true;
            p.flags |= PF_SCLS;
        }
        // per column: the horizontal gap term << 4 | sigma column class. With
        // anchors the term is gapB(j); without, the prefix sum
        // PA(j) = sum_{t=1..j} (gapB(t) + max(go, 0)), from which the fill
        // takes F by a prefix maximum (sankoff_group.cuh)
        p.gbc.assign(m + 1, 0);
        const bool prefix = !(p.flags & PF_ANCHORS);
        const long long gop = std::max(t.indel_opening, 0);
        long long pa = 0;
        for (int j = 0; j <= m; ++j) {
            if (j > 0) pa += t.gap_b[j] + gop;
            if (prefix && (pa >= (1ll << 26) || pa <= -(1ll << 26)))
                return bad(LCG_ERR_RANGE, "gap cost prefix sums exceed the device range");
            p.gbc[j] = (int)(prefix ? pa : t.gap_b[j]) * 16 + (p.use_cls ? p.ccls[j] : 0);
        }
    }
    if (cells > (1ll << 30)) return bad(LCG_ERR_UNSUPPORTED, "band too large");
    p.bandcells = (int)cells;
    if (!o.sequ_local && !(p.fe & (LCG_FREE_RIGHT_1 | LCG_FREE_RIGHT_2)) && p.max_col[n] != m)
        return bad(LCG_ERR_UNSUPPORTED, "global alignment needs (lenA,lenB) inside the band");
    if (p.min_col[0] != 0) return bad(LCG_ERR_UNSUPPORTED, "band must contain (0,0)");

    // score range: every alignment score is a sum of at most (n+m) position
    // terms, (n+m) gap openings and min(n,m)/2 arc-match terms
    long long ms = 0, mg = 0, mam = 0;
    for (long long q = 0; q < (long long)(n + 1) * (m + 1); ++q) ms = std::max(ms, (long long)std::llabs(t.sigma[q]));
    for (int i = 0; i <= n; ++i) mg = std::max(mg, (long long)std::llabs(t.gap_a[i]));
    for (int j = 0; j <= m; ++j) mg = std::max(mg, (long long)std::llabs(t.gap_b[j]));
    for (int k = 0; k < t.num_arcmatches; ++k) mam = std::max(mam, (long long)std::llabs(t.am_score[k]));
    if (stack)
        for (int k = 0; k < t.num_arcmatches; ++k)
            if (t.am_stack_score[k] > LCG_STACK_NONE) mam = std::max(mam, (long long)std::llabs(t.am_stack_score[k]));
    long long bound = (long long)(n + m) * (ms + mg + std::llabs(t.indel_opening) + std::llabs(t.exclusion)) +
                      (long long)(std::min(n, m) / 2 + 1) * mam;
    if (bound >= (1ll << 27)) return bad(LCG_ERR_RANGE, "scores may exceed the int32 device range");

    // arcs span at least 3 positions, as BasePairs makes them
    // (basepairs.cc:162-163: j from i+3), so every corner cell (ar-1,br-1)
    // lies below its group's first row
    for (int k = 0; k < t.num_arcs_a; ++k) {
        int l = t.arcs_a[2 * k], r = t.arcs_a[2 * k + 1];
        if (l < 1 || r > n || r - l < 3) return bad(LCG_ERR_ARG, "arc of A out of range (1 <= l, l+3 <= r <= len)");
    }
    for (int k = 0; k < t.num_arcs_b; ++k) {
        int l = t.arcs_b[2 * k], r = t.arcs_b[2 * k + 1];
        if (l < 1 || r > m || r - l < 3) return bad(LCG_ERR_ARG, "arc of B out of range (1 <= l, l+3 <= r <= len)");
    }
    const int na = t.num_arcmatches;
    p.am_ends.resize(4 * (size_t)na);
    for (int k = 0; k < na; ++k) {
        int a = t.am_arcs[2 * k], b = t.am_arcs[2 * k + 1];
        if (a < 0 || a >= t.num_arcs_a || b < 0 || b >= t.num_arcs_b) return bad(LCG_ERR_ARG, "arc match index out of range");
        p.am_ends[4 * k] = t.arcs_a[2 * a];
        p.am_ends[4 * k + 1] = t.arcs_a[2 * a + 1];
        p.am_ends[4 * k + 2] = t.arcs_b[2 * b];
        p.am_ends[4 * k + 3] = t.arcs_b[2 * b + 1];
    }
    auto in_band = [&](int i, int j) { return i >= 0 && i <= n && p.min_col[i] <= j && j <= p.max_col[i]; };

    // common right end lists over band cells, lex greater left ends
    // (arc_matches.cc:76-110, arc_matches.hh:188-220)
    std::vector<int> cnt(p.bandcells + 1, 0);
    std::vector<int> cell_of(na, -1);
    for (int k = 0; k < na; ++k) {
        int ar = p.am_ends[4 * k + 1], br = p.am_ends[4 * k + 3];
        if (in_band(ar, br)) {
            cell_of[k] = p.bandoff[ar] + br - p.min_col[ar];
            cnt[cell_of[k]]++;
        }
    }
    p.cre_start.assign(p.bandcells + 1, 0);
    for (int c = 0; c < p.bandcells; ++c) p.cre_start[c + 1] = p.cre_start[c] + cnt[c];
    std::vector<int> fillp(p.cre_start.begin(), p.cre_start.end() - 1);
    std::vector<int> ord(p.cre_start[p.bandcells]);
    for (int k = 0; k < na; ++k)
        if (cell_of[k] >= 0) ord[fillp[cell_of[k]]++] = k;
    p.cre.resize(4 * ord.size());
    // (arc matches in the reference's index order come per cell already in
    // this order; sort only where they do not)
    auto lex_greater_left = [&](int x, int y) {
        int alx = p.am_ends[4 * x], aly = p.am_ends[4 * y];
        if (alx != aly) return alx > aly;
        return p.am_ends[4 * x + 2] > p.am_ends[4 * y + 2];
    };
    for (int c = 0; c < p.bandcells; ++c) {
        auto b = ord.begin() + p.cre_start[c], e = ord.begin() + p.cre_start[c + 1];
        if (e - b > 1 && !std::is_sorted(b, e, lex_greater_left)) std::sort(b, e, lex_greater_left);
    }
    // the same candidates per row a.r: a.l descending, then b.l descending
    // (within a row, the valid ones for a group (al,bl) with a.l > al are a
    // prefix). The position of an arc match in this order is also the index
    // of its D entry, so a row's D values are contiguous.
    // bucket by a.r (counting sort of the arc matches in index order), then
    // order each row where the index order does not already give it
    std::vector<int> ordr(ord.size());
    {
        std::vector<int> rstart(n + 2, 0);
        for (int k = 0; k < na; ++k)
            if (cell_of[k] >= 0) rstart[p.am_ends[4 * k + 1] + 1]++;
        for (int r = 0; r <= n; ++r) rstart[r + 1] += rstart[r];
        std::vector<int> fill(rstart.begin(), rstart.end() - 1);
        for (int k = 0; k < na; ++k)
            if (cell_of[k] >= 0) ordr[fill[p.am_ends[4 * k + 1]]++] = k;
        auto row_less = [&](int x, int y) {
            const int *ex = &p.am_ends[4 * x], *ey = &p.am_ends[4 * y];
            if (ex[0] != ey[0]) return ex[0] > ey[0];
            if (ex[2] != ey[2]) return ex[2] > ey[2];
            return ex[3] < ey[3];
        };
        for (int r = 0; r <= n; ++r) {
            auto b = ordr.begin() + rstart[r], e = ordr.begin() + rstart[r + 1];
            if (e - b > 1 && !std::is_sorted(b, e, row_less)) std::sort(b, e, row_less);
        }
    }
    p.am_pos.assign(na, -1);
    p.crow.resize(2 * ordr.size());
    p.rowarc.assign(2 * (size_t)(n + 2), 0);
    for (size_t q = 0; q < ordr.size(); ++q) {
        int k = ordr[q];
        p.am_pos[k] = (int)q;
        // (a.l-1) | (b.l-1) << 16: the inner corner; positions are < 2^15
        p.crow[2 * q] = (p.am_ends[4 * k] - 1) | ((p.am_ends[4 * k + 2] - 1) << 16);
        p.crow[2 * q + 1] = p.am_ends[4 * k + 3];  // b.r: the cell's column
    }
    for (size_t q = 0, r = 0; r <= (size_t)n + 1; ++r) {
        p.rowarc[2 * r] = (int)q;
        while (q < ordr.size() && (size_t)p.am_ends[4 * ordr[q] + 1] == r) ++q;
        p.rowarc[2 * r + 1] = (int)q;
    }
    for (size_t q = 0; q < ord.size(); ++q) {
        int k = ord[q];
        p.cre[4 * q] = p.am_pos[k];                   // D entry
        p.cre[4 * q + 1] = p.am_ends[4 * k] - 1;      // a.l - 1: row of the inner corner
        p.cre[4 * q + 2] = p.am_ends[4 * k + 2] - 1;  // b.l - 1: column of the inner corner
        p.cre[4 * q + 3] = k;                         // the arc match
    }
    p.num_pos = (int)ordr.size();

    // left-end groups (aligner.cc:660-732): bucket arc matches by (al,bl)
    // ordered by (al, bl) descending, index order within equal left ends:
    // two stable counting sorts (by bl descending, then by al descending)
    std::vector<std::pair<long long, int>> byleft(na);
    {
        std::vector<int> tmp(na), cntb(m + 2, 0), cnta(n + 2, 0);
        for (int k = 0; k < na; ++k) cntb[m - p.am_ends[4 * k + 2] + 1]++;
        for (int j = 0; j <= m; ++j) cntb[j + 1] += cntb[j];
        for (int k = 0; k < na; ++k) tmp[cntb[m - p.am_ends[4 * k + 2]]++] = k;
        for (int k = 0; k < na; ++k) cnta[n - p.am_ends[4 * k] + 1]++;
        for (int i = 0; i <= n; ++i) cnta[i + 1] += cnta[i];
        for (int q = 0; q < na; ++q) {
            const int k = tmp[q];
            byleft[cnta[n - p.am_ends[4 * k]]++] = {(long long)p.am_ends[4 * k] * (m + 1) + p.am_ends[4 * k + 2], k};
        }
    }
    // no lonely pairs: the inner arc match of each arc match, the first one in
    // index order with left ends (a.l+1,b.l+1) and right ends (a.r-1,b.r-1)
    // (ArcMatches::init_inner_arc_matchs, arc_matches.cc:50-74); byleft
    // holds each left-end bucket in index order
    std::vector<int> inner;
    if (stack) {
        p.sscore.assign(std::max(na, 1), NEG);
        for (int k = 0; k < na; ++k) p.sscore[k] = t.am_stack_score[k] <= LCG_STACK_NONE ? NEG : t.am_stack_score[k];
    }
    if (nolp || stack) {
        inner.assign(na, -1);
        p.inner.assign(std::max(na, 1), make_int2(-1, -1));
        for (int k = 0; k < na; ++k) {
            const int *ek = &p.am_ends[4 * k];
            if (ek[0] + 1 > n || ek[2] + 1 > m) continue;
            const long long key = (long long)(ek[0] + 1) * (m + 1) + (ek[2] + 1);
            auto it = std::lower_bound(byleft.begin(), byleft.end(), key,
                                       [](const std::pair<long long, int> &x, long long v) { return x.first > v; });
            for (; it != byleft.end() && it->first == key; ++it) {
                const int x = it->second;
                if (p.am_ends[4 * x + 1] == ek[1] - 1 && p.am_ends[4 * x + 3] == ek[3] - 1) {
                    inner[k] = x;
                    p.inner[k] = make_int2(x, p.am_pos[x]);
                    break;
                }
            }
        }
    }
    p.Dinit.assign(p.num_pos, NEG);
    std::vector<int> ks;
    // band cells of rows [r0, r1) inside columns [A, B], in O(log n) from
    // prefix sums (min_col and max_col are nondecreasing)
    std::vector<long long> psmin(n + 2, 0), psmax(n + 2, 0);
    for (int i = 0; i <= n; ++i) {
        psmin[i + 1] = psmin[i] + p.min_col[i];
        psmax[i + 1] = psmax[i] + p.max_col[i];
    }
    auto rect_cells = [&](int r0, int r1, int A, int B) -> long long {
        if (r0 >= r1 || A > B) return 0;
        const int *mn = p.min_col.data(), *mx = p.max_col.data();
        // rows whose band lies left of A (max_col < A) or right of B (min_col > B) are empty
        const int u = (int)(std::lower_bound(mx + r0, mx + r1, A) - mx);
        const int v = (int)(std::upper_bound(mn + r0, mn + r1, B) - mn);
        if (u >= v) return 0;
        const int x = (int)(std::upper_bound(mx + u, mx + v, B) - mx);  // rows [u,x): max_col <= B
        const int y = (int)(std::upper_bound(mn + u, mn + v, A) - mn);  // rows [u,y): min_col <= A
        const long long shi = (psmax[x] - psmax[u]) + (long long)B * (v - x);
        const long long slo = (long long)A * (y - u) + (psmin[v] - psmin[y]);
        return shi - slo + (v - u);
    };
    p.rows_max = 0;
    p.width_max = 0;
    p.rect_cells = 0;
    p.am_rect.assign(std::max(na, 1), make_int2(-1, 0));
    for (size_t s = 0; s < byleft.size();) {
        size_t e = s;
        while (e < byleft.size() && byleft[e].first == byleft[s].first) ++e;
        int k0 = byleft[s].second;
        // the group's left ends: those of the bucket's arc matches, or, without
        // lonely pairs, one inside them (align_D, aligner.cc:660-732, with
        // get_max_right_ends(.., no_lonely_pairs), arc_matches.cc:313-355:
        // the bucket's arc matches that enclose an inner arc match, right
        // ends minus one)
        const int sh = nolp ? 1 : 0;
        int al = p.am_ends[4 * k0] + sh, bl = p.am_ends[4 * k0 + 2] + sh;
        if (al <= n && bl <= m && allowed_match(t, al, bl) && in_band(al, bl) && in_band(al - 1, bl - 1)) {
            int max_ar = al, max_br = bl;
            for (size_t q = s; q < e; ++q) {
                int k = byleft[q].second;
                if (nolp && inner[k] < 0) continue;
                max_ar = std::max(max_ar, p.am_ends[4 * k + 1] - sh);
                max_br = std::max(max_br, p.am_ends[4 * k + 3] - sh);
            }
            if (max_ar == al || max_br == bl) {
                s = e;
                continue;
            }
            GroupItem g{};
            g.al = al;
            g.ar = max_ar;
            g.bl = bl;
            g.br = max_br;
            g.dw_start = (int)p.dw.size();
            g.top = 0;
            ks.clear();
            for (size_t q = s; q < e; ++q) ks.push_back(byleft[q].second);
            auto ar_less = [&](int x, int y) { return p.am_ends[4 * x + 1] < p.am_ends[4 * y + 1]; };
            if (!std::is_sorted(ks.begin(), ks.end(), ar_less)) std::stable_sort(ks.begin(), ks.end(), ar_less);
            for (int k : ks) {
                // fill_D_entries_noLP: only arc matches with an inner arc
                // match, with stacking only stackable ones (aligner.cc:629-630)
                if (nolp && (inner[k] < 0 || (stack && !t.am_stackable[k]))) continue;
                // the corner: (ar-1,br-1) inside the arc match, or, without
                // lonely pairs, inside its inner arc match
                int ar = p.am_ends[4 * k + 1] - sh, br = p.am_ends[4 * k + 3] - sh;
                // the corner is computed by this group iff it is in the band
                // (only arc matches whose right ends are a band cell are ever read)
                if (ar - 1 > al && br - 1 > bl && in_band(ar - 1, br - 1) && p.am_pos[k] >= 0) {
                    if (nolp) {
                        const int in = inner[k];
                        const int sk = stack ? p.sscore[k] : t.am_score[k];  // arcmatch(am, stacking)
                        p.dw.push_back(make_int4(p.am_pos[k], ar - 1, br - 1, sk + t.am_score[in]));
                        p.dwn.push_back(make_int2(p.am_pos[in], sk));
                    } else {
                        p.dw.push_back(make_int4(p.am_pos[k], ar - 1, br - 1, t.am_score[k]));
                        if (stack) {
                            // fill_D_entries with stacking (aligner.cc:600-608)
                            const int in = inner[k];
                            if (in >= 0 && t.am_stackable[k]) p.dwn.push_back(make_int2(p.am_pos[in], p.sscore[k]));
                            else p.dwn.push_back(make_int2(-1, 0));
                        }
                    }
                    p.Dinit[p.am_pos[k]] = NOT_READY;
                }
            }
            g.dw_count = (int)p.dw.size() - g.dw_start;
            // the kept rectangle (rows al..ar-1, columns bl..br-1); the
            // traceback reads it for the arc matches of this bucket (left
            // ends (al, bl); without lonely pairs the group's left ends are
            // shifted, and the traceback recomputes)
            const int rect_pitch = max_br - bl;
            g.rect_off = -1;
            if (p.rect_cells >= 0) {
                const long long sz = (long long)(max_ar - al) * rect_pitch;
                if (p.rect_cells + sz >= (1ll << 31)) {
                    p.rect_cells = -1;
                } else {
                    g.rect_off = (int)p.rect_cells;
                    p.rect_cells += sz;
                    if (!nolp)
                        for (size_t q = s; q < e; ++q) p.am_rect[byleft[q].second] = make_int2(g.rect_off, rect_pitch);
                }
            }
            p.cells += rect_cells(al + 1, max_ar, bl + 1, max_br - 1);
            g.cpl = 1;
            p.groups.push_back(g);
            p.rows_max = std::max(p.rows_max, max_ar - al);
            p.width_max = std::max(p.width_max, max_br - bl + 1);
        }
        s = e;
    }
#ifdef LCG_TEST_DROP_LAST_D_WRITE
    // test build only (tests/test_zy_wait_timeout.py): the last group's last
    // D write is moved to a row the group never reaches, so that entry stays
    // NOT_READY and the top level's bounded wait for it runs out
    if (!p.dw.empty()) p.dw.back().y = INT_MAX;
#endif
    // byleft is sorted by (al*(m+1)+bl) descending = al descending, bl descending
    GroupItem top{};
    top.al = 0;
    top.ar = n + 1;
    top.bl = 0;
    top.br = m + 1;
    top.top = 1;
    int twmax = 1;
    for (int i = 1; i <= n; ++i) {
        int w = std::min(m, p.max_col[i]) - std::max(1, p.min_col[i]) + 1;
        p.cells += std::max(w, 0);
        twmax = std::max(twmax, w);
    }
    top.cpl = std::min(4, (twmax + 31) / 32);
    p.groups.push_back(top);
    p.token_cap = 2 * (n + m) + 3 * std::min(n, m) + 16;
    p.tq_cap = std::min(n, m) / 2 + 2;
    return LCG_OK;
}

}  // namespace lcg_host

namespace {

// expand token segments into the reference's append order
struct Assembler {
    const int2 *tok;
    std::vector<std::pair<int, int>> seg_of;  // am -> (start,end) ; index via map
    std::vector<int> seg_am;
    std::vector<int> seg_start, seg_end;
    int32_t *edges;
    int edge_cap, nedges = 0;
    int32_t *tam;
    int tam_cap, ntam = 0;
    bool ok = true;
    int find(int am) const {
        for (size_t s = 0; s < seg_am.size(); ++s)
            if (seg_am[s] == am) return (int)s;
        return -1;
    }
    void expand(int s, int depth) {
        if (s < 0 || depth > 100000) {
            ok = false;
            return;
        }
        for (int q = seg_end[s] - 1; q >= seg_start[s]; --q) {
            int2 t = tok[q];
            if (t.x == -2) {
                if (ntam < tam_cap && tam) tam[ntam] = t.y;
                ++ntam;
                expand(find(t.y), depth + 1);
            } else {
                if (nedges < edge_cap && edges) {
                    edges[2 * nedges] = t.x;
                    edges[2 * nedges + 1] = t.y;
                }
                ++nedges;
            }
        }
    }
};

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// One buffer set of the engine, by reference: set 0 is the engine's own
// fields, set 1 the second set of the pipeline.
struct Slot {
    cudaStream_t st;
    char **d_arena;
    size_t *arena_cap;
    char **h_stage;
    size_t *stage_cap;
    int **d_scratch;
    size_t *scratch_cap;
    cudaEvent_t ev0, ev1, ev2;
    lcg_graph_cache *graph;
};

Slot slot_of(lcg_engine e, int k) {
    if (k == 0)
        return Slot{e->stream, &e->d_arena, &e->arena_cap, &e->h_stage, &e->stage_cap,
                    &e->d_scratch, &e->scratch_cap, e->ev0, e->ev1, e->ev2, &e->graph};
    lcg_buffer_set &b = e->alt;
    return Slot{b.stream, &b.d_arena, &b.arena_cap, &b.h_stage, &b.stage_cap,
                &b.d_scratch, &b.scratch_cap, b.ev0, b.ev1, b.ev2, &b.graph};
}

// byte offsets of one pair's tables in the arena
struct PairOff {
    size_t sigma, scls, rcls, ccls, gapA, gapB, minc, maxc, bandoff, rowinfo, anc, cre_start, cre, crow, rowarc,
        am_score, D, topM, res, tok, tq, segs, groups, dw, gbc, dwn, inner, sscore, rect, am_rect;
};

// One chunk of an lcg_align_pairs call: pairs [q0, q0 + nq) of the batch.
struct Chunk {
    int q0 = 0, nq = 0;
    std::vector<Prep> prep;
    std::vector<PairOff> off;
    size_t off_ctrl = 0, down_begin = 0, down_end = 0;
    long long launches = 0;
    bool in_flight = false;
    std::vector<long long> ratio;  // normalized alignment: the final score ratio per pair
    // k-best alignment: the fill only (the top levels and traces follow per
    // round), and what the rounds need of the launch
    bool kbest = false;
    size_t off_pairs = 0, off_mod = 0;
    int sw = 0, rb = 0;
    long long stride = 0;
    bool sl = false;
    bool sl_fast = false;  // struct-local fast routines (every pair: class table, no anchors)
    int *scratch = nullptr;
    // launch configuration: resident fill blocks per SM (0 = as many as fit)
    // and the L2 budget of a pair wave in MB (0 = default)
    int bps = 0;
    double wave_mb = 0;
};

// pairs per chunk: one chunk for small batches, else up to 8 chunks of at
// least 128 pairs (the first chunk's host preparation is not overlapped)
int chunk_size(int npairs, int setting) {
    if (setting > 0) return setting;
    if (npairs < 256) return npairs;
    const int k = std::min(8, npairs / 128);
    return (npairs + k - 1) / k;
}

double ms_between(std::chrono::steady_clock::time_point a, std::chrono::steady_clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

// Top levels of normalized and penalized alignment after the fill
// (Aligner::normalized_align / penalized_align, aligner.cc:1527-1617): the top
// level of every pair under the scoring modified by its penalty lam
// (sankoff_top_kernel). Penalized: one pass with lam = PP. Normalized:
// Dinkelbach iterations per pair, lam <- (score + length lam) / (length + L)
// with length = (max_i - min_i + 1) + (max_j - min_j + 1) from a top-level
// walk, until lam repeats; each iteration runs the pairs whose lam changed,
// and the host reads their result words once per iteration. On return the
// device holds each pair's final lam and top level, and *sel selects the
// final traceback's penalties. Synchronises the stream once per iteration.
lcg_status mod_top_levels(const lcg_align_opts *opts, Chunk &c, const PairDev *dpairs, int *dmod, int npairs,
                          int *scratch, long long stride, int sw, int rb, bool sl, int *status, cudaStream_t st,
                          TraceSel *sel) {
    int *d_lam = dmod, *d_items = dmod + npairs, *d_res = dmod + 2 * npairs;
    std::vector<int> lam(npairs, 0), items(npairs);
    for (int q = 0; q < npairs; ++q) items[q] = q;
    sel->lam = d_lam;
    if (opts->penalized) {
        std::fill(lam.begin(), lam.end(), opts->position_penalty);
        CUDA_TRY(cudaMemcpyAsync(d_lam, lam.data(), 4ull * npairs, cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaMemcpyAsync(d_items, items.data(), 4ull * npairs, cudaMemcpyHostToDevice, st));
        CUDA_TRY(launch_top(dpairs, d_items, npairs, d_lam, nullptr, rb, status, st));
        c.launches += 1;
        return LCG_OK;
    }
    const long long L = opts->normalized_L;
    std::vector<long long> lambda(npairs, -1), nl(npairs, 0);
    std::vector<int> res(5ull * npairs);
    for (int iter = 0; !items.empty(); ++iter) {
        if (iter > 100000) return fail(LCG_ERR_DEVICE, "normalized alignment: Dinkelbach iterations do not converge");
        for (int q : items) {
            lambda[q] = nl[q];
            if (std::llabs(lambda[q]) * (c.prep[q].n + c.prep[q].m) >= (1ll << 26))
                return fail(LCG_ERR_RANGE, "normalized alignment: score ratio times length exceeds the device range");
            lam[q] = (int)lambda[q];
        }
        const int ni = (int)items.size();
        CUDA_TRY(cudaMemcpyAsync(d_lam, lam.data(), 4ull * npairs, cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaMemcpyAsync(d_items, items.data(), 4ull * ni, cudaMemcpyHostToDevice, st));
        CUDA_TRY(launch_top(dpairs, d_items, ni, d_lam, nullptr, rb, status, st));
        TraceSel ts;
        ts.items = d_items;
        ts.nitems = ni;
        ts.lam = d_lam;
        ts.flags = TRACE_TOP_ONLY | (iter ? TRACE_KEEP_MIN : 0);
        if (sl) CUDA_TRY(launch_sl_trace(dpairs, npairs, scratch, stride, sw, rb, c.sl_fast, status, st, ts));
        else CUDA_TRY(launch_trace(dpairs, npairs, scratch, stride, sw, rb, status, st, ts));
        CUDA_TRY(launch_gather_res(dpairs, d_items, ni, d_res, st));
        c.launches += 3;
        CUDA_TRY(cudaMemcpyAsync(res.data(), d_res, 20ull * ni, cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        std::vector<int> still;
        for (int k = 0; k < ni; ++k) {
            const int q = items[k];
            const int *r = &res[5ull * k];
            if (r[R_SCORE] < MIN_FINITE) return fail(LCG_ERR_DEVICE, "normalized alignment: -inf top level");
            const long long length = (long long)(r[R_MAXI] - r[R_MINI] + 1) + (r[R_MAXJ] - r[R_MINJ] + 1);
            const long long score = (long long)r[R_SCORE] + length * lambda[q];
            if (length + L <= 0)
                return fail(LCG_ERR_ARG, "normalized alignment: empty alignment with L = 0 (division by zero)");
            nl[q] = score / (length + L);
            if (nl[q] != lambda[q]) still.push_back(q);
        }
        items.swap(still);
    }
    c.ratio.assign(lambda.begin(), lambda.end());
    sel->flags = TRACE_KEEP_MIN;
    return LCG_OK;
}

// Lay out, pack and enqueue one prepared chunk on its buffer set: one
// host->device copy, the fill (and traceback) launch, one device->host copy.
// Returns without waiting.
lcg_status chunk_launch(lcg_engine e, const Slot &s, const lcg_pair_tables *all, const lcg_align_opts *opts,
                        Chunk &c, double *pack_ms) {
    const auto tp0 = std::chrono::steady_clock::now();
    const lcg_pair_tables *pairs = all + c.q0;
    const int npairs = c.nq;
    std::vector<Prep> &prep = c.prep;
    int sw = 0, rows_max = 1, span = 2;
    for (auto &p : prep) {
        sw = std::max(sw, std::max(p.width_max + 1, p.m + 2));
        rows_max = std::max(rows_max, p.rows_max + 1);
        span = std::max(span, p.span);
    }
    // Kept group rectangles: the fill writes every group's M to a rectangle
    // of its own and the traceback walks traced arc matches on them instead
    // of recomputing them, when the chunk's rectangles fit the engine's
    // budget (lcg_engine_set_rect_budget) - single pairs and small batches.
    // Structure-local rectangles hold all eight states (32 bytes per cell,
    // the traceback switches between them). Not with lonely pairs excluded
    // (shifted group left ends).
    const long long rect_bytes_per_cell = opts->struct_local ? 32 : 4;
    bool keep;
    {
        const long long budget = e->rect_budget >= 0 ? e->rect_budget
                                                     : (opts->struct_local ? RECT_BUDGET_SL : RECT_BUDGET_PLAIN);
        keep = budget > 0;
        long long cells = 0;
        for (auto &p : prep) {
            if (p.rect_cells < 0 || (p.flags & PF_NOLP)) keep = false;
            cells += p.rect_cells;
        }
        keep = keep && (double)rect_bytes_per_cell * (double)cells <= (double)budget;
    }
    c.off.assign(npairs, PairOff{});
    std::vector<PairOff> &off = c.off;
    size_t up = 0;  // upload section (bytes)
    auto take = [](size_t &cur, size_t bytes) {
        size_t o = cur;
        cur = align_up(cur + bytes, 16);
        return o;
    };
    size_t off_pairs = take(up, sizeof(PairDev) * npairs);
    size_t nitems = 0;
    for (auto &p : prep) nitems += p.groups.size();
    size_t off_queue = take(up, sizeof(int2) * nitems);  // (pair, group) work items
    c.off_ctrl = take(up, 64);  // qhead, status, abort, pad, 2 x u64 counters
    const size_t off_ctrl = c.off_ctrl;
    for (int q = 0; q < npairs; ++q) {
        const auto &p = prep[q];
        const auto &t = pairs[q];
        PairOff &o = off[q];
        o.gbc = take(up, 4ull * (p.m + 1));
        o.groups = take(up, sizeof(GroupItem) * p.groups.size());
        o.dw = take(up, sizeof(int4) * std::max<size_t>(p.dw.size(), 1));
        o.dwn = p.inner.empty() ? 0 : take(up, sizeof(int2) * std::max<size_t>(p.dwn.size(), 1));
        o.inner = p.inner.empty() ? 0 : take(up, sizeof(int2) * p.inner.size());
        o.sscore = p.sscore.empty() ? 0 : take(up, 4ull * p.sscore.size());
        // sigma: the class table when it exists, else the dense table
        o.sigma = p.use_cls ? 0 : take(up, 4ull * (p.n + 1) * (p.m + 1));
        o.scls = p.use_cls ? take(up, 4ull * 256) : 0;
        o.rcls = p.use_cls ? take(up, 4ull * (p.n + 2)) : 0;
        o.ccls = p.use_cls ? take(up, 4ull * (p.m + 1)) : 0;
        o.gapA = take(up, 4ull * (p.n + 1));
        o.gapB = take(up, 4ull * (p.m + 1));
        o.minc = take(up, 4ull * (p.n + 2));
        o.maxc = take(up, 4ull * (p.n + 2));
        o.bandoff = take(up, 4ull * (p.n + 2));
        o.rowinfo = take(up, 16ull * (p.n + 2));
        o.anc = t.match_lo ? take(up, 4ull * (2 * (p.n + 1) + 2 * (p.n + 1) + 2 * (p.m + 1))) : 0;
        o.cre_start = take(up, 4ull * (p.bandcells + 1));
        o.cre = take(up, 4ull * std::max<size_t>(p.cre.size(), 4));
        o.crow = take(up, 4ull * std::max<size_t>(p.crow.size(), 4));
        o.rowarc = take(up, 4ull * p.rowarc.size());
        o.am_score = take(up, 4ull * std::max(t.num_arcmatches, 1));
        o.D = take(up, 4ull * std::max(p.num_pos, 1));
        o.am_rect = keep ? take(up, 8ull * p.am_rect.size()) : 0;
    }
    c.down_begin = up;
    size_t dn = up;
    for (int q = 0; q < npairs; ++q) {
        const auto &p = prep[q];
        PairOff &o = off[q];
        o.res = take(dn, 4ull * R_NWORDS);
        o.tok = take(dn, 8ull * p.token_cap);
        o.segs = take(dn, 16ull * (p.tq_cap + 1));
    }
    c.down_end = dn;
    const size_t down_begin = c.down_begin, down_end = c.down_end;
    size_t dev_only = dn;
    for (int q = 0; q < npairs; ++q) {
        const auto &p = prep[q];
        PairOff &o = off[q];
        o.tq = take(dev_only, 16ull * p.tq_cap);
        o.topM = take(dev_only, 4ull * (p.n + 1) * (p.m + 1));
        o.rect = keep ? take(dev_only, (size_t)rect_bytes_per_cell * std::max<long long>(p.rect_cells, 1)) : 0;
    }
    // normalized / penalized alignment: per pair its penalty, the selected
    // pairs and their gathered result words
    const bool modv = opts->normalized || opts->penalized;
    // k-best: penalties, items, two gathered result sets, restrictions
    const size_t off_mod = (modv || c.kbest) ? take(dev_only, 4ull * 16 * npairs) : 0;
    size_t total = dev_only;

    // the set's graph addresses its arena, staging and scratch: it goes
    // before any of them is freed
    if (total > *s.arena_cap) {
        s.graph->release();
        if (*s.d_arena) cudaFree(*s.d_arena);
        *s.d_arena = nullptr;
        *s.arena_cap = 0;
        size_t cap = total + total / 4;
        if (cudaMalloc(s.d_arena, cap) != cudaSuccess) return fail(LCG_ERR_NOMEM, "device arena allocation failed");
        *s.arena_cap = cap;
    }
    if (down_end > *s.stage_cap) {
        s.graph->release();
        if (*s.h_stage) cudaFreeHost(*s.h_stage);
        *s.h_stage = nullptr;
        *s.stage_cap = 0;
        size_t cap = down_end + down_end / 4;
        if (cudaMallocHost(s.h_stage, cap) != cudaSuccess) return fail(LCG_ERR_NOMEM, "pinned staging allocation failed");
        *s.stage_cap = cap;
    }
    char *H = *s.h_stage;
    char *Dv = *s.d_arena;

    // ---- pack the upload
    PairDev *hp = (PairDev *)(H + off_pairs);
    {
        // pairs in waves whose per-pair tables (candidate lists, D, top
        // level) together stay within a share of L2; inside a wave the
        // pairs' work lists are interleaved so that every pair progresses
        // proportionally; within a pair the order is kept. Waves follow each
        // other in the queue without a barrier.
        std::vector<size_t> ng(npairs);
        for (int q = 0; q < npairs; ++q) ng[q] = prep[q].groups.size();
        lcg_host::queue_order(
            ng, [&](int q) { return 12.0 * prep[q].num_pos + 4.0 * prep[q].bandcells; }, (int2 *)(H + off_queue),
            [](int n, auto fn) { lcg_host::parallel_for(n, fn); }, c.wave_mb * 1048576.0);
    }
    std::memset(H + off_ctrl, 0, 64);
    lcg_host::parallel_for(npairs, [&](int q) {
        const auto &p = prep[q];
        const auto &t = pairs[q];
        const PairOff &o = off[q];
        if (p.use_cls) {
            std::memcpy(H + o.scls, p.scls.data(), 4ull * 256);
            std::memcpy(H + o.rcls, p.rcls.data(), 4ull * (p.n + 2));
            std::memcpy(H + o.ccls, p.ccls.data(), 4ull * (p.m + 1));
        } else {
            std::memcpy(H + o.sigma, t.sigma, 4ull * (p.n + 1) * (p.m + 1));
        }
        std::memcpy(H + o.gapA, t.gap_a, 4ull * (p.n + 1));
        std::memcpy(H + o.gapB, t.gap_b, 4ull * (p.m + 1));
        std::memcpy(H + o.minc, p.min_col.data(), 4ull * (p.n + 2));
        std::memcpy(H + o.maxc, p.max_col.data(), 4ull * (p.n + 2));
        std::memcpy(H + o.bandoff, p.bandoff.data(), 4ull * (p.n + 2));
        std::memcpy(H + o.rowinfo, p.rowinfo.data(), 16ull * (p.n + 2));
        if (t.match_lo) {
            int *a = (int *)(H + o.anc);
            std::memcpy(a, t.match_lo, 4ull * (p.n + 1));
            std::memcpy(a + (p.n + 1), t.match_hi, 4ull * (p.n + 1));
            std::memcpy(a + 2 * (p.n + 1), t.del_lo, 4ull * (p.n + 1));
            std::memcpy(a + 3 * (p.n + 1), t.del_hi, 4ull * (p.n + 1));
            std::memcpy(a + 4 * (p.n + 1), t.ins_lo, 4ull * (p.m + 1));
            std::memcpy(a + 4 * (p.n + 1) + (p.m + 1), t.ins_hi, 4ull * (p.m + 1));
        }
        std::memcpy(H + o.cre_start, p.cre_start.data(), 4ull * (p.bandcells + 1));
        if (!p.cre.empty()) std::memcpy(H + o.cre, p.cre.data(), 4ull * p.cre.size());
        if (!p.crow.empty()) std::memcpy(H + o.crow, p.crow.data(), 4ull * p.crow.size());
        std::memcpy(H + o.rowarc, p.rowarc.data(), 4ull * p.rowarc.size());
        if (p.num_pos) std::memcpy(H + o.D, p.Dinit.data(), 4ull * p.num_pos);
        if (t.num_arcmatches) {
            std::memcpy(H + o.am_score, t.am_score, 4ull * t.num_arcmatches);
        }
        std::memcpy(H + o.gbc, p.gbc.data(), 4ull * (p.m + 1));
        GroupItem *hg = (GroupItem *)(H + o.groups);
        for (size_t g = 0; g < p.groups.size(); ++g) {
            hg[g] = p.groups[g];
            hg[g].pair = q;
        }
        if (!p.dw.empty()) std::memcpy(H + o.dw, p.dw.data(), sizeof(int4) * p.dw.size());
        if (!p.dwn.empty()) std::memcpy(H + o.dwn, p.dwn.data(), sizeof(int2) * p.dwn.size());
        if (!p.inner.empty()) std::memcpy(H + o.inner, p.inner.data(), sizeof(int2) * p.inner.size());
        if (!p.sscore.empty()) std::memcpy(H + o.sscore, p.sscore.data(), 4ull * p.sscore.size());
        if (keep) std::memcpy(H + o.am_rect, p.am_rect.data(), 8ull * p.am_rect.size());
        PairDev &d = hp[q];
        std::memset(&d, 0, sizeof d);
        d.n = p.n;
        d.m = p.m;
        d.go = t.indel_opening;
        d.excl = t.exclusion;
        d.flags = p.flags;
        d.free_endgaps = p.fe;
        d.la = t.match_lo ? t.left_anchor_a : p.n + 1;
        d.lb = t.match_lo ? t.left_anchor_b : p.m + 1;
        d.ra = t.match_lo ? t.right_anchor_a : 0;
        d.rb = t.match_lo ? t.right_anchor_b : 0;
        d.num_am = t.num_arcmatches;
        d.bandcells = p.bandcells;
        d.sigma = p.use_cls ? nullptr : (const int *)(Dv + o.sigma);
        if (p.use_cls) {
            d.scls = (const int *)(Dv + o.scls);
            d.rcls = (const int *)(Dv + o.rcls);
            d.ccls = (const int *)(Dv + o.ccls);
        }
        d.gapA = (const int *)(Dv + o.gapA);
        d.gapB = (const int *)(Dv + o.gapB);
        d.min_col = (const int *)(Dv + o.minc);
        d.max_col = (const int *)(Dv + o.maxc);
        d.bandoff = (const int *)(Dv + o.bandoff);
        d.rowinfo = (const int4 *)(Dv + o.rowinfo);
        d.maxband = p.maxband;
        if (t.match_lo) {
            const int *a = (const int *)(Dv + o.anc);
            d.match_lo = a;
            d.match_hi = a + (p.n + 1);
            d.del_lo = a + 2 * (p.n + 1);
            d.del_hi = a + 3 * (p.n + 1);
            d.ins_lo = a + 4 * (p.n + 1);
            d.ins_hi = a + 4 * (p.n + 1) + (p.m + 1);
        }
        d.cre_start = (const int *)(Dv + o.cre_start);
        d.cre = (const int4 *)(Dv + o.cre);
        d.crow = (const int2 *)(Dv + o.crow);
        d.num_pos = p.num_pos;
        d.rowarc = (const int2 *)(Dv + o.rowarc);
        d.D = (int *)(Dv + o.D);
        d.am_score = (const int *)(Dv + o.am_score);
        d.topM = (int *)(Dv + o.topM);
        d.res = (int *)(Dv + o.res);
        d.tokens = (int2 *)(Dv + o.tok);
        d.token_cap = p.token_cap;
        d.tq = (int4 *)(Dv + o.tq);
        d.tq_cap = p.tq_cap;
        d.segs = (int4 *)(Dv + o.segs);
        d.gbc = (const int *)(Dv + o.gbc);
        d.groups = (const GroupItem *)(Dv + o.groups);
        d.rect = keep ? (int *)(Dv + o.rect) : nullptr;
        d.am_rect = keep ? (const int2 *)(Dv + o.am_rect) : nullptr;
        d.dw = (const int4 *)(Dv + o.dw);
        d.dwn = p.inner.empty() ? nullptr : (const int2 *)(Dv + o.dwn);
        d.inner = p.inner.empty() ? nullptr : (const int2 *)(Dv + o.inner);
        d.am_sscore = p.sscore.empty() ? nullptr : (const int *)(Dv + o.sscore);
    });
    *pack_ms += ms_between(tp0, std::chrono::steady_clock::now());

    // ---- scratch
    const bool sl = opts->struct_local != 0;
    const int rb = lcg_host::ring_size(span);
    bool fast = true, sl_fast = true;
    for (auto &p : prep) {
        fast = fast && (p.flags & PF_SCLS) && !(p.flags & (PF_ANCHORS | PF_NOLP | PF_STACK));
        sl_fast = sl_fast && (p.flags & PF_SCLS) && !(p.flags & PF_ANCHORS);
    }
    c.sl_fast = sl_fast;
    c.rb = rb;
    int blocks_per_sm = 0;
    if (sl) {
        CUDA_TRY(sl_prepare(sw, rb, sl_fast, keep, &blocks_per_sm));
    } else {
        CUDA_TRY(fill_occupancy(rb, e->counting, fast, &blocks_per_sm));
        CUDA_TRY(trace_prepare(rb));
    }
    if (blocks_per_sm < 1) return fail(LCG_ERR_UNSUPPORTED, "fill kernel does not fit on an SM");
    if (c.bps > 0 && c.bps < blocks_per_sm) blocks_per_sm = c.bps;
    int blocks = e->sms * blocks_per_sm;
    long long stride = (long long)rows_max * sw;
    // state matrices per slot: fill 1 (plain) / 4 (struct-local); traceback 1 / 8
    size_t fill_slots = (size_t)blocks * (sl ? sl_fill_warps_per_block() * 4 : fill_warps_per_block());
    size_t trace_slots = (size_t)npairs * (sl ? 8 : 1);
    size_t need = std::max(fill_slots, trace_slots) * (size_t)stride;
    if (need > *s.scratch_cap) {
        s.graph->release();
        if (*s.d_scratch) cudaFree(*s.d_scratch);
        *s.d_scratch = nullptr;
        *s.scratch_cap = 0;
        if (cudaMalloc(s.d_scratch, need * sizeof(int)) != cudaSuccess)
            return fail(LCG_ERR_NOMEM, "device scratch allocation failed");
        *s.scratch_cap = need;
    }
    int *scratch = *s.d_scratch;

    // ---- transfer + launch + transfer
    cudaStream_t st = s.st;
    // Without host steps between the launches (not normalized / penalized /
    // k-best), the chunk's device work is one CUDA graph: captured from the
    // stream on first use, replayed while the launch parameters (buffers,
    // sizes, grid) stay the same, updated in place otherwise.
    const bool use_graph = e->graphs && !modv && !c.kbest;
    std::vector<long long> key;
    if (use_graph) {
        key = {(long long)(uintptr_t)Dv, (long long)(uintptr_t)H, (long long)(uintptr_t)scratch, (long long)down_begin,
               (long long)down_end, (long long)off_ctrl, (long long)off_pairs, (long long)off_queue, (long long)nitems,
               blocks, sw, rb, stride, fast, e->counting, sl, sl_fast, keep, opts->do_trace, npairs};
        if (s.graph->exec && s.graph->key == key) {
            CUDA_TRY(cudaGraphLaunch(s.graph->exec, st));
            ++e->last_graph_replays;
            c.launches = opts->do_trace ? 2 : 1;
            c.off_pairs = off_pairs;
            c.off_mod = off_mod;
            c.sw = sw;
            c.rb = rb;
            c.stride = stride;
            c.sl = sl;
            c.scratch = scratch;
            c.in_flight = true;
            e->last_h2d += (long long)down_begin;
            e->last_d2h += 64 + (long long)(down_end - down_begin);
            return LCG_OK;
        }
        CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    }
    // timing events: inside a capture an event record becomes a graph node
    // only when it is marked external
    auto record = [&](cudaEvent_t ev) {
        return use_graph ? cudaEventRecordWithFlags(ev, st, cudaEventRecordExternal) : cudaEventRecord(ev, st);
    };
    // an error inside the capture ends it before returning
    auto end_capture = [&]() {
        if (!use_graph) return;
        cudaGraph_t g = nullptr;
        cudaStreamEndCapture(st, &g);
        if (g) cudaGraphDestroy(g);
    };
#undef CUDA_TRY_CAP
#define CUDA_TRY_CAP(call)                                                                      \
    do {                                                                                        \
        cudaError_t _e = (call);                                                                \
        if (_e != cudaSuccess) {                                                                \
            end_capture();                                                                      \
            return fail(LCG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e));      \
        }                                                                                       \
    } while (0)
    CUDA_TRY_CAP(cudaMemcpyAsync(Dv, H, down_begin, cudaMemcpyHostToDevice, st));
    CUDA_TRY_CAP(cudaMemsetAsync(Dv + down_begin, 0, down_end - down_begin, st));
    unsigned int *qhead = (unsigned int *)(Dv + off_ctrl);
    int *status = (int *)(Dv + off_ctrl + 4);
    int *abort_flag = (int *)(Dv + off_ctrl + 8);
    CUDA_TRY_CAP(record(s.ev0));
    unsigned long long *counters = e->counting ? (unsigned long long *)(Dv + off_ctrl + 16) : nullptr;
    if (sl) {
        if (counters) {
            end_capture();
            return fail(LCG_ERR_UNSUPPORTED, "work counting covers the plain mode only");
        }
        CUDA_TRY_CAP(launch_sl_fill((const PairDev *)(Dv + off_pairs), (const int2 *)(Dv + off_queue),
                                (int)nitems, scratch, stride, sw, rb, sl_fast, keep, qhead,
                                status, abort_flag, blocks, st));
    } else {
        CUDA_TRY_CAP(launch_fill((const PairDev *)(Dv + off_pairs), (const int2 *)(Dv + off_queue),
                             (int)nitems, scratch, stride, sw, rb, fast, qhead,
                             status, abort_flag, blocks, st, counters));
    }
    CUDA_TRY_CAP(record(s.ev1));
    c.launches = 1;
    TraceSel sel;
    if (modv) {
        lcg_status ms = mod_top_levels(opts, c, (const PairDev *)(Dv + off_pairs), (int *)(Dv + off_mod), npairs,
                                       scratch, stride, sw, rb, sl, status, st, &sel);
        if (ms != LCG_OK) return ms;
    }
    c.off_pairs = off_pairs;
    c.off_mod = off_mod;
    c.sw = sw;
    c.rb = rb;
    c.stride = stride;
    c.sl = sl;
    c.scratch = scratch;
    if ((opts->do_trace || modv) && !c.kbest) {
        if (sl)
            CUDA_TRY_CAP(launch_sl_trace((const PairDev *)(Dv + off_pairs), npairs, scratch, stride, sw, rb,
                                     sl_fast, status, st, sel));
        else
            CUDA_TRY_CAP(launch_trace((const PairDev *)(Dv + off_pairs), npairs, scratch, stride, sw, rb, status,
                                  st, sel));
        ++c.launches;
    }
    CUDA_TRY_CAP(record(s.ev2));
    CUDA_TRY_CAP(cudaMemcpyAsync(H + off_ctrl, Dv + off_ctrl, 64, cudaMemcpyDeviceToHost, st));
    CUDA_TRY_CAP(cudaMemcpyAsync(H + down_begin, Dv + down_begin, down_end - down_begin, cudaMemcpyDeviceToHost, st));
    if (use_graph) {
        cudaGraph_t g = nullptr;
        CUDA_TRY(cudaStreamEndCapture(st, &g));
        // the set's graph updated in place, or instantiated again when the
        // update is refused
        lcg_graph_cache &gc = *s.graph;
        cudaGraphExecUpdateResultInfo info;
        if (!gc.exec || cudaGraphExecUpdate(gc.exec, g, &info) != cudaSuccess) {
            cudaGetLastError();  // a refused update leaves the runtime's last error set: clear it
            gc.release();
            const cudaError_t ie = cudaGraphInstantiate(&gc.exec, g, 0);
            if (ie != cudaSuccess) {
                gc.exec = nullptr;
                cudaGraphDestroy(g);
                return fail(LCG_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(ie));
            }
        }
        cudaGraphDestroy(g);
        gc.key = key;
        ++e->last_graph_captures;
        CUDA_TRY(cudaGraphLaunch(gc.exec, st));
    }
#undef CUDA_TRY_CAP
    c.in_flight = true;
    e->last_h2d += (long long)down_begin;
    e->last_d2h += 64 + (long long)(down_end - down_begin);
    return LCG_OK;
}

// The traced alignment of one pair from the staged download: the edges in
// the reference's append order and the traced arc matches into r.
lcg_status assemble(const Prep &p, const PairOff &o, const char *H, lcg_align_result &r) {
    const int *res = (const int *)(H + o.res);
    Assembler as;
    as.tok = (const int2 *)(H + o.tok);
    int nseg = res[R_NSEG];
    const int4 *segs = (const int4 *)(H + o.segs);
    if (nseg < 1 || nseg > p.tq_cap + 1) return fail(LCG_ERR_DEVICE, "bad traceback segment count");
    for (int sg = 0; sg < nseg; ++sg) {
        as.seg_am.push_back(segs[sg].x);
        as.seg_start.push_back(segs[sg].y);
        as.seg_end.push_back(segs[sg].z);
    }
    as.edges = r.edges;
    as.edge_cap = r.edges ? p.n + p.m : 0;
    as.tam = r.traced_am;
    as.tam_cap = r.traced_am ? std::min(p.n, p.m) : 0;
    as.expand(0, 0);
    if (!as.ok) return fail(LCG_ERR_DEVICE, "traceback assembly failed");
    r.num_edges = as.nedges;
    r.num_traced_am = as.ntam;
    return LCG_OK;
}

// Wait for a launched chunk, check its status and assemble its alignments.
lcg_status chunk_finish(lcg_engine e, const Slot &s, const lcg_align_opts *opts, Chunk &c,
                        lcg_align_result *all_results, double *wait_ms, double *results_ms) {
    const auto t0 = std::chrono::steady_clock::now();
    c.in_flight = false;
    CUDA_TRY(cudaStreamSynchronize(s.st));
    const auto t1 = std::chrono::steady_clock::now();
    *wait_ms += ms_between(t0, t1);
    const char *H = *s.h_stage;
    float ms = 0, ms1 = 0;
    CUDA_TRY(cudaEventElapsedTime(&ms, s.ev0, s.ev2));
    CUDA_TRY(cudaEventElapsedTime(&ms1, s.ev0, s.ev1));
    e->last_ms += ms;
    e->last_fill_ms += ms1;
    e->last_trace_ms += ms - ms1;
    e->last_launches += c.launches;
    for (auto &p : c.prep) {
        e->last_groups += (long long)p.groups.size() - 1;
        e->last_cells += p.cells;
    }
    if (e->counting) {
        const unsigned long long *cn = (const unsigned long long *)(H + c.off_ctrl + 16);
        e->last_terms = std::max(e->last_terms, 0ll) + (long long)cn[0];
        e->last_visits = std::max(e->last_visits, 0ll) + (long long)cn[1];
    }
    int hstatus = ((const int *)(H + c.off_ctrl))[1];
    if (hstatus & ST_TIMEOUT) return fail(LCG_ERR_TIMEOUT, "a device wait for an arc-match entry timed out");
    if (hstatus & ST_OVERFLOW) return fail(LCG_ERR_DEVICE, "traceback buffer overflow");
    if (hstatus & ST_INTERNAL) return fail(LCG_ERR_DEVICE, "traceback found no predecessor");

    for (int q = 0; q < c.nq; ++q) {
        const auto &p = c.prep[q];
        const PairOff &o = c.off[q];
        const int *res = (const int *)(H + o.res);
        lcg_align_result &r = all_results[c.q0 + q];
        int sc = res[R_SCORE];
        r.score = sc < MIN_FINITE ? LCG_NEG_INF : (int64_t)sc;
        if (opts->normalized) r.score = c.ratio[q];  // the normalized score (aligner.cc:1587)
        const bool traced = opts->do_trace || opts->normalized || opts->penalized;
        r.max_i = res[R_MAXI];
        r.max_j = res[R_MAXJ];
        r.min_i = traced ? res[R_MINI] : 1;
        r.min_j = traced ? res[R_MINJ] : 1;
        r.num_edges = 0;
        r.num_traced_am = 0;
        if (!traced) continue;
        lcg_status as = assemble(p, o, H, r);
        if (as != LCG_OK) return as;
    }
    *results_ms += ms_between(t1, std::chrono::steady_clock::now());
    return LCG_OK;
}

// the second buffer set: its stream and events
lcg_status ensure_alt(lcg_engine e) {
    lcg_buffer_set &b = e->alt;
    if (b.stream) return LCG_OK;
    CUDA_TRY(cudaStreamCreateWithFlags(&b.stream, cudaStreamNonBlocking));
    b.own_stream = true;
    CUDA_TRY(cudaEventCreate(&b.ev0));
    CUDA_TRY(cudaEventCreate(&b.ev1));
    CUDA_TRY(cudaEventCreate(&b.ev2));
    return LCG_OK;
}

}  // namespace

// ------------------------------------------------------------------ engine

extern "C" {

const char *lcg_last_error(void) { return g_last_error.c_str(); }

int32_t lcg_abi_version(void) { return LCG_ABI_VERSION; }

lcg_status lcg_engine_create(int32_t device, void *stream, lcg_engine *out) {
    if (!out) return fail(LCG_ERR_ARG, "out is NULL");
    *out = nullptr;
    int ndev = 0;
    CUDA_TRY(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) return fail(LCG_ERR_ARG, "no such CUDA device");
    CUDA_TRY(cudaSetDevice(device));
    auto *e = new lcg_engine_s();
    e->device = device;
    if (stream) {
        e->stream = (cudaStream_t)stream;
    } else {
        if (cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking) != cudaSuccess) {
            delete e;
            return fail(LCG_ERR_CUDA, "cudaStreamCreate failed");
        }
        e->own_stream = true;
    }
    cudaDeviceGetAttribute(&e->sms, cudaDevAttrMultiProcessorCount, device);
    cudaEventCreate(&e->ev0);
    cudaEventCreate(&e->ev1);
    cudaEventCreate(&e->ev2);
    *out = e;
    return LCG_OK;
}

lcg_status lcg_engine_destroy(lcg_engine e) {
    if (!e) return LCG_OK;
    cudaSetDevice(e->device);
    if (e->stream) cudaStreamSynchronize(e->stream);
    if (e->alt.stream) cudaStreamSynchronize(e->alt.stream);
    // the graphs first: their nodes address the buffers and record the events
    e->graph.release();
    e->alt.graph.release();
    if (e->d_arena) cudaFree(e->d_arena);
    if (e->d_scratch) cudaFree(e->d_scratch);
    if (e->h_stage) cudaFreeHost(e->h_stage);
    if (e->ev0) cudaEventDestroy(e->ev0);
    if (e->ev1) cudaEventDestroy(e->ev1);
    if (e->ev2) cudaEventDestroy(e->ev2);
    if (e->own_stream) cudaStreamDestroy(e->stream);
    lcg_buffer_set &b = e->alt;
    if (b.stream) cudaStreamSynchronize(b.stream);
    if (b.d_arena) cudaFree(b.d_arena);
    if (b.d_scratch) cudaFree(b.d_scratch);
    if (b.h_stage) cudaFreeHost(b.h_stage);
    if (b.ev0) cudaEventDestroy(b.ev0);
    if (b.ev1) cudaEventDestroy(b.ev1);
    if (b.ev2) cudaEventDestroy(b.ev2);
    if (b.own_stream) cudaStreamDestroy(b.stream);
    if (e->env_dev) cudaFree(e->env_dev);
    if (e->env_host) cudaFreeHost(e->env_host);
    lcg_host::pf_release(e);
    delete e;
    return LCG_OK;
}

lcg_status lcg_engine_last_stats(lcg_engine e, double *kernel_ms, int64_t *launches) {
    if (!e) return fail(LCG_ERR_ARG, "engine is NULL");
    if (kernel_ms) *kernel_ms = e->last_ms;
    if (launches) *launches = e->last_launches;
    return LCG_OK;
}

lcg_status lcg_engine_last_transfer(lcg_engine e, int64_t *h2d_bytes, int64_t *d2h_bytes) {
    if (!e) return fail(LCG_ERR_ARG, "engine is NULL");
    if (h2d_bytes) *h2d_bytes = e->last_h2d;
    if (d2h_bytes) *d2h_bytes = e->last_d2h;
    return LCG_OK;
}

lcg_status lcg_engine_last_prep_transfer(lcg_engine e, int64_t *h2d_bytes, int64_t *d2h_bytes) {
    if (!e || !h2d_bytes || !d2h_bytes) return fail(LCG_ERR_ARG, "NULL argument");
    *h2d_bytes = e->prep_h2d;
    *d2h_bytes = e->prep_d2h;
    return LCG_OK;
}

lcg_status lcg_engine_last_timing(lcg_engine e, double *fill_ms, double *trace_ms) {
    if (!e) return fail(LCG_ERR_ARG, "engine is NULL");
    if (fill_ms) *fill_ms = e->last_fill_ms;
    if (trace_ms) *trace_ms = e->last_trace_ms;
    return LCG_OK;
}

lcg_status lcg_engine_set_counting(lcg_engine e, int32_t on) {
    if (!e) return fail(LCG_ERR_ARG, "engine is NULL");
    e->counting = on != 0;
    return LCG_OK;
}

lcg_status lcg_engine_last_work(lcg_engine e, lcg_work_counts *w) {
    if (!e || !w) return fail(LCG_ERR_ARG, "NULL argument");
    w->groups = e->last_groups;
    w->cells = e->last_cells;
    w->arc_terms = e->last_visits;
    w->valid_arc_terms = e->last_terms;
    return LCG_OK;
}

lcg_status lcg_pair_work(const lcg_pair_tables *pair, const lcg_align_opts *opts, lcg_work_counts *out) {
    if (!pair || !opts || !out) return fail(LCG_ERR_ARG, "NULL argument");
    lcg_host::Prep p;
    if (lcg_host::prep_pair(*pair, *opts, p) != LCG_OK) return fail(p.code, p.err);
    out->groups = (long long)p.groups.size() - 1;  // without the top level
    out->cells = p.cells;
    out->arc_terms = p.num_pos;  // arc matches whose right ends are band cells
    out->valid_arc_terms = -1;
    return LCG_OK;
}

// length buckets of the autotuner: max(len_a, len_b) <= kTuneBounds[b]
constexpr int kTuneBounds[LCG_TUNE_BUCKETS - 1] = {128, 224, 320};

static int tune_bucket(int len) {
    int b = 0;
    while (b < LCG_TUNE_BUCKETS - 1 && len > kTuneBounds[b]) ++b;
    return b;
}

// The chunk pipeline of lcg_align_pairs. ready(q0, nq), when given, is called
// before a chunk's host preparation and makes pairs[q0 .. q0+nq) valid (the
// tables of lcg_align_pp_pairs are built chunk by chunk, while the device
// aligns the previous chunk).
static lcg_status align_impl(lcg_engine e, const lcg_pair_tables *pairs, int32_t npairs, const lcg_align_opts *opts,
                             lcg_align_result *results, const std::function<lcg_status(int, int)> *ready) {
    lcg_align_result *const results_in = results;
    if (!e || !pairs || !opts || !results || npairs < 0) return fail(LCG_ERR_ARG, "NULL argument");
    if (npairs == 0) return LCG_OK;
    CUDA_TRY(cudaSetDevice(e->device));
    using clk = std::chrono::steady_clock;
    // normalized / penalized alignment: one chunk (their top levels iterate
    // with the host between launches)
    const bool modv = opts->normalized || opts->penalized;
    const int per = modv ? npairs : std::max(1, std::min<int>(npairs, chunk_size(npairs, e->chunk_pairs)));
    // the chunks: consecutive runs of at most `per` pairs; with autotune on,
    // the batch ordered by length bucket (stable) and no chunk spanning two
    // buckets, each chunk with its bucket's launch configuration
    struct Plan {
        int q0, nq, bps;
        double wave_mb;
    };
    std::vector<Plan> plan;
    std::vector<int> perm;
    std::vector<lcg_pair_tables> pairs_p;
    std::vector<lcg_align_result> results_p;
    const bool tuned = e->autotune && !modv && !ready;
    if (tuned) {
        perm.resize(npairs);
        std::vector<int> bucket(npairs);
        for (int q = 0; q < npairs; ++q) {
            perm[q] = q;
            bucket[q] = tune_bucket(std::max(pairs[q].len_a, pairs[q].len_b));
        }
        std::stable_sort(perm.begin(), perm.end(), [&](int x, int y) { return bucket[x] < bucket[y]; });
        pairs_p.resize(npairs);
        results_p.resize(npairs);
        for (int q = 0; q < npairs; ++q) {
            pairs_p[q] = pairs[perm[q]];
            results_p[q] = results[perm[q]];
        }
        for (int q0 = 0; q0 < npairs;) {
            const int b = bucket[perm[q0]];
            int q1 = q0;
            while (q1 < npairs && q1 - q0 < per && bucket[perm[q1]] == b) ++q1;
            plan.push_back({q0, q1 - q0, e->tune_bps[b], e->tune_wave_mb[b]});
            q0 = q1;
        }
        pairs = pairs_p.data();
        results = results_p.data();
    } else {
        for (int q0 = 0; q0 < npairs; q0 += per)
            plan.push_back({q0, std::min(per, npairs - q0), e->force_bps, e->force_wave_mb});
    }
    const int nchunks = (int)plan.size();
    if (nchunks > 1) {
        lcg_status st = ensure_alt(e);
        if (st != LCG_OK) return st;
    }
    e->last_ms = e->last_fill_ms = e->last_trace_ms = 0;
    e->last_launches = 0;
    e->last_h2d = e->last_d2h = 0;
    e->last_groups = e->last_cells = 0;
    e->last_terms = e->last_visits = -1;
    e->last_graph_captures = e->last_graph_replays = 0;
    double t_prep = 0, t_pack = 0, t_wait = 0, t_res = 0;

    // Pipeline over chunks of pairs on two buffer sets: the host prepares
    // chunk k while the device runs chunks k-1 (other set) and k-2 (this
    // set, finished just before its buffers are reused).
    Chunk ch[2];
    std::vector<Prep> next;
    lcg_status rc = LCG_OK;
    for (int k = 0; k < nchunks && rc == LCG_OK; ++k) {
        const int q0 = plan[k].q0, nq = plan[k].nq;
        const auto a = clk::now();
        if (ready) {
            rc = (*ready)(q0, nq);
            if (rc != LCG_OK) break;
        }
        next.clear();
        next.resize(nq);
        lcg_host::parallel_for(nq, [&](int q) { prep_pair(pairs[q0 + q], *opts, next[q]); });
        t_prep += ms_between(a, clk::now());
        for (int q = 0; q < nq && rc == LCG_OK; ++q)
            if (next[q].code != LCG_OK)
                rc = fail(next[q].code, "pair " + std::to_string(q0 + q) + ": " + next[q].err);
        if (rc != LCG_OK) break;
        Chunk &c = ch[k & 1];
        const Slot s = slot_of(e, k & 1);
        if (c.in_flight) {
            rc = chunk_finish(e, s, opts, c, results, &t_wait, &t_res);
            if (rc != LCG_OK) break;
        }
        c.prep.swap(next);
        c.q0 = q0;
        c.nq = nq;
        c.bps = plan[k].bps;
        c.wave_mb = plan[k].wave_mb;
        rc = chunk_launch(e, s, pairs, opts, c, &t_pack);
    }
    // the chunks still in flight, in batch order; after an error only wait
    // for them (nothing of the call stays in flight)
    const int first = ch[0].q0 <= ch[1].q0 ? 0 : 1;
    for (int u = 0; u < 2; ++u) {
        const int k = u == 0 ? first : 1 - first;
        const Slot s = slot_of(e, k);
        if (!s.st) continue;
        if (ch[k].in_flight && rc == LCG_OK) {
            rc = chunk_finish(e, s, opts, ch[k], results, &t_wait, &t_res);
        } else {
            cudaStreamSynchronize(s.st);
            ch[k].in_flight = false;
        }
    }
    if (rc != LCG_OK)
        for (int k = 0; k < 2; ++k)
            if (slot_of(e, k).st) cudaStreamSynchronize(slot_of(e, k).st);
    e->last_phase_ms[0] = t_prep;
    e->last_phase_ms[1] = t_pack;
    e->last_phase_ms[2] = t_wait;
    e->last_phase_ms[3] = t_res;
    if (tuned && rc == LCG_OK)
        for (int q = 0; q < npairs; ++q) results_in[perm[q]] = results_p[q];
    return rc;
}

lcg_status lcg_align_pairs(lcg_engine e, const lcg_pair_tables *pairs, int32_t npairs,
                           const lcg_align_opts *opts, lcg_align_result *results) {
    return align_impl(e, pairs, npairs, opts, results, nullptr);
}

lcg_status lcg_align_pp_pairs(lcg_engine e, const char *const *pp_a, const char *const *pp_b, int32_t npairs,
                              const lcg_prep_opts *popts, const lcg_align_opts *opts, lcg_align_result *results,
                              int32_t *host_envelopes) {
    if (!e || !pp_a || !pp_b || !opts || !results || npairs < 0) return fail(LCG_ERR_ARG, "NULL argument");
    if (npairs == 0) return LCG_OK;
    CUDA_TRY(cudaSetDevice(e->device));
    // the first chunk's envelopes are finished before its tables are built;
    // the other pairs' run on the device meanwhile
    const bool modv = opts->normalized || opts->penalized;
    const int first = modv ? npairs : std::min<int>(npairs, chunk_size(npairs, e->chunk_pairs));
    lcg_host::StagedBatch *B = nullptr;
    const auto t0 = std::chrono::steady_clock::now();
    lcg_status rc = lcg_host::stage_batch(e, pp_a, pp_b, npairs, popts, &B, host_envelopes, first);
    const double stage_ms = ms_between(t0, std::chrono::steady_clock::now());
    if (rc != LCG_OK) {
        lcg_host::free_batch(B);
        return rc;
    }
    std::vector<lcg_prepared> handles((size_t)npairs, nullptr);
    std::vector<lcg_pair_tables> tabs((size_t)npairs);
    const std::function<lcg_status(int, int)> ready = [&](int q0, int nq) {
        lcg_status r = lcg_host::finish_tables(B, q0, nq, handles.data() + q0);
        for (int q = q0; q < q0 + nq && r == LCG_OK; ++q) r = lcg_prepared_tables(handles[q], &tabs[q]);
        return r;
    };
    rc = align_impl(e, tabs.data(), npairs, opts, results, &ready);
    e->last_phase_ms[0] += stage_ms;  // host preparation includes the staging of the inputs
    for (auto h : handles)
        if (h) lcg_prepared_free(h);
    if (host_envelopes) *host_envelopes = lcg_host::batch_host_envelopes(B);
    lcg_host::free_batch(B);
    return rc;
}

lcg_status lcg_engine_set_rect_budget(lcg_engine e, int64_t bytes) {
    if (!e) return fail(LCG_ERR_ARG, "null engine");
    e->rect_budget = bytes < 0 ? -1 : bytes;
    return LCG_OK;
}

lcg_status lcg_engine_set_graphs(lcg_engine e, int32_t on) {
    if (!e) return fail(LCG_ERR_ARG, "NULL argument");
    e->graphs = on != 0;
    return LCG_OK;
}

lcg_status lcg_engine_last_graphs(lcg_engine e, int64_t *captures, int64_t *replays) {
    if (!e || !captures || !replays) return fail(LCG_ERR_ARG, "NULL argument");
    *captures = e->last_graph_captures;
    *replays = e->last_graph_replays;
    return LCG_OK;
}

lcg_status lcg_engine_set_autotune(lcg_engine e, int32_t on) {
    if (!e) return fail(LCG_ERR_ARG, "NULL argument");
    e->autotune = on != 0;
    return LCG_OK;
}

lcg_status lcg_engine_autotune(lcg_engine e, const lcg_pair_tables *pairs, int32_t npairs,
                               const lcg_align_opts *opts, int32_t sample_pairs, lcg_tune_entry *report) {
    if (!e || !pairs || !opts || npairs < 0 || sample_pairs < 0) return fail(LCG_ERR_ARG, "NULL argument");
    if (opts->normalized || opts->penalized || opts->struct_local)
        return fail(LCG_ERR_UNSUPPORTED, "the autotuner covers the plain and sequence-local fill");
    const int sample = sample_pairs > 0 ? sample_pairs : 64;
    lcg_align_opts o = *opts;
    o.do_trace = 0;
    // the grid: resident blocks per SM x wave budget (MB); the first entry
    // is the default configuration
    const int bps_grid[] = {0, 3, 2};
    const double wave_grid[] = {0, 4, 16, 64};
    const bool keep_auto = e->autotune;
    const int keep_chunk = e->chunk_pairs;
    e->autotune = false;
    lcg_status rc = LCG_OK;
    for (int b = 0; b < LCG_TUNE_BUCKETS && rc == LCG_OK; ++b) {
        std::vector<int> idx;
        for (int q = 0; q < npairs; ++q)
            if (tune_bucket(std::max(pairs[q].len_a, pairs[q].len_b)) == b) idx.push_back(q);
        lcg_tune_entry ent{};
        ent.max_len = b + 1 < LCG_TUNE_BUCKETS ? kTuneBounds[b] : INT32_MAX;
        if (idx.empty()) {
            ent.blocks_per_sm = e->tune_bps[b];
            ent.wave_mb = e->tune_wave_mb[b];
            if (report) report[b] = ent;
            continue;
        }
        std::vector<lcg_pair_tables> tb;
        const size_t step = std::max<size_t>(1, idx.size() / (size_t)sample);
        for (size_t k = 0; k < idx.size() && (int)tb.size() < sample; k += step) tb.push_back(pairs[idx[k]]);
        std::vector<lcg_align_result> res(tb.size());
        for (auto &r : res) r = lcg_align_result{};
        e->chunk_pairs = (int)tb.size();
        double best = 1e300;
        for (int bi = 0; bi < 3 && rc == LCG_OK; ++bi)
            for (int wi = 0; wi < 4 && rc == LCG_OK; ++wi) {
                e->force_bps = bps_grid[bi];
                e->force_wave_mb = wave_grid[wi];
                double ms = 1e300;
                for (int rep = 0; rep < 2 && rc == LCG_OK; ++rep) {  // the first run warms up
                    rc = lcg_align_pairs(e, tb.data(), (int32_t)tb.size(), &o, res.data());
                    if (rep == 1) ms = e->last_fill_ms;
                }
                ++ent.trials;
                if (bi == 0 && wi == 0) ent.default_ms = ms;
                if (ms < best) {
                    best = ms;
                    ent.blocks_per_sm = bps_grid[bi];
                    ent.wave_mb = wave_grid[wi];
                }
            }
        ent.best_ms = best;
        ent.pairs_sampled = (int32_t)tb.size();
        e->tune_bps[b] = ent.blocks_per_sm;
        e->tune_wave_mb[b] = ent.wave_mb;
        if (report) report[b] = ent;
    }
    e->force_bps = 0;
    e->force_wave_mb = 0;
    e->chunk_pairs = keep_chunk;
    e->autotune = keep_auto;
    return rc;
}

lcg_status lcg_align_kbest(lcg_engine e, const lcg_pair_tables *pairs, int32_t npairs, const lcg_align_opts *opts,
                           int32_t k, int64_t threshold, lcg_align_result *results, int32_t *num_hits) {
    if (!e || !pairs || !opts || !results || !num_hits || npairs < 0) return fail(LCG_ERR_ARG, "NULL argument");
    if (k < 1) return fail(LCG_ERR_ARG, "k must be >= 1");
    if (opts->penalized) return fail(LCG_ERR_UNSUPPORTED, "k-best alignment with penalized scores is not supported");
    for (int q = 0; q < npairs; ++q) num_hits[q] = 0;
    if (npairs == 0) return LCG_OK;
    CUDA_TRY(cudaSetDevice(e->device));
    e->last_ms = e->last_fill_ms = e->last_trace_ms = 0;
    e->last_launches = 0;
    e->last_h2d = e->last_d2h = 0;
    e->last_groups = e->last_cells = 0;
    e->last_terms = e->last_visits = -1;
    const bool norm = opts->normalized != 0;
    // the fill (and the whole-sequence top levels): one chunk, traced pairs
    // (PF_TRACE) but no traceback launch; normalized alignment is iterated
    // below, per interval
    lcg_align_opts o = *opts;
    o.do_trace = 1;
    o.normalized = 0;
    Chunk c;
    c.q0 = 0;
    c.nq = npairs;
    c.kbest = true;
    c.prep.resize(npairs);
    lcg_host::parallel_for(npairs, [&](int q) { prep_pair(pairs[q], *opts, c.prep[q]); });
    for (int q = 0; q < npairs; ++q)
        if (c.prep[q].code != LCG_OK) return fail(c.prep[q].code, "pair " + std::to_string(q) + ": " + c.prep[q].err);
    const Slot sl0 = slot_of(e, 0);
    double t_pack = 0, t_wait = 0, t_res = 0;
    lcg_status rc = chunk_launch(e, sl0, pairs, &o, c, &t_pack);
    if (rc != LCG_OK) return rc;
    std::vector<lcg_align_result> first(npairs);
    for (auto &r : first) std::memset(&r, 0, sizeof r);
    lcg_align_opts o_score = o;
    o_score.do_trace = 0;
    rc = chunk_finish(e, sl0, &o_score, c, first.data(), &t_wait, &t_res);
    if (rc != LCG_OK) return rc;

    char *Dv = *sl0.d_arena;
    char *H = *sl0.h_stage;
    const PairDev *dpairs = (const PairDev *)(Dv + c.off_pairs);
    int *dmod = (int *)(Dv + c.off_mod);
    int *d_lam = dmod, *d_items = dmod + npairs, *d_res1 = dmod + 2 * npairs, *d_res2 = dmod + 7 * npairs;
    int4 *d_rst = (int4 *)(dmod + 12 * npairs);
    int *status = (int *)(Dv + c.off_ctrl + 4);
    cudaStream_t st = sl0.st;
    std::vector<int> lam(npairs, 0);
    bool first_trace = true;  // the reference's min_i_/min_j_ start at 1 and then carry over between traces
    auto trace_flags = [&](int f) {
        const int r = f | (first_trace ? 0 : TRACE_KEEP_MIN);
        first_trace = false;
        return r;
    };
    auto trace_launch = [&](const TraceSel &ts) -> lcg_status {
        if (c.sl) CUDA_TRY(launch_sl_trace(dpairs, npairs, c.scratch, c.stride, c.sw, c.rb, c.sl_fast, status, st, ts));
        else CUDA_TRY(launch_trace(dpairs, npairs, c.scratch, c.stride, c.sw, c.rb, status, st, ts));
        return LCG_OK;
    };
    // The score of each listed pair's interval rr[q] (Aligner::align() or,
    // normalized, Aligner::normalized_align(), aligner.cc:1527-1588, with its
    // Dinkelbach iterations: top level with penalty lam, top-level walk for
    // the end cells, lam <- (score + length lam) / (length + L) until it
    // repeats). Afterwards the device holds each listed pair's last top level
    // and, normalized, its final lam in d_lam.
    auto evaluate = [&](const std::vector<int> &its, const std::vector<int4> &rr, int *d_res,
                        std::vector<long long> &score) -> lcg_status {
        if (its.empty()) return LCG_OK;
        std::vector<int> g(5 * its.size());
        CUDA_TRY(cudaMemcpyAsync(d_rst, rr.data(), sizeof(int4) * npairs, cudaMemcpyHostToDevice, st));
        if (!norm) {
            const int ni = (int)its.size();
            CUDA_TRY(cudaMemcpyAsync(d_items, its.data(), 4ull * ni, cudaMemcpyHostToDevice, st));
            CUDA_TRY(launch_top(dpairs, d_items, ni, nullptr, d_rst, c.rb, status, st));
            CUDA_TRY(launch_gather_res(dpairs, d_items, ni, d_res, st));
            CUDA_TRY(cudaMemcpyAsync(g.data(), d_res, 20ull * ni, cudaMemcpyDeviceToHost, st));
            CUDA_TRY(cudaStreamSynchronize(st));
            e->last_launches += 2;
            for (int t = 0; t < ni; ++t) score[its[t]] = g[5 * t] < MIN_FINITE ? LCG_NEG_INF : g[5 * t];
            return LCG_OK;
        }
        const long long L = opts->normalized_L;
        std::vector<long long> lambda(npairs, -1), nl(npairs, 0);
        std::vector<int> act = its;
        for (int iter = 0; !act.empty(); ++iter) {
            if (iter > 100000) return fail(LCG_ERR_DEVICE, "normalized alignment: Dinkelbach iterations do not converge");
            for (int q : act) {
                lambda[q] = nl[q];
                if (std::llabs(lambda[q]) * (c.prep[q].n + c.prep[q].m) >= (1ll << 26))
                    return fail(LCG_ERR_RANGE, "normalized alignment: score ratio times length exceeds the device range");
                lam[q] = (int)lambda[q];
            }
            const int ni = (int)act.size();
            CUDA_TRY(cudaMemcpyAsync(d_lam, lam.data(), 4ull * npairs, cudaMemcpyHostToDevice, st));
            CUDA_TRY(cudaMemcpyAsync(d_items, act.data(), 4ull * ni, cudaMemcpyHostToDevice, st));
            CUDA_TRY(launch_top(dpairs, d_items, ni, d_lam, d_rst, c.rb, status, st));
            TraceSel ts;
            ts.items = d_items;
            ts.nitems = ni;
            ts.lam = d_lam;
            ts.rst = d_rst;
            ts.flags = trace_flags(TRACE_TOP_ONLY);
            lcg_status tr = trace_launch(ts);
            if (tr != LCG_OK) return tr;
            CUDA_TRY(launch_gather_res(dpairs, d_items, ni, d_res, st));
            CUDA_TRY(cudaMemcpyAsync(g.data(), d_res, 20ull * ni, cudaMemcpyDeviceToHost, st));
            CUDA_TRY(cudaStreamSynchronize(st));
            e->last_launches += 3;
            std::vector<int> still;
            for (int t = 0; t < ni; ++t) {
                const int q = act[t];
                const int *r = &g[5 * t];
                if (r[R_SCORE] < MIN_FINITE) return fail(LCG_ERR_DEVICE, "normalized alignment: -inf top level");
                const long long length = (long long)(r[R_MAXI] - r[R_MINI] + 1) + (r[R_MAXJ] - r[R_MINJ] + 1);
                if (length + L <= 0)
                    return fail(LCG_ERR_ARG, "normalized alignment: empty alignment with L = 0 (division by zero)");
                nl[q] = ((long long)r[R_SCORE] + length * lambda[q]) / (length + L);
                if (nl[q] != lambda[q]) still.push_back(q);
            }
            act.swap(still);
        }
        for (int q : its) score[q] = lambda[q];
        return LCG_OK;
    };

    // Aligner::suboptimal (aligner.cc:1384-1512) per pair: a task queue of
    // (interval, score) with the reference's comparator (greater_second,
    // aligner.hh:32-44); each round pops one task per pair, aligns and traces
    // its interval, and scores the two halves of the split
    struct Task {
        int4 r;  // (sA, sB, eA, eB)
        long long score;
    };
    struct ScoreLess {
        bool operator()(const Task &a, const Task &b) const { return a.score < b.score; }
    };
    std::vector<std::priority_queue<Task, std::vector<Task>, ScoreLess>> tasks(npairs);
    std::vector<int> count(npairs, 1);  // i of the reference's loop
    std::vector<bool> done(npairs, false);
    std::vector<Task> cur(npairs);
    std::vector<int> items, split_items, all(npairs);
    std::vector<int4> rst(npairs), r1(npairs), r2(npairs);
    std::vector<long long> s0(npairs, LCG_NEG_INF), s1(npairs, LCG_NEG_INF), s2(npairs, LCG_NEG_INF);
    for (int q = 0; q < npairs; ++q) {
        all[q] = q;
        rst[q] = make_int4(1, 1, c.prep[q].n, c.prep[q].m);
        s0[q] = first[q].score;
    }
    const auto t0 = std::chrono::steady_clock::now();
    if (norm) {
        rc = evaluate(all, rst, d_res1, s0);
        if (rc != LCG_OK) return rc;
    }
    for (int q = 0; q < npairs; ++q) tasks[q].push(Task{rst[q], s0[q]});
    // an interval the top level can align (the reference leaves others undefined)
    auto valid_r = [&](int q, int4 r) {
        return r.x >= 1 && r.y >= 1 && r.z <= c.prep[q].n && r.w <= c.prep[q].m && r.z >= r.x - 1 && r.w >= r.y - 1;
    };
    for (int round = 0;; ++round) {
        items.clear();
        for (int q = 0; q < npairs; ++q) {
            if (done[q]) continue;
            // the reference reads top() of an empty queue here (undefined);
            // the enumeration ends instead
            if (tasks[q].empty()) {
                done[q] = true;
                continue;
            }
            cur[q] = tasks[q].top();
            tasks[q].pop();
            if (cur[q].score == LCG_NEG_INF || cur[q].score < (long long)threshold + 1) {
                done[q] = true;
                continue;
            }
            rst[q] = cur[q].r;
            items.push_back(q);
        }
        if (items.empty()) break;
        const int ni = (int)items.size();
        // the task's alignment: its top level (normalized: its Dinkelbach
        // iterations) and the traceback
        TraceSel ts;
        if (norm) {
            rc = evaluate(items, rst, d_res1, s0);
            if (rc != LCG_OK) return rc;
            ts.lam = d_lam;
        } else {
            CUDA_TRY(cudaMemcpyAsync(d_rst, rst.data(), sizeof(int4) * npairs, cudaMemcpyHostToDevice, st));
            CUDA_TRY(cudaMemcpyAsync(d_items, items.data(), 4ull * ni, cudaMemcpyHostToDevice, st));
            CUDA_TRY(launch_top(dpairs, d_items, ni, nullptr, d_rst, c.rb, status, st));
        }
        CUDA_TRY(cudaMemcpyAsync(d_items, items.data(), 4ull * ni, cudaMemcpyHostToDevice, st));
        ts.items = d_items;
        ts.nitems = ni;
        ts.rst = d_rst;
        ts.flags = trace_flags(0);
        rc = trace_launch(ts);
        if (rc != LCG_OK) return rc;
        CUDA_TRY(cudaMemcpyAsync(H + c.down_begin, Dv + c.down_begin, c.down_end - c.down_begin,
                                 cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaMemcpyAsync(H + c.off_ctrl, Dv + c.off_ctrl, 64, cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        e->last_launches += 2;
        e->last_d2h += (long long)(c.down_end - c.down_begin) + 64;
        const int hstatus = ((const int *)(H + c.off_ctrl))[1];
        if (hstatus & ST_OVERFLOW) return fail(LCG_ERR_DEVICE, "traceback buffer overflow");
        if (hstatus & ST_INTERNAL) return fail(LCG_ERR_DEVICE, "traceback found no predecessor");
        split_items.clear();
        for (int q : items) {
            lcg_align_result &r = results[(size_t)q * k + num_hits[q]];
            const int *res = (const int *)(H + c.off[q].res);
            rc = assemble(c.prep[q], c.off[q], H, r);
            if (rc != LCG_OK) return rc;
            if (r.num_edges == 0) continue;  // empty alignment: no hit, the count stays
            r.score = cur[q].score;
            r.max_i = res[R_MAXI];
            r.max_j = res[R_MAXJ];
            r.min_i = res[R_MINI];
            r.min_j = res[R_MINJ];
            ++num_hits[q];
            if (count[q] == k) {
                done[q] = true;
                continue;
            }
            if (!r.edges) return fail(LCG_ERR_ARG, "k-best alignment needs edge buffers");
            // Alignment::start_positions / end_positions (alignment.cc:169-195)
            int sa = c.prep[q].n, sb = c.prep[q].m, ea = 0, eb = 0;
            const int ne = std::min(r.num_edges, c.prep[q].n + c.prep[q].m);
            for (int t = 0; t < ne; ++t) if (r.edges[2 * t] >= 0) { sa = r.edges[2 * t]; break; }
            for (int t = 0; t < ne; ++t) if (r.edges[2 * t + 1] >= 0) { sb = r.edges[2 * t + 1]; break; }
            for (int t = ne - 1; t >= 0; --t) if (r.edges[2 * t] >= 0) { ea = r.edges[2 * t]; break; }
            for (int t = ne - 1; t >= 0; --t) if (r.edges[2 * t + 1] >= 0) { eb = r.edges[2 * t + 1]; break; }
            const int4 tr = cur[q].r;
            r1[q] = tr;
            r2[q] = tr;
            // the reference's interval lengths are size_t differences
            if ((unsigned long)(long)(tr.z - tr.x) > (unsigned long)(long)(tr.w - tr.y)) {
                const int split = (sa + ea) / 2;
                r1[q].z = split;
                r2[q].x = split;
            } else {
                const int split = (sb + eb) / 2;
                r1[q].w = split;
                r2[q].y = split;
            }
            split_items.push_back(q);
        }
        if (split_items.empty()) continue;
        // the scores of both halves, r1 first (the reference's order)
        std::vector<int> run1, run2;
        for (int q : split_items) {
            s1[q] = s2[q] = LCG_NEG_INF;
            if (valid_r(q, r1[q])) run1.push_back(q);
            if (valid_r(q, r2[q])) run2.push_back(q);
        }
        rc = evaluate(run1, r1, d_res1, s1);
        if (rc != LCG_OK) return rc;
        rc = evaluate(run2, r2, d_res2, s2);
        if (rc != LCG_OK) return rc;
        for (int q : split_items) {
            tasks[q].push(Task{r1[q], s1[q]});
            tasks[q].push(Task{r2[q], s2[q]});
            ++count[q];
        }
    }
    e->last_trace_ms = ms_between(t0, std::chrono::steady_clock::now());
    const int hstatus = ((const int *)(H + c.off_ctrl))[1];
    if (hstatus & ST_TIMEOUT) return fail(LCG_ERR_TIMEOUT, "a device wait for an arc-match entry timed out");
    return LCG_OK;
}

lcg_status lcg_engine_set_chunk_pairs(lcg_engine e, int32_t pairs_per_chunk) {
    if (!e) return fail(LCG_ERR_ARG, "engine is NULL");
    if (pairs_per_chunk < 0) return fail(LCG_ERR_ARG, "pairs_per_chunk < 0");
    e->chunk_pairs = pairs_per_chunk;
    return LCG_OK;
}

lcg_status lcg_engine_last_phases(lcg_engine e, double *prep_ms, double *pack_ms, double *device_ms,
                                  double *results_ms) {
    if (!e) return fail(LCG_ERR_ARG, "engine is NULL");
    if (prep_ms) *prep_ms = e->last_phase_ms[0];
    if (pack_ms) *pack_ms = e->last_phase_ms[1];
    if (device_ms) *device_ms = e->last_phase_ms[2];
    if (results_ms) *results_ms = e->last_phase_ms[3];
    return LCG_OK;
}

}  // extern "C"
