// Device-side data layout of the GB300 Sankoff engine.
//
// One batch = many independent sequence pairs. Every per-pair table lives in
// one device arena; PairDev holds device pointers into it. The work list is a
// flat array of GroupItem, one per left-end group (al,bl) of the reference's
// align_D (src/LocARNA/aligner.cc:660-732) plus one top-level item per pair
// (aligner.cc:736-880), in an order where every group comes after all groups
// whose D entries it reads (per pair: al descending, then bl descending, as
// the reference iterates).
#pragma once
#include <stdint.h>

namespace lcg {

// Scores are int32 with the reference's InftyInt semantics
// (src/LocARNA/infty_int.hh:56-480) scaled down: finite values satisfy
// |v| < 2^27 (checked on the host), every value below MIN_FINITE is negative
// infinity, and stored values are normalised to NEG. Sums of up to four
// stored values never overflow int32.
constexpr int NEG = -(1 << 29);
constexpr int MIN_FINITE = -(1 << 28);
// D entries not yet written by their producer group (a D wait spins on this)
constexpr int NOT_READY = INT32_MIN;

__host__ __device__ __forceinline__ int norm(int v) { return v < MIN_FINITE ? NEG : v; }

enum PairFlags : int {
    PF_STRUCT_LOCAL = 1,
    PF_SEQU_LOCAL = 2,
    PF_ANCHORS = 4,
    PF_TRACE = 8,
    PF_SCLS = 16,  // sigma(i,j) = scls[rcls[i] * 16 + ccls[j]] (at most 16 row / column classes)
    PF_NOLP = 32,  // no lonely pairs (AlignerParams::no_lonely_pairs)
    PF_STACK = 64, // stacking terms (Scoring::stacking())
};

// status word bits (device -> host)
enum StatusBits : int {
    ST_TIMEOUT = 1,     // a bounded D wait gave up
    ST_OVERFLOW = 2,    // a token / queue buffer would overflow
    ST_INTERNAL = 4,    // traceback found no predecessor
};

struct GroupItem;

struct PairDev {
    int n, m;
    int go, excl;
    int flags;       // PairFlags
    int free_endgaps;
    int la, lb, ra, rb;  // leftmost / rightmost anchor
    int num_am;
    int bandcells;
    int maxband;          // widest band row (columns)
    const int *sigma;     // (n+1)*(m+1)
    const int *scls;      // PF_SCLS: 256-entry class table of sigma
    const int *rcls;      // PF_SCLS: n+2 row classes
    const int *ccls;      // PF_SCLS: m+1 column classes
    const int *gbc;       // m+1: gap term << 4 | sigma column class (0 without PF_SCLS); the gap
                          // term is gapB(j) with anchors, else the prefix sum sum_{t<=j} (gapB(t) + max(go,0))
    const int *gapA;      // n+1
    const int *gapB;      // m+1
    const int *min_col;   // n+2 (entry n+1 = m+1 sentinel)
    const int *max_col;   // n+2
    const int *bandoff;   // n+2: band cell offset of row i
    const int4 *rowinfo;  // n+2: (min_col, max_col, gapA, bandoff) of row i
    const int *match_lo, *match_hi, *del_lo, *del_hi, *ins_lo, *ins_hi;
    const int *cre_start; // bandcells+1: arc matches with right ends at a band cell
    const int4 *cre;      // (D index, a.l-1, b.l-1, am), lex-greater-left-ends order
    const int2 *crow;     // the same arc matches by row a.r, then a.l descending, b.l descending:
                          // ((a.l-1) | (b.l-1) << 16, b.r); the position is the D index
    const int2 *rowarc;   // n+2: [start, end) of row i's entries in crow
    int *D;               // num_pos, by crow position
    int num_pos;
    const int *am_score;  // per am
    int *topM;            // (n+1)*(m+1), top-level M
    int *res;             // result words, see Res
    int2 *tokens;         // traceback tokens
    int token_cap;
    int4 *tq;             // traceback queue of arc matches (capacity tq_cap):
                          // (am, D index, a.l | b.l << 16, a.r | b.r << 16)
    int tq_cap;
    int4 *segs;           // traceback segments: (am or -1, token start, token end, 0)
    const GroupItem *groups;  // the pair's left-end groups (work items) in dependency order
    const int4 *dw;           // the pair's D writes; GroupItem::dw_start indexes it
    // PF_NOLP or PF_STACK (else nullptr): per D write, (D index of the inner
    // arc match or -1, a score), parallel to dw; the write is
    // D = max(M(corner) + dw.w, D(inner) + score). No lonely pairs
    // (fill_D_entries_noLP, aligner.cc:612-657): dw.w = score'(outer) +
    // score(inner), score = score'(outer), score' the stacked score with
    // PF_STACK; stacking alone (fill_D_entries, :600-608): dw.w =
    // score(outer), score = its stacked score (inner -1 unless stackable)
    const int2 *dwn;
    // PF_NOLP or PF_STACK: per arc match, (inner arc match or -1, its D index
    // or -1) (ArcMatches::inner_arc_match, arc_matches.hh:466-476)
    const int2 *inner;
    // PF_STACK: per arc match Scoring::arcmatch(am, true), NEG where the
    // tables give LCG_STACK_NONE
    const int *am_sscore;
    // Kept group rectangles (nullptr: not kept). The fill writes group g's M
    // to rect + g.rect_off (row i-al, column j-bl, pitch g.br - g.bl)
    // instead of the warp's scratch slot, and the traceback walks a traced
    // arc match on its group's rectangle instead of recomputing it; am_rect
    // holds per arc match its group's (rect_off, rect_pitch), (-1, 0) when no
    // group computes it.
    int *rect;
    const int2 *am_rect;
};

// Scoring::basematch(i,j) from the class table or the dense table
__device__ __forceinline__ int sigma_at(const PairDev &P, int i, int j) {
    return (P.flags & PF_SCLS) ? P.scls[P.rcls[i] * 16 + P.ccls[j]] : P.sigma[(size_t)i * (P.m + 1) + j];
}

// Selection and options of a traceback launch: items (NULL = every pair)
// lists the pairs to trace; lam[pair] (NULL = 0) is the top level's penalty of
// normalized / penalized alignment; TRACE_KEEP_MIN keeps the result words
// min_i/min_j unless the walk sets them (the reference's members carry over
// between the traces of Dinkelbach iterations); TRACE_TOP_ONLY walks the top
// level only (enough for the end cells).
enum TraceFlags : int { TRACE_KEEP_MIN = 1, TRACE_TOP_ONLY = 2 };
struct TraceSel {
    const int *items = nullptr;
    int nitems = 0;
    const int *lam = nullptr;
    int flags = 0;
    const int4 *rst = nullptr;  // per pair (sA, sB, eA, eB) of k-best alignment; NULL = whole sequences
};

enum Res : int {
    R_SCORE = 0, R_MAXI, R_MAXJ, R_MINI, R_MINJ, R_NTOK, R_NSEG, R_NWORDS
};

struct GroupItem {
    int pair;
    int al, ar, bl, br;
    int dw_start, dw_count;  // D writes: int4 (D index, corner row, corner column, score), rows ascending
    int top;                 // 1 for the top-level item
    int cpl;                 // columns per lane: ceil(widest band row of the group / 32), <= 4
    int rect_off;            // the group's kept rectangle in PairDev::rect (pitch br - bl), when kept
};

// anchor helpers: reference AnchorConstraints::allowed_match/del/ins
// (anchor_constraints.hh:157-253)
__device__ __forceinline__ bool a_match(const PairDev &P, int i, int j) {
    return !(P.flags & PF_ANCHORS) || (P.match_lo[i] <= j && j <= P.match_hi[i]);
}
__device__ __forceinline__ bool a_del(const PairDev &P, int i, int j) {
    return !(P.flags & PF_ANCHORS) || (P.del_lo[i] <= j && j <= P.del_hi[i]);
}
__device__ __forceinline__ bool a_ins(const PairDev &P, int i, int j) {
    return !(P.flags & PF_ANCHORS) || (P.ins_lo[j] <= i && i <= P.ins_hi[j]);
}

}  // namespace lcg
