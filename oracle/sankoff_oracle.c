/*
 * ORACLE — test infrastructure only. Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg may load this file's library, and only as the
 * checker or the timed CPU baseline, never as the product path.
 *
 * A plain-C restatement of the reference's sparsified Sankoff aligner
 * (LocARNA::AlignerImpl, src/LocARNA/aligner.cc) over the prepared tables of
 * include/locarna_gb300.h. Scores use the reference's InftyInt semantics in
 * 64 bits (src/LocARNA/infty_int.hh:56-480, infty_int.cc:7-23): values below
 * LONG_MIN/5 are negative infinity and are normalised to LONG_MIN/5*2 whenever
 * they are stored, while sums and maxima in flight stay un-normalised
 * ("tainted"), exactly as in align_noex.
 *
 * The M matrices are allocated once and reused across left-end groups without
 * clearing, as in the reference (aligner.cc:118-131), so that any read of a
 * cell the current group did not write would give the same (stale) value the
 * reference sees. With LCG_ORACLE_CHECK_READS the oracle counts such reads.
 */
#include <limits.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/locarna_gb300.h"

typedef int64_t sc_t;
#define MIN_FINITY (LONG_MIN / 5)
#define NEG_INF (LONG_MIN / 5 * 2)

static inline sc_t norm(sc_t x) { return x < MIN_FINITY ? NEG_INF : x; }
static inline sc_t smax(sc_t a, sc_t b) { return a > b ? a : b; }

/* structure-local states, aligner_impl.hh:113-122 */
enum { E_NO_NO, E_X_NO, E_NO_X, E_X_X, E_OP_NO, E_NO_OP, E_OP_X, E_X_OP };

typedef struct {
    const lcg_pair_tables *t;
    const lcg_align_opts *o;
    int n, m;
    /* adjacency: right_adj_x[pos] = list of arc indices with right end pos,
     * sorted by left end descending, sentinel left 0 (basepairs.cc:110-122,212-220) */
    int *radjA_start, *radjA; /* CSR, each list followed by -1 sentinel */
    int *radjB_start, *radjB;
    /* common left end lists (creation order) and common right end lists
     * (sorted lex greater left ends), CSR over (n+1)*(m+1) */
    int *cle_start, *cle;
    int *cre_start, *cre;
    int *inner;    /* per arc match: the inner arc match, or -1 */
    /* ModifiedScoringView (aligner_impl.hh:190-275): with mod set, sigma -
     * 2 lam, gaps - lam and D(a,b) - lam (|a| + |b|) (Scoring::
     * modify_by_parameter, scoring.cc:77-90); used by the top level of
     * normalized and penalized alignment */
    sc_t lam;
    int lam_on, mod;
    /* AlignerRestriction (aligner_restriction.hh): the top level aligns
     * A[rsA..reA] with B[rsB..reB] (default: the whole sequences) */
    int rsA, rsB, reA, reB;
    /* restricted top levels read M cells outside the band in their final
     * argmax (see top_free_endgaps); count of reads where that changed the
     * result, which then follows the defined rule */
    int stale_argmax;
    sc_t *D;       /* |arcsA| x |arcsB| */
    sc_t *M[8];    /* (n+1) x (m+1) */
    sc_t *E[4];    /* m+1 */
    sc_t F[4];
    int max_i, max_j, min_i, min_j;
    /* trace output */
    int32_t *edges; int nedges, edge_cap;
    int32_t *tam; int ntam, tam_cap;
    lcg_work_counts *cnt;
} Ctx;

#define MM(c, s, i, j) ((c)->M[s][(size_t)(i) * ((c)->m + 1) + (j)])
#define DD(c, a, b) ((c)->D[(size_t)(a) * (c)->t->num_arcs_b + (b)])

static inline int arcL(const int32_t *arcs, int k) { return arcs[2 * k]; }
static inline int arcR(const int32_t *arcs, int k) { return arcs[2 * k + 1]; }

static inline int minc(const Ctx *c, int i) { return c->t->min_col[i]; }
static inline int maxc(const Ctx *c, int i) { return c->t->max_col[i]; }
static inline int valid(const Ctx *c, int i, int j) {
    return i >= 0 && i <= c->n && minc(c, i) <= j && j <= maxc(c, i);
}
static inline int valid_match(const Ctx *c, int i, int j) { return valid(c, i, j) && valid(c, i - 1, j - 1); }
static inline int a_match(const Ctx *c, int i, int j) {
    return !c->t->match_lo || (c->t->match_lo[i] <= j && j <= c->t->match_hi[i]);
}
static inline int a_del(const Ctx *c, int i, int j) {
    return !c->t->del_lo || (c->t->del_lo[i] <= j && j <= c->t->del_hi[i]);
}
static inline int a_ins(const Ctx *c, int i, int j) {
    return !c->t->ins_lo || (c->t->ins_lo[j] <= i && i <= c->t->ins_hi[j]);
}
static inline sc_t sigma(const Ctx *c, int i, int j) { return c->t->sigma[(size_t)i * (c->m + 1) + j]; }
static inline sc_t sigma_v(const Ctx *c, int i, int j) { return sigma(c, i, j) - (c->mod ? 2 * c->lam : 0); }
static inline sc_t gapA_v(const Ctx *c, int i) { return c->t->gap_a[i] - (c->mod ? c->lam : 0); }
static inline sc_t gapB_v(const Ctx *c, int j) { return c->t->gap_b[j] - (c->mod ? c->lam : 0); }
/* the scoring view of the current trace level: modified on the top level */
static inline void set_view(Ctx *c, int tl) { c->mod = tl && c->lam_on; }

/* Scoring::stacking() (scoring.hh:653) */
static inline int stacking(const Ctx *c) { return c->t->am_stack_score != NULL; }
/* Scoring::arcmatch(am, true); LCG_STACK_NONE (a score outside the table
 * range, only from an undefined zero-probability weight) as -infinity */
static inline sc_t stack_score(const Ctx *c, int k) {
    int32_t v = c->t->am_stack_score[k];
    return v <= LCG_STACK_NONE ? NEG_INF : v;
}
/* Scoring::arcmatch(am, scoring->stacking()) */
static inline sc_t am_score_st(const Ctx *c, int k) { return stacking(c) ? stack_score(c, k) : c->t->am_score[k]; }

/* ---------------------------------------------------------------- setup */

static int *g_sort_arcs; /* qsort context (single-threaded use per call) */
static int cmp_left_desc(const void *x, const void *y) {
    int a = *(const int *)x, b = *(const int *)y;
    return g_sort_arcs[2 * b] - g_sort_arcs[2 * a];
}

/* right adjacency lists (basepairs.cc:110-122, 212-220): per right end, the
 * arcs sorted by left end descending, followed by a sentinel with left end 0;
 * stored as (arc index, left end) pairs */
static void build_radj(const int32_t *arcs, int narcs, int len, int **start, int **lst) {
    int *cntv = calloc(len + 2, sizeof(int));
    for (int k = 0; k < narcs; ++k) cntv[arcR(arcs, k)]++;
    *start = malloc((len + 2) * sizeof(int));
    int acc = 0;
    for (int p = 0; p <= len; ++p) { (*start)[p] = acc; acc += cntv[p] + 1; }
    (*start)[len + 1] = acc;
    int *tmp = malloc((acc > 0 ? acc : 1) * sizeof(int));
    int *fill = calloc(len + 2, sizeof(int));
    for (int k = 0; k < narcs; ++k) { int r = arcR(arcs, k); tmp[(*start)[r] + fill[r]++] = k; }
    g_sort_arcs = (int *)arcs;
    *lst = malloc(2 * (acc > 0 ? acc : 1) * sizeof(int));
    for (int p = 0; p <= len; ++p) {
        qsort(tmp + (*start)[p], cntv[p], sizeof(int), cmp_left_desc);
        for (int q = 0; q < cntv[p]; ++q) {
            int k = tmp[(*start)[p] + q];
            (*lst)[2 * ((*start)[p] + q)] = k;
            (*lst)[2 * ((*start)[p] + q) + 1] = arcL(arcs, k);
        }
        (*lst)[2 * ((*start)[p] + cntv[p])] = -1;
        (*lst)[2 * ((*start)[p] + cntv[p]) + 1] = 0;
    }
    free(tmp); free(cntv); free(fill);
}

static const Ctx *g_sort_ctx;
static int cmp_lex_greater_left(const void *x, const void *y) {
    const Ctx *c = g_sort_ctx;
    int i = *(const int *)x, j = *(const int *)y;
    int ali = arcL(c->t->arcs_a, c->t->am_arcs[2 * i]), bli = arcL(c->t->arcs_b, c->t->am_arcs[2 * i + 1]);
    int alj = arcL(c->t->arcs_a, c->t->am_arcs[2 * j]), blj = arcL(c->t->arcs_b, c->t->am_arcs[2 * j + 1]);
    if (ali != alj) return ali > alj ? -1 : 1;
    if (bli != blj) return bli > blj ? -1 : 1;
    return 0;
}

static void build_am_lists(Ctx *c) {
    int n = c->n, m = c->m, na = c->t->num_arcmatches;
    size_t cells = (size_t)(n + 1) * (m + 1);
    int *cl = calloc(cells + 1, sizeof(int)), *cr = calloc(cells + 1, sizeof(int));
    for (int k = 0; k < na; ++k) {
        int a = c->t->am_arcs[2 * k], b = c->t->am_arcs[2 * k + 1];
        cl[(size_t)arcL(c->t->arcs_a, a) * (m + 1) + arcL(c->t->arcs_b, b)]++;
        cr[(size_t)arcR(c->t->arcs_a, a) * (m + 1) + arcR(c->t->arcs_b, b)]++;
    }
    c->cle_start = malloc((cells + 1) * sizeof(int));
    c->cre_start = malloc((cells + 1) * sizeof(int));
    int al = 0, ar = 0;
    for (size_t q = 0; q < cells; ++q) {
        c->cle_start[q] = al; al += cl[q];
        c->cre_start[q] = ar; ar += cr[q];
    }
    c->cle_start[cells] = al; c->cre_start[cells] = ar;
    c->cle = malloc((na > 0 ? na : 1) * sizeof(int));
    c->cre = malloc((na > 0 ? na : 1) * sizeof(int));
    memset(cl, 0, (cells + 1) * sizeof(int));
    memset(cr, 0, (cells + 1) * sizeof(int));
    for (int k = 0; k < na; ++k) {
        int a = c->t->am_arcs[2 * k], b = c->t->am_arcs[2 * k + 1];
        size_t ql = (size_t)arcL(c->t->arcs_a, a) * (m + 1) + arcL(c->t->arcs_b, b);
        size_t qr = (size_t)arcR(c->t->arcs_a, a) * (m + 1) + arcR(c->t->arcs_b, b);
        c->cle[c->cle_start[ql] + cl[ql]++] = k;
        c->cre[c->cre_start[qr] + cr[qr]++] = k;
    }
    g_sort_ctx = c;
    for (size_t q = 0; q < cells; ++q) {
        int s = c->cre_start[q], e = c->cre_start[q + 1];
        if (e - s > 1) qsort(c->cre + s, e - s, sizeof(int), cmp_lex_greater_left);
    }
    free(cl); free(cr);
}

/* ---------------------------------------------------------------- DP */

/* AlignerImpl::align_noex, aligner.cc:153-233 */
static sc_t align_noex(Ctx *c, int state, int al, int bl, int i, int j) {
    sc_t *E = c->E[state];
    sc_t max_score = NEG_INF;
    if (a_match(c, i, j)) max_score = MM(c, state, i - 1, j - 1) + sigma_v(c, i, j);
    if (a_del(c, i, j)) {
        E[j] = norm(smax(E[j] + gapA_v(c, i), MM(c, state, i - 1, j) + gapA_v(c, i) + c->t->indel_opening));
        max_score = smax(max_score, E[j]);
    } else {
        E[j] = NEG_INF;
    }
    if (a_ins(c, i, j)) {
        c->F[state] = norm(smax(c->F[state] + gapB_v(c, j), MM(c, state, i, j - 1) + gapB_v(c, j) + c->t->indel_opening));
        max_score = smax(max_score, c->F[state]);
    } else {
        c->F[state] = NEG_INF;
    }
    if (a_match(c, i, j)) {
        /* adjacency entries carry (arc index, left end); the sentinel has left end 0 */
        const int *la = c->radjA + 2 * c->radjA_start[i];
        const int *lb0 = c->radjB + 2 * c->radjB_start[j];
        const int nb = c->t->num_arcs_b;
        const size_t mp = (size_t)c->m + 1;
        const sc_t *Ms = c->M[state];
        for (; la[1] > al; la += 2) {
            const sc_t *Drow = c->D + (size_t)la[0] * nb;
            const sc_t *Mrow = Ms + (size_t)(la[1] - 1) * mp - 1;
            for (const int *lb = lb0; lb[1] > bl; lb += 2) {
                sc_t d = Drow[lb[0]];
                if (c->mod) d -= c->lam * ((i - la[1] + 1) + (j - lb[1] + 1));
                if (c->cnt) {
                    c->cnt->arc_terms++;
                    if (d != NEG_INF) c->cnt->valid_arc_terms++;
                }
                sc_t ns = Mrow[lb[1]] + d;
                if (ns <= max_score) continue;
                max_score = ns;
            }
        }
    }
    return max_score;
}

/* AlignerImpl::init_state, aligner.cc:264-368 */
static void init_state(Ctx *c, int state, int al, int ar, int bl, int br,
                       int globalA, int exclA, int globalB, int exclB) {
    if (state < 4) {
        for (int j = bl; j < br; ++j) c->E[state][j] = NEG_INF;
    }
    MM(c, state, al, bl) = 0;
    sc_t indel = c->t->indel_opening;
    if (exclA) indel = c->t->exclusion;
    else if (!globalA) indel = 0;
    int i;
    for (i = al + 1; i < ar; ++i) {
        if (minc(c, i) > bl) break;
        if (indel != NEG_INF) {
            if (!a_del(c, i, bl)) indel = NEG_INF;
            else if (!exclA && globalA) indel = norm(indel + gapA_v(c, i));
        }
        MM(c, state, i, bl) = indel;
    }
    for (; i < ar; ++i) MM(c, state, i, minc(c, i) - 1) = NEG_INF;

    indel = c->t->indel_opening;
    if (exclB) indel = c->t->exclusion;
    else if (!globalB) indel = 0;
    int j;
    int lim = maxc(c, al) + 1 < br ? maxc(c, al) + 1 : br;
    for (j = bl + 1; j < lim; ++j) {
        if (indel != NEG_INF) {
            if (!a_ins(c, al, j)) indel = NEG_INF;
            else if (!exclB && globalB) indel = norm(indel + gapB_v(c, j));
        }
        MM(c, state, al, j) = indel;
    }
    for (i = al + 1; i < ar; ++i) {
        int l2 = maxc(c, i) + 1 < br ? maxc(c, i) + 1 : br;
        for (; j < l2; ++j) MM(c, state, i - 1, j) = NEG_INF;
    }
}

static inline int imax(int a, int b) { return a > b ? a : b; }
static inline int imin(int a, int b) { return a < b ? a : b; }

/* AlignerImpl::align_in_arcmatch, aligner.cc:373-565 */
static void align_in_arcmatch(Ctx *c, int al, int ar, int bl, int br, int excl, int count) {
    init_state(c, E_NO_NO, al, ar, bl, br, 1, 0, 1, 0);
    if (excl) {
        init_state(c, E_X_NO, al, ar, bl, br, 1, 1, 1, 0);
        init_state(c, E_NO_X, al, ar, bl, br, 1, 0, 1, 1);
        init_state(c, E_X_X, al, ar, bl, br, 1, 1, 1, 1);
        init_state(c, E_OP_NO, al, ar, bl, br, 0, 0, 1, 0);
        init_state(c, E_NO_OP, al, ar, bl, br, 1, 0, 0, 0);
        init_state(c, E_X_OP, al, ar, bl, br, 1, 1, 0, 0);
        init_state(c, E_OP_X, al, ar, bl, br, 0, 0, 1, 1);
    }
    for (int i = al + 1; i < ar; ++i) {
        c->F[E_NO_NO] = NEG_INF;
        int lo = imax(bl + 1, minc(c, i)), hi = imin(br - 1, maxc(c, i));
        for (int j = lo; j <= hi; ++j) {
            MM(c, E_NO_NO, i, j) = norm(align_noex(c, E_NO_NO, al, bl, i, j));
            if (count && c->cnt) c->cnt->cells++;
        }
    }
    if (!excl) return;
    sc_t X = c->t->exclusion;
#define ROWS_BEGIN for (int i = al + 1; i < ar; ++i) { int lo = imax(bl + 1, minc(c, i)), hi = imin(br - 1, maxc(c, i));
#define ROWS_END }
    ROWS_BEGIN for (int j = lo; j <= hi; ++j)
        MM(c, E_OP_NO, i, j) = norm(smax(!a_del(c, i, j) ? NEG_INF : MM(c, E_OP_NO, i - 1, j), MM(c, E_NO_NO, i, j)));
    ROWS_END
    ROWS_BEGIN for (int j = lo; j <= hi; ++j)
        MM(c, E_NO_OP, i, j) = norm(smax(!a_ins(c, i, j) ? NEG_INF : MM(c, E_NO_OP, i, j - 1), MM(c, E_NO_NO, i, j)));
    ROWS_END
    ROWS_BEGIN c->F[E_NO_X] = NEG_INF; for (int j = lo; j <= hi; ++j)
        MM(c, E_NO_X, i, j) = norm(smax(align_noex(c, E_NO_X, al, bl, i, j), MM(c, E_NO_OP, i, j) + X));
    ROWS_END
    ROWS_BEGIN for (int j = lo; j <= hi; ++j)
        MM(c, E_OP_X, i, j) = norm(smax(!a_del(c, i, j) ? NEG_INF : MM(c, E_OP_X, i - 1, j), MM(c, E_NO_X, i, j)));
    ROWS_END
    ROWS_BEGIN c->F[E_X_NO] = NEG_INF; for (int j = lo; j <= hi; ++j)
        MM(c, E_X_NO, i, j) = norm(smax(align_noex(c, E_X_NO, al, bl, i, j), MM(c, E_OP_NO, i, j) + X));
    ROWS_END
    ROWS_BEGIN for (int j = lo; j <= hi; ++j)
        MM(c, E_X_OP, i, j) = norm(smax(!a_ins(c, i, j) ? NEG_INF : MM(c, E_X_OP, i, j - 1), MM(c, E_X_NO, i, j)));
    ROWS_END
    ROWS_BEGIN c->F[E_X_X] = NEG_INF; for (int j = lo; j <= hi; ++j)
        MM(c, E_X_X, i, j) = norm(smax(align_noex(c, E_X_X, al, bl, i, j),
                                       smax(MM(c, E_OP_X, i, j) + X, MM(c, E_X_OP, i, j) + X)));
    ROWS_END
#undef ROWS_BEGIN
#undef ROWS_END
}

/* AlignerImpl::fill_D_entries, aligner.cc:574-610; with stacking the arc
 * match may also stack on its inner arc match (:600-608) */
static void fill_D_entries(Ctx *c, int al, int bl) {
    size_t q = (size_t)al * (c->m + 1) + bl;
    for (int p = c->cle_start[q]; p < c->cle_start[q + 1]; ++p) {
        int k = c->cle[p];
        int a = c->t->am_arcs[2 * k], b = c->t->am_arcs[2 * k + 1];
        int ar = arcR(c->t->arcs_a, a), br = arcR(c->t->arcs_b, b);
        sc_t mv = MM(c, 0, ar - 1, br - 1);
        if (c->o->struct_local)
            for (int s = 1; s < 4; ++s) mv = smax(mv, MM(c, s, ar - 1, br - 1));
        sc_t d = mv + c->t->am_score[k];
        int in = c->inner ? c->inner[k] : -1;
        if (stacking(c) && in >= 0 && c->t->am_stackable[k]) {
            int ia = c->t->am_arcs[2 * in], ib = c->t->am_arcs[2 * in + 1];
            d = smax(d, DD(c, ia, ib) + stack_score(c, k));
        }
        DD(c, a, b) = norm(d);
    }
}

/* AlignerImpl::fill_D_entries_noLP, aligner.cc:612-657: the arc matches
 * with left ends (al-1,bl-1) that enclose an inner arc match (left ends
 * (al,bl), right ends one less; with stacking, only stackable ones) take the
 * better of the inner arc match's own D and the inner interior plus the
 * inner arc-match score, plus their own (stacked) score */
static void fill_D_entries_noLP(Ctx *c, int al, int bl) {
    size_t q = (size_t)(al - 1) * (c->m + 1) + (bl - 1);
    for (int p = c->cle_start[q]; p < c->cle_start[q + 1]; ++p) {
        int k = c->cle[p];
        int in = c->inner[k];
        if (in < 0 || (stacking(c) && !c->t->am_stackable[k])) continue;
        int a = c->t->am_arcs[2 * k], b = c->t->am_arcs[2 * k + 1];
        int ar = arcR(c->t->arcs_a, a) - 1, br = arcR(c->t->arcs_b, b) - 1;
        sc_t mv = MM(c, 0, ar - 1, br - 1);
        if (c->o->struct_local)
            for (int s = 1; s < 4; ++s) mv = smax(mv, MM(c, s, ar - 1, br - 1));
        int ia = c->t->am_arcs[2 * in], ib = c->t->am_arcs[2 * in + 1];
        DD(c, a, b) = norm(smax(mv + c->t->am_score[in], DD(c, ia, ib)) + am_score_st(c, k));
    }
}

/* ArcMatches::init_inner_arc_matchs, arc_matches.cc:50-74: the first arc
 * match (in creation order) with left ends (a.l+1,b.l+1) and right ends
 * (a.r-1,b.r-1), or -1 */
static void init_inner(Ctx *c) {
    int na = c->t->num_arcmatches;
    c->inner = malloc((na > 0 ? na : 1) * sizeof(int));
    for (int k = 0; k < na; ++k) {
        int a = c->t->am_arcs[2 * k], b = c->t->am_arcs[2 * k + 1];
        int al = arcL(c->t->arcs_a, a), ar = arcR(c->t->arcs_a, a);
        int bl = arcL(c->t->arcs_b, b), br = arcR(c->t->arcs_b, b);
        c->inner[k] = -1;
        if (al + 1 > c->n || bl + 1 > c->m) continue;
        size_t q = (size_t)(al + 1) * (c->m + 1) + (bl + 1);
        for (int p = c->cle_start[q]; p < c->cle_start[q + 1]; ++p) {
            int x = c->cle[p];
            if (arcR(c->t->arcs_a, c->t->am_arcs[2 * x]) == ar - 1 &&
                arcR(c->t->arcs_b, c->t->am_arcs[2 * x + 1]) == br - 1) {
                c->inner[k] = x;
                break;
            }
        }
    }
}

/* AlignerImpl::align_D, aligner.cc:660-732; group extents by
 * ArcMatches::get_max_right_ends, arc_matches.cc:313-355 */
static void align_D(Ctx *c) {
    const int nolp = c->o->no_lonely_pairs;
    for (int al = c->n; al >= 1; --al) {
        int max_bl = imin(c->m, maxc(c, al));
        int min_bl = imax(1, minc(c, al));
        for (int bl = max_bl; bl >= min_bl; --bl) {
            if (!(a_match(c, al, bl) && valid_match(c, al, bl))) continue;
            int max_ar = al, max_br = bl;
            /* without lonely pairs: the arc matches that start at
             * (al-1,bl-1) and enclose an inner arc match, right ends minus one */
            size_t q = nolp ? (size_t)(al - 1) * (c->m + 1) + (bl - 1) : (size_t)al * (c->m + 1) + bl;
            if (nolp) { max_ar++; max_br++; }
            for (int p = c->cle_start[q]; p < c->cle_start[q + 1]; ++p) {
                int k = c->cle[p];
                if (nolp && c->inner[k] < 0) continue;
                max_ar = imax(max_ar, arcR(c->t->arcs_a, c->t->am_arcs[2 * k]));
                max_br = imax(max_br, arcR(c->t->arcs_b, c->t->am_arcs[2 * k + 1]));
            }
            if (nolp) { max_ar--; max_br--; }
            if (al == max_ar || bl == max_br) continue;
            if (c->cnt) c->cnt->groups++;
            align_in_arcmatch(c, al, max_ar, bl, max_br, c->o->struct_local, 1);
            if (nolp) fill_D_entries_noLP(c, al, bl);
            else fill_D_entries(c, al, bl);
        }
    }
}

/* align_top_level_free_endgaps, aligner.cc:736-819 */
static sc_t top_free_endgaps(Ctx *c) {
    int fe = c->o->free_endgaps;
    int sA = c->rsA, sB = c->rsB, n = c->reA, m = c->reB;  /* the restriction */
    init_state(c, E_NO_NO, sA - 1, n + 1, sB - 1, m + 1, !(fe & LCG_FREE_LEFT_2), 0, !(fe & LCG_FREE_LEFT_1), 0);
    for (int i = sA; i <= n; ++i) {
        c->F[E_NO_NO] = NEG_INF;
        int lo = imax(sB, minc(c, i)), hi = imin(m, maxc(c, i));
        for (int j = lo; j <= hi; ++j) {
            MM(c, E_NO_NO, i, j) = norm(align_noex(c, E_NO_NO, sA - 1, sB - 1, i, j));
            if (c->cnt) c->cnt->cells++;
        }
    }
    /* The final argmax reads M(n,m) and, with free right end gaps, column m
     * of every row whose band reaches m (aligner.cc:771-799). For an interval
     * of k-best alignment these cells can lie outside the band, where the
     * reference's reused M holds whatever earlier computations left
     * (aligner.cc:118-131). Such a cell counts as -inf here (the rule the GPU
     * follows); the reference's value is still evaluated, and a difference in
     * the outcome is counted in stale_argmax. On the whole sequences every
     * cell read is in the band. */
    int origin_nm = (n == sA - 1 && m == sB - 1);
    sc_t best = (valid(c, n, m) || origin_nm) ? MM(c, E_NO_NO, n, m) : NEG_INF;
    sc_t best_ref = MM(c, E_NO_NO, n, m);
    c->max_i = n; c->max_j = m;
    int ri = n, rj = m;
    if (fe & (LCG_FREE_RIGHT_1 | LCG_FREE_RIGHT_2)) {
        best = NEG_INF; c->max_i = sA - 1; c->max_j = sB - 1;
        best_ref = NEG_INF; ri = sA - 1; rj = sB - 1;
    }
    int ra = c->t->right_anchor_a, rb = c->t->right_anchor_b;
    if (fe & LCG_FREE_RIGHT_2) {
        for (int i = imax(ra + 1, sA); i <= n; ++i) {
            if (maxc(c, i) < m) continue;
            if (minc(c, i) <= m && MM(c, E_NO_NO, i, m) > best) { best = MM(c, E_NO_NO, i, m); c->max_i = i; c->max_j = m; }
            if (MM(c, E_NO_NO, i, m) > best_ref) { best_ref = MM(c, E_NO_NO, i, m); ri = i; rj = m; }
        }
    }
    if (fe & LCG_FREE_RIGHT_1) {
        int lo = imax(imax(rb + 1, sB), minc(c, n)), hi = imin(m, maxc(c, n));
        for (int j = lo; j <= hi; ++j) {
            if (MM(c, E_NO_NO, n, j) > best) { best = MM(c, E_NO_NO, n, j); c->max_i = n; c->max_j = j; }
            if (MM(c, E_NO_NO, n, j) > best_ref) { best_ref = MM(c, E_NO_NO, n, j); ri = n; rj = j; }
        }
    }
    if (norm(best_ref) != norm(best) || ri != c->max_i || rj != c->max_j) c->stale_argmax++;
    return best;
}

/* align_top_level_locally, aligner.cc:823-880 */
static sc_t top_locally(Ctx *c) {
    int sA = c->rsA, sB = c->rsB, n = c->reA, m = c->reB;  /* the restriction */
    sc_t best = 0;
    c->max_i = sA - 1; c->max_j = sB - 1;
    init_state(c, E_NO_NO, sA - 1, n + 1, sB - 1, m + 1, 0, 0, 0, 0);
    int ra = c->t->right_anchor_a, rb = c->t->right_anchor_b;
    int la = c->t->left_anchor_a, lb = c->t->left_anchor_b;
    for (int i = sA; i <= n; ++i) {
        c->F[E_NO_NO] = NEG_INF;
        int lo = imax(sB, minc(c, i)), hi = imin(m, maxc(c, i));
        for (int j = lo; j <= hi; ++j) {
            sc_t v = norm(align_noex(c, E_NO_NO, sA - 1, sB - 1, i, j));
            if (i < la && j < lb) v = smax(0, v);
            MM(c, E_NO_NO, i, j) = v;
            if (c->cnt) c->cnt->cells++;
            if (i >= ra && j >= rb && best < v) { best = v; c->max_i = i; c->max_j = j; }
        }
    }
    return best;
}

/* ---------------------------------------------------------------- trace */

static void append(Ctx *c, int a, int b) {
    if (c->nedges < c->edge_cap) { c->edges[2 * c->nedges] = a; c->edges[2 * c->nedges + 1] = b; }
    c->nedges++;
}

static void trace_in_arcmatch(Ctx *c, int state, int al, int i, int bl, int j, int tl);

/* AlignerImpl::trace_arcmatch, aligner.cc:967-1028 */
static void trace_arcmatch(Ctx *c, int k) {
    c->mod = 0;
    int a = c->t->am_arcs[2 * k], b = c->t->am_arcs[2 * k + 1];
    int al = arcL(c->t->arcs_a, a), ar = arcR(c->t->arcs_a, a);
    int bl = arcL(c->t->arcs_b, b), br = arcR(c->t->arcs_b, b);
    int in = c->inner ? c->inner[k] : -1;
    if (stacking(c) && in >= 0) {
        /* stacked on the inner arc match (aligner.cc:986-1006) */
        int ia = c->t->am_arcs[2 * in], ib = c->t->am_arcs[2 * in + 1];
        if (DD(c, a, b) == DD(c, ia, ib) + stack_score(c, k)) {
            if (c->ntam < c->tam_cap) c->tam[c->ntam] = in;
            c->ntam++;
            append(c, arcL(c->t->arcs_a, ia), arcL(c->t->arcs_b, ib));
            trace_arcmatch(c, in);
            append(c, arcR(c->t->arcs_a, ia), arcR(c->t->arcs_b, ib));
            return;
        }
    }
    align_in_arcmatch(c, al, ar, bl, br, c->o->struct_local, 0);
    if (!c->o->struct_local) {
        trace_in_arcmatch(c, 0, al, ar - 1, bl, br - 1, 0);
    } else {
        for (int s = 0; s < 4; ++s) {
            if (DD(c, a, b) == MM(c, s, ar - 1, br - 1) + c->t->am_score[k]) {
                trace_in_arcmatch(c, s, al, ar - 1, bl, br - 1, 0);
                break;
            }
        }
    }
}

/* AlignerImpl::trace_arcmatch_noLP, aligner.cc:1030-1079:
 * the inner arc match is part of the alignment; below it, either the inner
 * arc match's own stack continues (D(am) = D(inner) + score(am)) or its
 * interior is recomputed and traced */
static void trace_arcmatch_noLP(Ctx *c, int k) {
    c->mod = 0;
    int in = c->inner[k];
    int a = c->t->am_arcs[2 * k], b = c->t->am_arcs[2 * k + 1];
    int ia = c->t->am_arcs[2 * in], ib = c->t->am_arcs[2 * in + 1];
    int ial = arcL(c->t->arcs_a, ia), iar = arcR(c->t->arcs_a, ia);
    int ibl = arcL(c->t->arcs_b, ib), ibr = arcR(c->t->arcs_b, ib);
    if (c->ntam < c->tam_cap) c->tam[c->ntam] = in;
    c->ntam++;
    append(c, ial, ibl);
    if (DD(c, a, b) == DD(c, ia, ib) + am_score_st(c, k)) {
        trace_arcmatch_noLP(c, in);
    } else {
        align_in_arcmatch(c, ial, iar, ibl, ibr, c->o->struct_local, 0);
        if (!c->o->struct_local) {
            trace_in_arcmatch(c, 0, ial, iar - 1, ibl, ibr - 1, 0);
        } else {
            for (int s = 0; s < 4; ++s) {
                if (DD(c, a, b) == MM(c, s, iar - 1, ibr - 1) + am_score_st(c, k) + c->t->am_score[in]) {
                    trace_in_arcmatch(c, s, ial, iar - 1, ibl, ibr - 1, 0);
                    break;
                }
            }
        }
    }
    append(c, iar, ibr);
}

/* AlignerImpl::trace_noex, aligner.cc:1082-1229 */
static void trace_noex(Ctx *c, int state, int oal, int i, int obl, int j, int tl) {
    set_view(c, tl);
    sc_t Mij = MM(c, state, i, j);
    if (a_match(c, i, j) && valid(c, i - 1, j - 1) && Mij == MM(c, state, i - 1, j - 1) + sigma_v(c, i, j)) {
        trace_in_arcmatch(c, state, oal, i - 1, obl, j - 1, tl);
        append(c, i, j);
        return;
    }
    if (c->t->indel_opening == 0) {
        if (a_del(c, i, j) && valid(c, i - 1, j) && Mij == MM(c, state, i - 1, j) + gapA_v(c, i)) {
            trace_in_arcmatch(c, state, oal, i - 1, obl, j, tl);
            append(c, i, -1);
            return;
        }
        if (a_ins(c, i, j) && valid(c, i, j - 1) && Mij == MM(c, state, i, j - 1) + gapB_v(c, j)) {
            trace_in_arcmatch(c, state, oal, i, obl, j - 1, tl);
            append(c, -1, j);
            return;
        }
    } else {
        sc_t gap = c->t->indel_opening;
        for (int k = 1; i >= oal + k && a_del(c, i - k + 1, j); ++k) {
            if (!valid(c, i - k, j)) break;
            gap += gapA_v(c, i - k + 1);
            if (Mij == MM(c, state, i - k, j) + gap) {
                trace_in_arcmatch(c, state, oal, i - k, obl, j, tl);
                for (int l = k; l > 0; --l) append(c, i - l + 1, -1);
                return;
            }
        }
        gap = c->t->indel_opening;
        for (int k = 1; j >= obl + k && a_ins(c, i, j - k + 1); ++k) {
            if (!valid(c, i, j - k)) break;
            gap += gapB_v(c, j - k + 1);
            if (Mij == MM(c, state, i, j - k) + gap) {
                trace_in_arcmatch(c, state, oal, i, obl, j - k, tl);
                for (int l = k; l > 0; --l) append(c, -1, j - l + 1);
                return;
            }
        }
    }
    if (!(a_match(c, i, j) && valid(c, i - 1, j - 1))) return;
    size_t q = (size_t)i * (c->m + 1) + j;
    for (int p = c->cre_start[q]; p < c->cre_start[q + 1]; ++p) {
        int k = c->cre[p];
        int a = c->t->am_arcs[2 * k], b = c->t->am_arcs[2 * k + 1];
        int al = arcL(c->t->arcs_a, a), bl = arcL(c->t->arcs_b, b);
        if (al <= oal || bl <= obl) continue;
        sc_t dv = DD(c, a, b) - (c->mod ? c->lam * ((i - al + 1) + (j - bl + 1)) : 0);
        if (Mij == MM(c, state, al - 1, bl - 1) + dv) {
            trace_in_arcmatch(c, state, oal, al - 1, obl, bl - 1, tl);
            if (c->ntam < c->tam_cap) c->tam[c->ntam] = k;
            c->ntam++;
            append(c, al, bl);
            if (c->o->no_lonely_pairs) trace_arcmatch_noLP(c, k);
            else trace_arcmatch(c, k);
            append(c, i, j);
            return;
        }
    }
}

/* AlignerImpl::trace_in_arcmatch, aligner.cc:1233-1343 */
static void trace_in_arcmatch(Ctx *c, int state, int al, int i, int bl, int j, int tl) {
    set_view(c, tl);
    sc_t Mij = MM(c, state, i, j);
    if (tl && c->o->sequ_local && Mij == 0) { c->min_i = i; c->min_j = j; return; }
    int fe = c->o->free_endgaps;
    if (i <= al) {
        if (state == E_NO_NO || state == E_OP_NO || state == E_X_NO) {
            if (!(tl && (c->o->sequ_local || (fe & LCG_FREE_LEFT_1))))
                for (int k = bl + 1; k <= j; ++k) append(c, -1, k);
        }
        return;
    }
    if (j <= bl) {
        if (state == E_NO_NO || state == E_NO_OP || state == E_NO_X) {
            if (!(tl && (c->o->sequ_local || (fe & LCG_FREE_LEFT_2))))
                for (int k = al + 1; k <= i; ++k) append(c, k, -1);
        }
        return;
    }
    sc_t X = c->t->exclusion;
    switch (state) {
    case E_NO_NO: trace_noex(c, state, al, i, bl, j, tl); break;
    case E_OP_NO:
        if (Mij == MM(c, state, i - 1, j)) trace_in_arcmatch(c, state, al, i - 1, bl, j, tl);
        else if (Mij == MM(c, E_NO_NO, i, j)) trace_in_arcmatch(c, E_NO_NO, al, i, bl, j, tl);
        break;
    case E_NO_OP:
        if (Mij == MM(c, state, i, j - 1)) trace_in_arcmatch(c, state, al, i, bl, j - 1, tl);
        else if (Mij == MM(c, E_NO_NO, i, j)) trace_in_arcmatch(c, E_NO_NO, al, i, bl, j, tl);
        break;
    case E_NO_X:
        if (Mij == MM(c, E_NO_OP, i, j) + X) trace_in_arcmatch(c, E_NO_OP, al, i, bl, j, tl);
        else trace_noex(c, state, al, i, bl, j, tl);
        break;
    case E_OP_X:
        if (Mij == MM(c, state, i - 1, j)) trace_in_arcmatch(c, state, al, i - 1, bl, j, tl);
        else if (Mij == MM(c, E_NO_X, i, j)) trace_in_arcmatch(c, E_NO_X, al, i, bl, j, tl);
        break;
    case E_X_NO:
        if (Mij == MM(c, E_OP_NO, i, j) + X) trace_in_arcmatch(c, E_OP_NO, al, i, bl, j, tl);
        else trace_noex(c, state, al, i, bl, j, tl);
        break;
    case E_X_OP:
        if (Mij == MM(c, state, i, j - 1)) trace_in_arcmatch(c, state, al, i, bl, j - 1, tl);
        else if (Mij == MM(c, E_X_NO, i, j)) trace_in_arcmatch(c, E_X_NO, al, i, bl, j, tl);
        break;
    case E_X_X:
        if (Mij == MM(c, E_OP_X, i, j) + X) trace_in_arcmatch(c, E_OP_X, al, i, bl, j, tl);
        else if (Mij == MM(c, E_X_OP, i, j) + X) trace_in_arcmatch(c, E_X_OP, al, i, bl, j, tl);
        else trace_noex(c, state, al, i, bl, j, tl);
        break;
    }
}

/* AlignerImpl::normalized_align, aligner.cc:1527-1588: Dinkelbach iterations
 * of the top level (under the current restriction); each traces, and
 * min_i/min_j carry over when a trace does not reach a zero cell, as the
 * reference's members do. The score is the final ratio; the edges of the last
 * trace stay in the context's buffers. Returns -2 on a zero denominator. */
static int normalized_align(Ctx *c, sc_t *score) {
    sc_t lambda = -1, new_lambda = 0;
    c->lam_on = 1;
    while (lambda != new_lambda) {
        lambda = new_lambda;
        c->lam = lambda;
        c->mod = 1;
        sc_t s = top_locally(c);
        c->nedges = 0; c->ntam = 0;
        trace_in_arcmatch(c, E_NO_NO, c->rsA - 1, c->max_i, c->rsB - 1, c->max_j, 1);
        sc_t length = (sc_t)(c->max_i - c->min_i + 1) + (c->max_j - c->min_j + 1);
        s += length * lambda;
        if (length + c->o->normalized_L <= 0) return -2;
        new_lambda = s / (length + c->o->normalized_L);
    }
    c->lam_on = 0;
    c->mod = 0;
    *score = new_lambda;
    return 0;
}

/* ---------------------------------------------------------------- entry */

static void ctx_free(Ctx *c) {
    free(c->radjA_start); free(c->radjA); free(c->radjB_start); free(c->radjB);
    free(c->cle_start); free(c->cle); free(c->cre_start); free(c->cre);
    free(c->D); free(c->inner);
    for (int s = 0; s < 8; ++s) free(c->M[s]);
    for (int s = 0; s < 4; ++s) free(c->E[s]);
}

/*
 * Align one pair: Aligner::align() and, if opts->do_trace, Aligner::trace()
 * (aligner.cc:924-957, 1345-1358). Returns 0, or -1 on allocation failure.
 * counts may be NULL.
 */
int lcg_oracle_align(const lcg_pair_tables *t, const lcg_align_opts *o,
                     lcg_align_result *r, lcg_work_counts *counts) {
    Ctx c;
    memset(&c, 0, sizeof c);
    c.t = t; c.o = o; c.n = t->len_a; c.m = t->len_b; c.cnt = counts;
    if (counts) memset(counts, 0, sizeof *counts);
    build_radj(t->arcs_a, t->num_arcs_a, c.n, &c.radjA_start, &c.radjA);
    build_radj(t->arcs_b, t->num_arcs_b, c.m, &c.radjB_start, &c.radjB);
    build_am_lists(&c);
    if (o->no_lonely_pairs || t->am_stack_score) init_inner(&c);
    size_t nd = (size_t)t->num_arcs_a * t->num_arcs_b;
    c.D = malloc((nd > 0 ? nd : 1) * sizeof(sc_t));
    for (size_t q = 0; q < nd; ++q) c.D[q] = NEG_INF;
    int ns = o->struct_local ? 8 : 1;
    size_t cells = (size_t)(c.n + 1) * (c.m + 1);
    for (int s = 0; s < ns; ++s) c.M[s] = calloc(cells, sizeof(sc_t));
    for (int s = 0; s < (o->struct_local ? 4 : 1); ++s) c.E[s] = calloc(c.m + 1, sizeof(sc_t));
    for (int s = 0; s < 8; ++s) if (!c.M[s]) c.M[s] = NULL;
    if (!c.D || !c.M[0]) { ctx_free(&c); return -1; }
    c.min_i = 1; c.min_j = 1; c.max_i = c.n; c.max_j = c.m;
    c.rsA = 1; c.rsB = 1; c.reA = c.n; c.reB = c.m;

    align_D(&c);
    c.edges = r->edges; c.edge_cap = r->edges ? c.n + c.m : 0;
    c.tam = r->traced_am; c.tam_cap = r->traced_am ? (c.n < c.m ? c.n : c.m) : 0;
    sc_t score;
    int traced = 0;
    if (o->normalized) {
        if (normalized_align(&c, &score) != 0) { ctx_free(&c); return -2; }
        traced = 1;
    } else if (o->penalized) {
        /* AlignerImpl::penalized_align, aligner.cc:1597-1617 */
        c.lam_on = 1;
        c.lam = o->position_penalty;
        c.mod = 1;
        score = o->sequ_local ? top_locally(&c) : top_free_endgaps(&c);
        trace_in_arcmatch(&c, E_NO_NO, c.rsA - 1, c.max_i, c.rsB - 1, c.max_j, 1);
        traced = 1;
    } else {
        score = o->sequ_local ? top_locally(&c) : top_free_endgaps(&c);
    }
    r->score = score < MIN_FINITY ? LCG_NEG_INF : score;
    r->num_edges = 0; r->num_traced_am = 0;
    if (o->do_trace && !traced) trace_in_arcmatch(&c, E_NO_NO, c.rsA - 1, c.max_i, c.rsB - 1, c.max_j, 1);
    if (o->do_trace || traced) { r->num_edges = c.nedges; r->num_traced_am = c.ntam; }
    r->max_i = c.max_i; r->max_j = c.max_j; r->min_i = c.min_i; r->min_j = c.min_j;
    ctx_free(&c);
    return 0;
}

/* ---------------------------------------------------------------- k-best
 *
 * A context for Aligner::suboptimal (aligner.cc:1384-1512, driven by
 * oracle/kbest_oracle.cc): D is filled once for the whole sequences (the
 * first align() of an Aligner), then the top level and its trace run again
 * per restriction, as set_restriction() + align() + trace() do.
 */
void *lcg_oracle_ctx_new(const lcg_pair_tables *t, const lcg_align_opts *o) {
    Ctx *c = calloc(1, sizeof(Ctx));
    if (!c) return NULL;
    c->t = t; c->o = o; c->n = t->len_a; c->m = t->len_b;
    build_radj(t->arcs_a, t->num_arcs_a, c->n, &c->radjA_start, &c->radjA);
    build_radj(t->arcs_b, t->num_arcs_b, c->m, &c->radjB_start, &c->radjB);
    build_am_lists(c);
    if (o->no_lonely_pairs || t->am_stack_score) init_inner(c);
    size_t nd = (size_t)t->num_arcs_a * t->num_arcs_b;
    c->D = malloc((nd > 0 ? nd : 1) * sizeof(sc_t));
    for (size_t q = 0; q < nd; ++q) c->D[q] = NEG_INF;
    size_t cells = (size_t)(c->n + 1) * (c->m + 1);
    for (int s = 0; s < (o->struct_local ? 8 : 1); ++s) c->M[s] = calloc(cells, sizeof(sc_t));
    for (int s = 0; s < (o->struct_local ? 4 : 1); ++s) c->E[s] = calloc(c->m + 1, sizeof(sc_t));
    c->min_i = 1; c->min_j = 1; c->max_i = c->n; c->max_j = c->m;
    c->rsA = 1; c->rsB = 1; c->reA = c->n; c->reB = c->m;
    align_D(c);
    return c;
}

/* Aligner::set_restriction + align(): the score of the top level restricted
 * to A[sA..eA], B[sB..eB] (LCG_NEG_INF for -inf) */
long long lcg_oracle_ctx_top(void *ctx, int sA, int sB, int eA, int eB) {
    Ctx *c = ctx;
    c->rsA = sA; c->rsB = sB; c->reA = eA; c->reB = eB;
    sc_t s = c->o->sequ_local ? top_locally(c) : top_free_endgaps(c);
    return s < MIN_FINITY ? LCG_NEG_INF : s;
}

/* Aligner::set_restriction + normalized_align(L): the ratio of the interval;
 * its last trace goes to r as in lcg_oracle_ctx_trace. -2 on a zero
 * denominator. */
int lcg_oracle_ctx_normalized(void *ctx, int sA, int sB, int eA, int eB, lcg_align_result *r, long long *score) {
    Ctx *c = ctx;
    c->rsA = sA; c->rsB = sB; c->reA = eA; c->reB = eB;
    c->edges = r ? r->edges : NULL; c->edge_cap = (r && r->edges) ? c->n + c->m : 0;
    c->tam = r ? r->traced_am : NULL; c->tam_cap = (r && r->traced_am) ? (c->n < c->m ? c->n : c->m) : 0;
    sc_t s;
    if (normalized_align(c, &s) != 0) return -2;
    *score = s;
    if (r) {
        r->num_edges = c->nedges; r->num_traced_am = c->ntam;
        r->max_i = c->max_i; r->max_j = c->max_j; r->min_i = c->min_i; r->min_j = c->min_j;
    }
    return 0;
}

/* Aligner::trace() of the last top level: edges, traced arc matches and end
 * cells into r (capacities as for lcg_oracle_align) */
void lcg_oracle_ctx_trace(void *ctx, lcg_align_result *r) {
    Ctx *c = ctx;
    c->edges = r->edges; c->edge_cap = r->edges ? c->n + c->m : 0; c->nedges = 0;
    c->tam = r->traced_am; c->tam_cap = r->traced_am ? (c->n < c->m ? c->n : c->m) : 0; c->ntam = 0;
    trace_in_arcmatch(c, E_NO_NO, c->rsA - 1, c->max_i, c->rsB - 1, c->max_j, 1);
    r->num_edges = c->nedges; r->num_traced_am = c->ntam;
    r->max_i = c->max_i; r->max_j = c->max_j; r->min_i = c->min_i; r->min_j = c->min_j;
}

/* number of restricted top levels whose argmax the reference would have
 * taken from a cell outside the band (see top_free_endgaps) */
int lcg_oracle_ctx_stale(void *ctx) { return ((Ctx *)ctx)->stale_argmax; }

void lcg_oracle_ctx_free(void *ctx) {
    if (!ctx) return;
    ctx_free((Ctx *)ctx);
    free(ctx);
}
