/*
 * ORACLE — test infrastructure only. Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg may load this file's library, and only as the
 * checker or the timed CPU baseline, never as the product path.
 *
 * A plain-C restatement of the reference's LocARNA-P partition-function
 * aligner (LocARNA::AlignerP<double>, src/LocARNA/aligner_p.icc) over the
 * prepared integer tables of include/locarna_gb300.h:
 *   inside      align_inside / align_D / align_inside_arcmatch (:148-438)
 *   reverse     align_reverse (:450-627)
 *   outside     align_outside / align_Dprime / align_outside_arcmatch (:761-1139)
 *   probability compute_arcmatch_probabilities (:1150-1195),
 *               compute_basematch_probabilities (:1201-1399)
 * with the Boltzmann weights of PFScoring (src/LocARNA/scoring.hh:744-931):
 * w(s) = exp(s / temperature). Arithmetic follows the reference expression by
 * expression in double (long double where the reference casts to it).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/locarna_gb300.h"

typedef double pf_t;

/* The value Mprime is filled with before each outside rectangle. The
 * reference fills -1 ("only for debugging", aligner_p.icc:921), and case 5 of
 * comp_Mprime_entry (:862-878) then reads virtual_Mprime(a.r, b.r) (:785-797)
 * at cells outside the band that no loop writes (pf150: Mprime(109, 74), band
 * of row 109 = 78..129), adding -D(am) pf_scale: the source of the
 * reference's negative and pf_scale-dependent probabilities. A build with 0
 * here gives the marginals of the reference's Z (tests/test_pf_outside_fill.py). */
#ifndef LCG_ORACLE_MPRIME_FILL
#define LCG_ORACLE_MPRIME_FILL (-1)
#endif

typedef struct {
    const lcg_pair_tables *t;
    int n, m, na, nb;
    double pf_scale;
    /* Boltzmann weights */
    pf_t *wbm;   /* (n+1)(m+1) */
    pf_t *wgA, *wgB;
    pf_t wgo;
    pf_t *wam;   /* per arc match */
    /* arc adjacency: right lists (left desc) and left lists (right asc) as
     * arc indices terminated by -1 */
    int *rA_s, *rA, *rB_s, *rB, *lA_s, *lA, *lB_s, *lB;
    int *amidx;  /* |arcsA| x |arcsB| -> am index or -1 */
    int *cle_s, *cle; /* common left end lists (creation order) */
    /* matrices */
    pf_t *D, *Dp;     /* per arc pair (dense) */
    pf_t *M, *Mrev, *Mprime, *Erev_mat, *Frev_mat;
    pf_t *E, *Erev, *Eprime;
    pf_t F, Frev, Fprime;
    pf_t Z;
    double *am_prob;  /* per am */
    double *bm_prob;  /* (n+1)(m+1) */
} P;

#define IDX(c, i, j) ((size_t)(i) * ((c)->m + 1) + (j))
#define Mx(c, i, j) ((c)->M[IDX(c, i, j)])
#define Mr(c, i, j) ((c)->Mrev[IDX(c, i, j)])
#define Mp(c, i, j) ((c)->Mprime[IDX(c, i, j)])
#define DD(c, a, b) ((c)->D[(size_t)(a) * (c)->nb + (b)])
#define DP(c, a, b) ((c)->Dp[(size_t)(a) * (c)->nb + (b)])

static inline int aL(const P *c, int k) { return c->t->arcs_a[2 * k]; }
static inline int aR(const P *c, int k) { return c->t->arcs_a[2 * k + 1]; }
static inline int bL(const P *c, int k) { return c->t->arcs_b[2 * k]; }
static inline int bR(const P *c, int k) { return c->t->arcs_b[2 * k + 1]; }
static inline int minc(const P *c, int i) { return c->t->min_col[i]; }
static inline int maxc(const P *c, int i) { return c->t->max_col[i]; }
static inline int valid(const P *c, int i, int j) { return i >= 0 && i <= c->n && minc(c, i) <= j && j <= maxc(c, i); }
static inline int valid_match(const P *c, int i, int j) { return valid(c, i, j) && valid(c, i - 1, j - 1); }
static inline size_t zmax(size_t a, size_t b) { return a > b ? a : b; }
static inline size_t zmin(size_t a, size_t b) { return a < b ? a : b; }

/* ---------------------------------------------------------------- lists */

static const int32_t *g_arcs;
static int cmp_left_desc(const void *x, const void *y) {
    return g_arcs[2 * *(const int *)y] - g_arcs[2 * *(const int *)x];
}
static int cmp_right_asc(const void *x, const void *y) {
    return g_arcs[2 * *(const int *)x + 1] - g_arcs[2 * *(const int *)y + 1];
}

/* per position lists of arc indices terminated by -1 (the sentinel) */
static void build_lists(const int32_t *arcs, int narcs, int len, int by_right, int **start, int **lst) {
    int *cnt = calloc(len + 2, sizeof(int));
    for (int k = 0; k < narcs; ++k) cnt[arcs[2 * k + by_right]]++;
    *start = malloc((len + 2) * sizeof(int));
    int acc = 0;
    for (int p = 0; p <= len; ++p) { (*start)[p] = acc; acc += cnt[p] + 1; }
    (*start)[len + 1] = acc;
    *lst = malloc((acc ? acc : 1) * sizeof(int));
    int *fill = calloc(len + 2, sizeof(int));
    for (int k = 0; k < narcs; ++k) { int p = arcs[2 * k + by_right]; (*lst)[(*start)[p] + fill[p]++] = k; }
    g_arcs = arcs;
    for (int p = 0; p <= len; ++p) {
        qsort(*lst + (*start)[p], cnt[p], sizeof(int), by_right ? cmp_left_desc : cmp_right_asc);
        (*lst)[(*start)[p] + cnt[p]] = -1;
    }
    free(cnt); free(fill);
}

/* ---------------------------------------------------------------- inside */

/* AlignerP::init_M (:149-190) */
static void init_M(P *c, size_t al, size_t ar, size_t bl, size_t br) {
    Mx(c, al, bl) = ((pf_t)1) / c->pf_scale;
    pf_t indel = c->wgo / c->pf_scale;
    size_t i;
    for (i = al + 1; i < ar; i++) {
        if ((size_t)minc(c, i) > bl) break;
        indel *= c->wgA[i];
        Mx(c, i, bl) = indel;
    }
    for (; i < ar; i++) Mx(c, i, minc(c, i) - 1) = 0;
    size_t max_col = zmin(br - 1, (size_t)maxc(c, al));
    indel = c->wgo / c->pf_scale;
    size_t j;
    for (j = bl + 1; j <= max_col; j++) {
        indel *= c->wgB[j];
        Mx(c, al, j) = indel;
    }
    for (size_t i2 = al + 1; i2 < ar; i2++)
        for (; j < zmin(br, (size_t)maxc(c, i2) + 1); ++j) Mx(c, i2 - 1, j) = 0;
}

/* align_inside_arcmatch with comp_E/F/M_entry (:209-312) */
static void align_inside_arcmatch(P *c, size_t al, size_t ar, size_t bl, size_t br) {
    init_M(c, al, ar, bl, br);
    for (size_t j = bl; j < br; j++) c->E[j] = 0;
    for (size_t i = al + 1; i < ar; i++) {
        c->F = 0;
        size_t lo = zmax(bl + 1, (size_t)minc(c, i)), hi = zmin(br - 1, (size_t)maxc(c, i));
        for (size_t j = lo; j <= hi; j++) {
            c->E[j] = c->E[j] * c->wgA[i] + (Mx(c, i - 1, j) - c->E[j]) * c->wgA[i] * c->wgo;
            c->F = c->F * c->wgB[j] + (Mx(c, i, j - 1) - c->F) * c->wgB[j] * c->wgo;
            pf_t pf = Mx(c, i - 1, j - 1) * c->wbm[IDX(c, i, j)] + c->E[j] + c->F;
            for (const int *a = c->rA + c->rA_s[i]; *a >= 0 && (size_t)aL(c, *a) > al; ++a)
                for (const int *b = c->rB + c->rB_s[j]; *b >= 0 && (size_t)bL(c, *b) > bl; ++b)
                    pf += Mx(c, aL(c, *a) - 1, bL(c, *b) - 1) * DD(c, *a, *b) * c->pf_scale;
            Mx(c, i, j) = pf;
        }
    }
}

/* align_D + fill_D (:318-407) */
static void align_D(P *c) {
    for (size_t al = c->n; al >= 1; al--) {
        size_t min_bl = zmax(1, (size_t)minc(c, al)), max_bl = zmin(c->m, (size_t)maxc(c, al));
        for (size_t bl = max_bl; bl >= min_bl && bl >= 1; bl--) {
            size_t max_ar = al, max_br = bl;
            size_t q = IDX(c, al, bl);
            for (int p = c->cle_s[q]; p < c->cle_s[q + 1]; ++p) {
                int k = c->cle[p];
                int a = c->t->am_arcs[2 * k], b = c->t->am_arcs[2 * k + 1];
                if ((size_t)aR(c, a) > max_ar) max_ar = aR(c, a);
                if ((size_t)bR(c, b) > max_br) max_br = bR(c, b);
            }
            align_inside_arcmatch(c, al, max_ar, bl, max_br);
            for (int p = c->cle_s[q]; p < c->cle_s[q + 1]; ++p) {
                int k = c->cle[p];
                int a = c->t->am_arcs[2 * k], b = c->t->am_arcs[2 * k + 1];
                size_t ar = aR(c, a), br = bR(c, b);
                if (ar > max_ar || br > max_br) DD(c, a, b) = 0;
                else DD(c, a, b) = Mx(c, ar - 1, br - 1) * c->wam[k];
            }
            if (bl == 0) break;
        }
    }
}

/* ---------------------------------------------------------------- reverse */

/* init_Mrev (:450-508) */
static void init_Mrev(P *c, size_t al, size_t ar, size_t bl, size_t br) {
    Mr(c, ar, br) = ((pf_t)1) / c->pf_scale;
    pf_t indel = c->wgo / c->pf_scale;
    size_t i;
    for (i = ar; i >= al;) {
        i--;
        if ((size_t)maxc(c, i) < br) { ++i; break; }
        indel *= c->wgA[i + 1];
        Mr(c, i, br) = indel;
    }
    for (; i >= al;) {
        i--;
        Mr(c, i, maxc(c, i) + 1) = 0;
    }
    indel = c->wgo / c->pf_scale;
    size_t min_col = zmax(bl - 1, (size_t)minc(c, ar));
    size_t j;
    for (j = br; j > min_col;) {
        j--;
        indel *= c->wgB[j + 1];
        Mr(c, ar, j) = indel;
    }
    for (size_t i2 = ar; i2 >= al;) {
        i2--;
        for (; j > zmax(bl - 1, (size_t)minc(c, i2));) {
            --j;
            Mr(c, i2 + 1, j) = 0;
        }
    }
}

/* align_reverse with comp_Erev/Frev/Mrev_entry (:521-627) */
static void align_reverse(P *c, size_t al, size_t ar, size_t bl, size_t br, int copy) {
    for (size_t i = al; i <= ar; ++i)
        for (size_t j = bl; j <= br; ++j) Mr(c, i, j) = -1;
    init_Mrev(c, al, ar, bl, br);
    for (size_t j = br; j >= bl;) { --j; c->Erev[j] = 0; }
    for (size_t i = ar; i >= al;) {
        --i;
        c->Frev = 0;
        size_t lo = zmax(bl, (size_t)minc(c, i) + 1) - 1;
        size_t hi = zmin(br, (size_t)maxc(c, i) + 1) - 1;
        for (size_t j = hi + 1; j > lo;) {
            --j;
            c->Erev[j] = c->Erev[j] * c->wgA[i + 1] + (Mr(c, i + 1, j) - c->Erev[j]) * c->wgA[i + 1] * c->wgo;
            c->Frev = c->Frev * c->wgB[j + 1] + (Mr(c, i, j + 1) - c->Frev) * c->wgB[j + 1] * c->wgo;
            if (copy) {
                c->Erev_mat[IDX(c, i, j)] = c->Erev[j];
                c->Frev_mat[IDX(c, i, j)] = c->Frev;
            }
            pf_t pf = Mr(c, i + 1, j + 1) * c->wbm[IDX(c, i + 1, j + 1)] + c->Erev[j] + c->Frev;
            for (const int *a = c->lA + c->lA_s[i + 1]; *a >= 0 && (size_t)aR(c, *a) <= ar; ++a)
                for (const int *b = c->lB + c->lB_s[j + 1]; *b >= 0 && (size_t)bR(c, *b) <= br; ++b)
                    pf += DD(c, *a, *b) * Mr(c, aR(c, *a), bR(c, *b)) * c->pf_scale;
            Mr(c, i, j) = pf;
        }
    }
}

/* ---------------------------------------------------------------- outside */

/* leftmost_covering_arc / rightmost_covering_arc (:663-735) */
static size_t leftmost_covering(const P *c, int isA, size_t start, size_t l, size_t r) {
    const int *ls = isA ? c->lA_s : c->lB_s;
    const int *lst = isA ? c->lA : c->lB;
    for (size_t i = start; i < l; ++i)
        for (const int *a = lst + ls[i]; *a >= 0; ++a)
            if ((size_t)(isA ? aR(c, *a) : bR(c, *a)) > r) return i;
    return l;
}

static size_t rightmost_covering(const P *c, int isA, size_t l, size_t r, size_t stop) {
    const int *rs = isA ? c->rA_s : c->rB_s;
    const int *lst = isA ? c->rA : c->rB;
    for (size_t i = stop + 1; i > r + 1;) {
        --i;
        const int *a = lst + rs[i];
        for (; *a >= 0 && (size_t)(isA ? aL(c, *a) : bL(c, *a)) >= l; ++a) {}
        if (*a >= 0) return i;
    }
    return r;
}

static inline pf_t virtual_Mprime(const P *c, size_t al, size_t bl, size_t i, size_t j, size_t max_ar, size_t max_br) {
    if (i >= max_ar || j >= max_br) return Mx(c, al - 1, bl - 1) * Mr(c, i, j) * c->pf_scale;
    return Mp(c, i, j);
}

/* comp_Mprime_entry (:804-886) */
static pf_t comp_Mprime_entry(P *c, size_t al, size_t bl, size_t i, size_t j, size_t max_ar, size_t max_br) {
    pf_t pf = Mp(c, i + 1, j + 1) * c->wbm[IDX(c, i + 1, j + 1)] + c->Eprime[j] + c->Fprime;
    /* case 4: arcs with right ends i+1, j+1 and left ends < al, bl, left ascending */
    {
        int sa = c->rA_s[i + 1], ea = sa; while (c->rA[ea] >= 0) ++ea;
        int sb = c->rB_s[j + 1], eb = sb; while (c->rB[eb] >= 0) ++eb;
        for (int pa = ea - 1; pa >= sa && (size_t)aL(c, c->rA[pa]) < al; --pa)
            for (int pb = eb - 1; pb >= sb && (size_t)bL(c, c->rB[pb]) < bl; --pb) {
                int a = c->rA[pa], b = c->rB[pb];
                pf += DP(c, a, b) * Mr(c, aL(c, a), bL(c, b)) * c->pf_scale;
            }
    }
    /* case 5: arcs with left ends i+1, j+1 */
    for (const int *a = c->lA + c->lA_s[i + 1]; *a >= 0; ++a)
        for (const int *b = c->lB + c->lB_s[j + 1]; *b >= 0; ++b)
            pf += virtual_Mprime(c, al, bl, aR(c, *a), bR(c, *b), max_ar, max_br) * DD(c, *a, *b) * c->pf_scale;
    return pf;
}

/* align_outside_arcmatch (:894-998) */
static void align_outside_arcmatch(P *c, size_t al, size_t ar, size_t max_ar, size_t bl, size_t br, size_t max_br) {
    size_t sA = leftmost_covering(c, 1, 1, al, ar), sB = leftmost_covering(c, 0, 1, bl, br);
    align_reverse(c, sA + 1, al - 1, sB + 1, bl - 1, 0);
    size_t cells = (size_t)(c->n + 1) * (c->m + 1);
    for (size_t q = 0; q < cells; ++q) c->Mprime[q] = LCG_ORACLE_MPRIME_FILL;
    pf_t Mal = Mx(c, al - 1, bl - 1);
    if (valid(c, max_ar, max_br)) Mp(c, max_ar, max_br) = Mal * Mr(c, max_ar, max_br) * c->pf_scale;
    size_t i;
    for (i = max_ar; i > ar;) {
        i--;
        if ((size_t)maxc(c, i) < max_br) { i++; break; }
        if (valid(c, i, max_br)) Mp(c, i, max_br) = Mal * Mr(c, i, max_br) * c->pf_scale;
    }
    for (; i > ar;) {
        i--;
        if ((size_t)maxc(c, i) + 1 <= max_br) Mp(c, i, maxc(c, i) + 1) = 0;
    }
    size_t j;
    size_t lo = zmax(br, (size_t)minc(c, max_ar)), hi = zmin(max_br - 1, (size_t)maxc(c, max_ar));
    for (j = hi + 1; j > lo;) {
        j--;
        c->Eprime[j] = Mal * c->Erev_mat[IDX(c, max_ar, j)] * c->pf_scale;
        Mp(c, max_ar, j) = Mal * Mr(c, max_ar, j) * c->pf_scale;
    }
    for (size_t i2 = max_ar; i2 > ar;) {
        i2--;
        for (; j > zmax(bl, (size_t)minc(c, i2));) {
            --j;
            Mp(c, i2 + 1, j) = 0;
            c->Eprime[j] = 0;
        }
    }
    for (size_t i2 = max_ar; i2 > ar;) {
        i2--;
        if (valid(c, i2, max_br)) c->Fprime = Mal * c->Frev_mat[IDX(c, i2, max_br)] * c->pf_scale;
        else c->Fprime = 0;
        size_t lo2 = zmax(br, (size_t)minc(c, i2)), hi2 = zmin(max_br - 1, (size_t)maxc(c, i2));
        for (size_t j2 = hi2 + 1; j2 > lo2;) {
            j2--;
            c->Fprime = c->Fprime * c->wgB[j2 + 1] + (Mp(c, i2, j2 + 1) - c->Fprime) * c->wgB[j2 + 1] * c->wgo;
            c->Eprime[j2] = c->Eprime[j2] * c->wgA[i2 + 1] + (Mp(c, i2 + 1, j2) - c->Eprime[j2]) * c->wgA[i2 + 1] * c->wgo;
            Mp(c, i2, j2) = comp_Mprime_entry(c, al, bl, i2, j2, max_ar, max_br);
        }
    }
}

/* align_Dprime + fill_Dprime (:1011-1108) */
static void align_Dprime(P *c) {
    for (size_t al = 1; al <= (size_t)c->n; al++) {
        size_t min_bl = zmax(1, (size_t)minc(c, al)), max_bl = zmin(c->m, (size_t)maxc(c, al));
        for (size_t bl = min_bl; bl <= max_bl; bl++) {
            size_t min_ar = c->n + 1, min_br = c->m + 1;
            size_t q = IDX(c, al, bl);
            for (int p = c->cle_s[q]; p < c->cle_s[q + 1]; ++p) {
                int k = c->cle[p];
                int a = c->t->am_arcs[2 * k], b = c->t->am_arcs[2 * k + 1];
                if ((size_t)aR(c, a) < min_ar) min_ar = aR(c, a);
                if ((size_t)bR(c, b) < min_br) min_br = bR(c, b);
            }
            if (min_ar > (size_t)c->n || min_br > (size_t)c->m) continue;
            size_t mA = rightmost_covering(c, 1, al, min_ar, c->n);
            size_t mB = rightmost_covering(c, 0, bl, min_br, c->m);
            align_outside_arcmatch(c, al, min_ar, mA, bl, min_br, mB);
            for (int p = c->cle_s[q]; p < c->cle_s[q + 1]; ++p) {
                int k = c->cle[p];
                int a = c->t->am_arcs[2 * k], b = c->t->am_arcs[2 * k + 1];
                size_t ar = aR(c, a), br = bR(c, b);
                if (ar < min_ar || br < min_br) DP(c, a, b) = 0;
                else DP(c, a, b) = virtual_Mprime(c, al, bl, ar, br, mA, mB) * c->wam[k];
            }
        }
    }
}

/* ---------------------------------------------------------------- probabilities */

static void arcmatch_probs(P *c) {
    for (int k = 0; k < c->t->num_arcmatches; ++k) {
        int a = c->t->am_arcs[2 * k], b = c->t->am_arcs[2 * k + 1];
        c->am_prob[k] = (double)((DD(c, a, b) / (long double)c->Z) * DP(c, a, b) * c->pf_scale / c->wam[k]);
    }
}

static void basematch_probs(P *c, double min_am_prob, int include_am) {
    double thr = sqrt(min_am_prob);
    double *amp = calloc((size_t)c->na * c->nb + 1, sizeof(double));
    for (int k = 0; k < c->t->num_arcmatches; ++k)
        amp[(size_t)c->t->am_arcs[2 * k] * c->nb + c->t->am_arcs[2 * k + 1]] = c->am_prob[k];
    for (size_t al = 1; al <= (size_t)c->n; al++) {
        size_t lo = zmax(1, (size_t)minc(c, al)), hi = zmin(c->m, (size_t)maxc(c, al));
        for (size_t bl = lo; bl <= hi; bl++) {
            if (!valid_match(c, al, bl)) continue;
            /* the reference tests the adjacency lists' sizes, which include
             * their sentinels, so every valid (al,bl) is processed */
            const int *la = c->lA + c->lA_s[al], *lb = c->lB + c->lB_s[bl];
            size_t max_ar = al, max_br = bl;
            for (const int *a = la; *a >= 0; ++a)
                for (const int *b = lb; *b >= 0; ++b)
                    if (amp[(size_t)*a * c->nb + *b] > thr) {
                        if ((size_t)aR(c, *a) > max_ar) max_ar = aR(c, *a);
                        if ((size_t)bR(c, *b) > max_br) max_br = bR(c, *b);
                    }
            align_inside_arcmatch(c, al, max_ar, bl, max_br);
            for (const int *a = la; *a >= 0; ++a)
                for (const int *b = lb; *b >= 0; ++b) {
                    if (!(amp[(size_t)*a * c->nb + *b] > thr)) continue;
                    size_t ar = aR(c, *a), br = bR(c, *b);
                    align_reverse(c, al + 1, ar - 1, bl + 1, br - 1, 0);
                    pf_t out = DP(c, *a, *b);
                    for (size_t i = al + 1; i < ar; i++) {
                        size_t l2 = zmax(bl + 1, (size_t)minc(c, i)), h2 = zmin(br - 1, (size_t)maxc(c, i));
                        for (size_t j = l2; j <= h2; j++) {
                            if (!valid_match(c, i, j)) continue;
                            c->bm_prob[IDX(c, i, j)] += Mx(c, i - 1, j - 1) * c->wbm[IDX(c, i, j)] * Mr(c, i, j) *
                                                        c->pf_scale * out * c->pf_scale;
                        }
                    }
                }
        }
    }
    align_inside_arcmatch(c, 0, c->n + 1, 0, c->m + 1);
    align_reverse(c, 1, c->n, 1, c->m, 0);
    for (size_t i = 1; i <= (size_t)c->n; i++) {
        size_t lo = zmax(1, (size_t)minc(c, i)), hi = zmin(c->m, (size_t)maxc(c, i));
        for (size_t j = lo; j <= hi; j++) {
            if (!valid_match(c, i, j)) continue;
            c->bm_prob[IDX(c, i, j)] += Mx(c, i - 1, j - 1) * c->wbm[IDX(c, i, j)] * Mr(c, i, j) * c->pf_scale;
        }
    }
    for (size_t i = 1; i <= (size_t)c->n; i++) {
        size_t lo = zmax(1, (size_t)minc(c, i)), hi = zmin(c->m, (size_t)maxc(c, i));
        for (size_t j = lo; j <= hi; j++) {
            if (!valid_match(c, i, j)) continue;
            c->bm_prob[IDX(c, i, j)] = c->bm_prob[IDX(c, i, j)] / c->Z;
        }
    }
    if (include_am) {
        for (int k = 0; k < c->t->num_arcmatches; ++k) {
            int a = c->t->am_arcs[2 * k], b = c->t->am_arcs[2 * k + 1];
            c->bm_prob[IDX(c, aL(c, a), bL(c, b))] += c->am_prob[k];
            c->bm_prob[IDX(c, aR(c, a), bR(c, b))] += c->am_prob[k];
        }
    }
    free(amp);
}

/* ---------------------------------------------------------------- entry */

/*
 * LocARNA-P on one pair (AlignerP<double>): partition function Z
 * (align_inside), arc-match probabilities (am_prob, per arc match, reference
 * order) and base-match probabilities (bm_prob, (len_a+1)*(len_b+1)
 * row-major), as computed by src/locarna_p.cc:466-531.
 * Returns 0, or -1 on allocation failure.
 */
int lcg_oracle_pf(const lcg_pair_tables *t, double temperature, double pf_scale, double min_am_prob,
                  int include_am_in_bm, double *Z_out, double *am_prob, double *bm_prob) {
    P c;
    memset(&c, 0, sizeof c);
    c.t = t;
    c.n = t->len_a;
    c.m = t->len_b;
    c.na = t->num_arcs_a;
    c.nb = t->num_arcs_b;
    c.pf_scale = pf_scale;
    size_t cells = (size_t)(c.n + 1) * (c.m + 1);
    size_t nd = (size_t)c.na * c.nb;
    c.wbm = calloc(cells, sizeof(pf_t));
    c.wgA = calloc(c.n + 2, sizeof(pf_t));
    c.wgB = calloc(c.m + 2, sizeof(pf_t));
    c.wam = calloc(t->num_arcmatches + 1, sizeof(pf_t));
    c.D = calloc(nd + 1, sizeof(pf_t));
    c.Dp = calloc(nd + 1, sizeof(pf_t));
    c.M = calloc(cells, sizeof(pf_t));
    c.Mrev = calloc(cells, sizeof(pf_t));
    c.Mprime = calloc(cells, sizeof(pf_t));
    c.Erev_mat = calloc(cells, sizeof(pf_t));
    c.Frev_mat = calloc(cells, sizeof(pf_t));
    c.E = calloc(c.m + 2, sizeof(pf_t));
    c.Erev = calloc(c.m + 2, sizeof(pf_t));
    c.Eprime = calloc(c.m + 2, sizeof(pf_t));
    c.am_prob = am_prob;
    c.bm_prob = bm_prob;
    if (!c.wbm || !c.D || !c.Dp || !c.M || !c.Mrev || !c.Mprime || !c.Erev_mat || !c.Frev_mat) return -1;
    /* PFScoring::boltzmann_weight(s) = exp(s / (pf_score_t)temperature) */
    for (int i = 1; i <= c.n; ++i)
        for (int j = 1; j <= c.m; ++j) c.wbm[IDX(&c, i, j)] = exp((pf_t)t->sigma[IDX(&c, i, j)] / (pf_t)temperature);
    for (int i = 1; i <= c.n; ++i) c.wgA[i] = exp((pf_t)t->gap_a[i] / (pf_t)temperature);
    for (int j = 1; j <= c.m; ++j) c.wgB[j] = exp((pf_t)t->gap_b[j] / (pf_t)temperature);
    c.wgo = exp((pf_t)t->indel_opening / (pf_t)temperature);
    for (int k = 0; k < t->num_arcmatches; ++k) c.wam[k] = exp((pf_t)t->am_score[k] / (pf_t)temperature);
    build_lists(t->arcs_a, c.na, c.n, 1, &c.rA_s, &c.rA);
    build_lists(t->arcs_b, c.nb, c.m, 1, &c.rB_s, &c.rB);
    build_lists(t->arcs_a, c.na, c.n, 0, &c.lA_s, &c.lA);
    build_lists(t->arcs_b, c.nb, c.m, 0, &c.lB_s, &c.lB);
    /* common left end lists in creation order */
    c.cle_s = calloc(cells + 1, sizeof(int));
    c.cle = malloc((t->num_arcmatches + 1) * sizeof(int));
    for (int k = 0; k < t->num_arcmatches; ++k)
        c.cle_s[IDX(&c, aL(&c, t->am_arcs[2 * k]), bL(&c, t->am_arcs[2 * k + 1])) + 1]++;
    for (size_t q = 0; q < cells; ++q) c.cle_s[q + 1] += c.cle_s[q];
    int *fill = calloc(cells + 1, sizeof(int));
    for (int k = 0; k < t->num_arcmatches; ++k) {
        size_t q = IDX(&c, aL(&c, t->am_arcs[2 * k]), bL(&c, t->am_arcs[2 * k + 1]));
        c.cle[c.cle_s[q] + fill[q]++] = k;
    }
    free(fill);

    /* inside */
    align_D(&c);
    align_inside_arcmatch(&c, 0, c.n + 1, 0, c.m + 1);
    c.Z = Mx(&c, c.n, c.m);
    if (Z_out) *Z_out = c.Z;
    /* outside */
    if (am_prob || bm_prob) {
        align_reverse(&c, 1, c.n, 1, c.m, 1);
        align_Dprime(&c);
        double *amp_local = am_prob ? am_prob : calloc(t->num_arcmatches + 1, sizeof(double));
        c.am_prob = amp_local;
        arcmatch_probs(&c);
        if (bm_prob) {
            memset(bm_prob, 0, cells * sizeof(double));
            basematch_probs(&c, min_am_prob, include_am_in_bm);
        }
        if (!am_prob) free(amp_local);
    }
    free(c.wbm); free(c.wgA); free(c.wgB); free(c.wam); free(c.D); free(c.Dp); free(c.M); free(c.Mrev);
    free(c.Mprime); free(c.Erev_mat); free(c.Frev_mat); free(c.E); free(c.Erev); free(c.Eprime);
    free(c.rA_s); free(c.rA); free(c.rB_s); free(c.rB); free(c.lA_s); free(c.lA); free(c.lB_s); free(c.lB);
    free(c.cle_s); free(c.cle);
    return 0;
}
