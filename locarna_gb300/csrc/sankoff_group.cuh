// Device routines shared by the plain and the structure-local Sankoff
// kernels: one left-end group's row sweep (run_group), the top level with its
// final argmax (run_top) and the traceback walk (walk). See sankoff_kernels.cu
// for the work decomposition and the dataflow protocol.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <climits>

#include "lcg_device.cuh"

namespace lcg {


// dynamic shared memory of every kernel in this family
extern __shared__ int lcg_smem[];

#ifndef LCG_FILL_WARPS
#define LCG_FILL_WARPS 8
#endif
#ifndef LCG_FILL_MIN_BLOCKS
#define LCG_FILL_MIN_BLOCKS 4
#endif
constexpr int FILL_WARPS = LCG_FILL_WARPS;  // warps per block of the fill kernel
// shared ints per warp of the row sweep for ring size rb (see run_group)
__host__ __device__ inline int smem_warp_ints(int rb) { return 5 * rb + 256; }
constexpr int FILL_MIN_BLOCKS = LCG_FILL_MIN_BLOCKS;  // resident blocks per SM the register budget targets
constexpr int TRACE_WARPS = 4;  // warps per block of the trace kernel
// polls of a bounded device wait (~ seconds), then ST_TIMEOUT; a test build
// shortens it (LCG_SPIN_LIMIT)
#ifndef LCG_SPIN_LIMIT
#define LCG_SPIN_LIMIT (1ll << 22)
#endif
constexpr long long SPIN_LIMIT = LCG_SPIN_LIMIT;

__device__ __forceinline__ int addc(int x, int y) {
    // saturating add of two values >= 2*NEG; result clamped to >= NEG
    int s = x + y;
    return s < NEG ? NEG : s;
}

__device__ __forceinline__ int ld_volatile(const int *p) {
    return *(const volatile int *)p;
}
__device__ __forceinline__ void st_volatile(int *p, int v) { *(volatile int *)p = v; }

struct TopOut {
    int best, bi, bj;
};

// Read D[k], spinning while its producer has not written it yet.
__device__ __forceinline__ int wait_D(int *D, int k, int *status, volatile int *abort_flag) {
    int v = ld_volatile(D + k);
    if (v != NOT_READY) return v;
    long long spins = 0;
    while (v == NOT_READY) {
        __nanosleep(64);
        v = ld_volatile(D + k);
        if (++spins > SPIN_LIMIT || *abort_flag) {
            atomicOr(status, ST_TIMEOUT);
            *abort_flag = 1;
            return NEG;
        }
    }
    return v;
}

// No lonely pairs or stacking: D(inner) + score for the D write *e of a
// group (PairDev::dwn, parallel to PairDev::dw); kept out of line, it is rare.
template <bool WAIT>
__device__ __noinline__ int inner_term(const PairDev &P, const int4 *e, int *status, volatile int *abort_flag) {
    const int2 x = P.dwn[e - P.dw];
    const int din = x.x < 0 ? NEG : (WAIT ? wait_D(P.D, x.x, status, abort_flag) : P.D[x.x]);
    return din + x.y;
}

// One left-end group (or the top level) in state E_NO_NO:
// init_state (aligner.cc:264-368) + the row sweep of align_in_arcmatch
// (aligner.cc:424-437) with align_noex per cell. M of the rectangle is
// written to Mg (row r = i-al, column c = j-bl, row pitch `pitch`).
// Shared-memory rows (offsets into lcg_smem) hold the previous and current M
// row, the E vector, the group's gap costs gapB and the arc-term maxima of
// the current row, indexed by c = j-bl.
//
// Per row, the arc-match terms come first: the row's candidates (arc matches
// with a.r = i, sorted by a.l descending) are read 32 at a time by the whole
// warp until the first a.l <= al; each valid term M(a.l-1,b.l-1) + D(a,b) is
// reduced into its column with a shared-memory atomicMax. The maxima row is
// -inf at the group's start, and the cell sweep puts -inf back into every
// column it reads, so no row needs a clearing pass. Then lanes own
// consecutive columns (chunks of 32) for the affine recursion; the horizontal
// gap chain is a max-plus warp scan. ANCH = false drops every anchor test and
// uses plain (non-saturating) adds: without anchors every gap term is finite,
// so no sum can leave the int32 range. MOD: the scoring view of normalized and
// penalized alignment (ModifiedScoringView, aligner_impl.hh:190-275) with
// every position penalised by lam: sigma - 2 lam, gap costs - lam, arc-match
// terms D(a,b) - lam (|a| + |b|) (the host bounds lam (n+m) below 2^27).
template <int NCH, bool ANCH, bool SCLS, bool TOP, bool WAIT, bool DWRITE, bool COUNT, bool MOD = false,
          bool INNER = true>
__device__ void run_group_c(const PairDev &P, int al, int ar, int bl, int br, int *__restrict__ Mg,
                            int pitch, int sbase, int ringn,
                            const int4 *__restrict__ dw, int ndw, bool globalA, bool globalB,
                            bool local_top, int *status, volatile int *abort_flag, TopOut *tout,
                            unsigned long long *counters, int lam = 0) {
    unsigned long long n_terms = 0, n_visits = 0;
    const int lane = threadIdx.x & 31;
    const int4 *__restrict__ rowinfo = P.rowinfo;
    const int2 *__restrict__ rowarc = P.rowarc;
    const int *__restrict__ sigma = P.sigma;
    const int2 *__restrict__ crow = P.crow;
    int *const Dp = P.D;
    const int m1 = P.m + 1;
    const int go = P.go;
    const int gop = max(go, 0);
    const unsigned rmagic = 0xFFFFFFFFu / (unsigned)ringn + 1u;  // j / ringn = umulhi(j, rmagic), j < 2^20
    int *const E = lcg_smem + sbase + 2 * ringn;
    int *const gBs = lcg_smem + sbase + 3 * ringn;   // gap term (PairDev::gbc) << 4 | sigma column class
    int *const Arow = lcg_smem + sbase + 4 * ringn;  // arc-term maxima of the current row
    int *const Stab = lcg_smem + sbase + 5 * ringn;  // SCLS: 16 x 16 sigma class table
    int pv = sbase, cu = sbase + ringn;  // shared-memory offsets of the previous / current row
#define RG(j) ((j) - ringn * (int)__umulhi((unsigned)(j), rmagic))
#define PREV(j) lcg_smem[pv + RG(j)]
#define CUR(j) lcg_smem[cu + RG(j)]
#define PREVR(r) lcg_smem[pv + (r)]  // by ring index
#define CURR(r) lcg_smem[cu + (r)]
    for (int c = lane; c < ringn; c += 32) {
        E[c] = NEG;
        Arow[c] = NEG;
    }
    if (SCLS)
        for (int k = lane; k < 256; k += 32) Stab[k] = P.scls[k];

    // ---- row al: M(al,bl)=0, M(al,j) = prefix of gap costs, -inf once blocked
    const int L0 = min(br, rowinfo[al].y + 1);
    // without anchors the column table holds the prefix sums
    // PA(j) = sum_{t<=j} (gapB(t) + gop); PA(bl) anchors the group's sums
    // MOD: the prefix sums of the penalised gap costs, PA(j) - lam j
#define PAX(gbcv, jj) (((gbcv) >> 4) - (MOD ? lam * (jj) : 0))
    const int PAbl = ANCH ? 0 : PAX(P.gbc[bl], bl);
    const int gdel = go - gop;
    {
        int carry = globalB ? go : 0;
        bool blocked_carry = false;
        for (int base = bl + 1; base < L0; base += 32) {
            int j = base + lane;
            bool act = j < L0;
            const int gbcj = act ? P.gbc[j] : 0;  // gap term << 4 | sigma column class
            if (act) gBs[RG(j)] = gbcj;
            int val;
            if (ANCH) {
                bool blk = act && !a_ins(P, al, j);
                int s = globalB ? (gbcj >> 4) - (MOD ? lam : 0) : 0;
                unsigned bm = __ballot_sync(0xffffffffu, blk);
#pragma unroll
                for (int off = 1; off < 32; off <<= 1) {
                    int t = __shfl_up_sync(0xffffffffu, s, off);
                    if (lane >= off) s += t;
                }
                bool anyblk = blocked_carry || (bm & (0xffffffffu >> (31 - lane)));
                val = anyblk ? NEG : carry + s;
                carry += __shfl_sync(0xffffffffu, s, 31);
                blocked_carry = blocked_carry || bm != 0;
            } else {
                // go + sum_{bl<t<=j} gapB(t)
                val = globalB ? go + PAX(gbcj, j) - PAbl - (j - bl) * gop : 0;
            }
            if (act) {
                PREV(j) = val;
                Mg[j - bl] = val;
            }
        }
        if (lane == 0) {
            PREV(bl) = 0;
            Mg[0] = 0;
        }
        // cells above the band of row al+1 (aligner.cc:361-367)
        if (al + 1 < ar) {
            int L1 = min(br, rowinfo[al + 1].y + 1);
            for (int j = L0 + lane; j < L1; j += 32) {
                PREV(j) = NEG;
                gBs[RG(j)] = P.gbc[j];
            }
        }
    }
    __syncwarp();

    int colval = globalA ? go : 0;
    bool colblocked = false;
    int dwp = 0;
    int dw_row = (DWRITE && ndw > 0) ? dw[0].y : INT_MAX;  // D-write lists are by row ascending
    int best = TOP ? 0 : NEG, bi = 0, bj = 0;  // sequence-local argmax (aligner.cc:865-875)
    const int la = P.la, lb = P.lb, ra = P.ra, rb = P.rb;
    int4 rnxt = rowinfo[min(al + 1, P.n + 1)];
    int2 anxt = rowarc[min(al + 1, P.n + 1)];
    int cnxt = SCLS ? P.rcls[min(al + 1, P.n + 1)] : 0;

    for (int i = al + 1; i < ar; ++i) {
        const int4 rcur = rnxt;
        const int2 acur = anxt;
        const int rcl16 = cnxt * 16;  // SCLS: row class of row i
        rnxt = rowinfo[min(i + 1, P.n + 1)];
        anxt = rowarc[min(i + 1, P.n + 1)];
        if (SCLS) cnxt = P.rcls[min(i + 1, P.n + 1)];
        const int minc = rcur.x;
        const int gAi = rcur.z - (MOD ? lam : 0);
        const int lo = max(bl + 1, minc);
        const int hi = min(br - 1, rcur.y);
        const int *srow = sigma + (size_t)i * m1;
        // sigma of the first NCH chunks of the row, issued before any use
        // (dense table only)
        int sgv[SCLS ? 1 : NCH];
        if (!SCLS) {
#pragma unroll
            for (int k = 0; k < NCH; ++k) {
                const int j = lo + 32 * k + lane;
                sgv[k] = j <= hi ? srow[j] : 0;
            }
        }
        // ---- arc-match terms of row i into Arow[lo .. hi]: two batches of 32
        // entries per step, their loads issued together
        bool rowarcs = false;
        for (int e0 = acur.x; e0 < acur.y; e0 += 64) {
            int2 en[2];
            bool okA[2];
            unsigned ball[2];
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int e = e0 + 32 * u + lane;
                en[u] = e < acur.y ? crow[e] : make_int2(0xffff, 0);
            }
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int ca = en[u].x & 0xffff;  // a.l - 1 (0xffff: no entry)
                okA[u] = ca >= al && ca != 0xffff;  // a.l > al
                ball[u] = __ballot_sync(0xffffffffu, okA[u]);
            }
            if (ball[0] == 0u) break;
            rowarcs = true;
            bool ok[2];
            int dv[2], mv[2];
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int ca = en[u].x & 0xffff, cbl = en[u].x >> 16;  // inner corner (a.l-1, b.l-1)
                ok[u] = okA[u] && cbl >= bl && en[u].y >= lo && en[u].y <= hi;
                if (COUNT) {
                    n_visits += okA[u];
                    n_terms += ok[u];
                }
                const int e = e0 + 32 * u + lane;
                dv[u] = ok[u] ? (WAIT ? ld_volatile(Dp + e) : Dp[e]) : 0;
                mv[u] = ok[u] ? Mg[(ca - al) * pitch + (cbl - bl)] : 0;
            }
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                if (ok[u]) {
                    if (WAIT && dv[u] == NOT_READY) dv[u] = wait_D(Dp, e0 + 32 * u + lane, status, abort_flag);
                    int term = mv[u] + dv[u];
                    if (MOD) term -= lam * ((i - (en[u].x & 0xffff)) + (en[u].y - (en[u].x >> 16)));
                    atomicMax(&Arow[RG(en[u].y)], term);
                }
            }
            if (ball[0] != 0xffffffffu || ball[1] != 0xffffffffu) break;
        }
        __syncwarp();
        int B;  // M(i, lo-1)
        if (minc <= bl) {
            if (!colblocked) {
                if (ANCH && !a_del(P, i, bl)) colblocked = true;
                else if (globalA) colval += gAi;
            }
            B = colblocked ? NEG : colval;
            if (lane == 0) Mg[(i - al) * pitch] = B;
        } else {
            B = NEG;
        }
        if (lane == 0) CUR(lo - 1) = B;
        int *Mrow = Mg + (i - al) * pitch - bl;
        int Fc = NEG, Xc = B;
        // without anchors: Pc = max over k < base of M-open terms X(k) - PA(k),
        // starting with k = lo-1 (column lo-1 > bl is in the ring: it is in
        // the band of an earlier row of the group)
        int Pc = 0;
        if (!ANCH) Pc = B - (lo - 1 == bl ? PAbl : PAX(gBs[RG(lo - 1)], lo - 1));
        int k = 0;
        int rbase = RG(lo);  // ring index of column base, advanced by 32 per chunk
        for (int base = lo; base <= hi; base += 32, ++k) {
            const int j = base + lane;
            const bool act = j <= hi;
            int rj = rbase + lane;  // ring index of column j
            if (rj >= ringn) rj -= ringn;
            const int rjm = rj == 0 ? ringn - 1 : rj - 1;  // of column j-1
            rbase += 32;
            if (rbase >= ringn) rbase -= ringn;
            const int gbc = act ? gBs[rj] : 0;  // gap cost << 4 | sigma column class
            int sgx = 0;
            if (SCLS) {
                if (act) sgx = Stab[rcl16 + (gbc & 15)];
            } else {
#pragma unroll
                for (int kk = 0; kk < NCH; ++kk)
                    if (k == kk) sgx = sgv[kk];
                if (k >= NCH && act) sgx = srow[j];
            }
            if (MOD) sgx -= 2 * lam;
            int X = NEG;
            if (act) {
                const bool mok = !ANCH || a_match(P, i, j);
                const bool dok = !ANCH || a_del(P, i, j);
                const int d = mok ? PREVR(rjm) + sgx : NEG;
                int e = dok ? __viaddmax_s32(E[rj], gAi, PREVR(rj) + gAi + go) : NEG;
                e = norm(e);
                E[rj] = e;
                X = max(d, e);
                if (rowarcs) {
                    if (mok) X = max(X, Arow[rj]);
                    Arow[rj] = NEG;
                }
            }
            if (TOP && local_top && act && i < la && j < lb) X = max(X, 0);
            int F;
            if (ANCH) {
                // horizontal gaps: max-plus scan of F(j) = max(F(j-1)+a_j, b_j)
                int Xp = __shfl_up_sync(0xffffffffu, X, 1);
                if (lane == 0) Xp = Xc;
                int a = 0, b = NEG;
                if (act) {
                    if (a_ins(P, i, j)) {
                        const int gb = (gbc >> 4) - (MOD ? lam : 0);
                        a = gb + gop;
                        b = addc(Xp, gb + go);
                    } else {
                        a = NEG;
                    }
                }
#pragma unroll
                for (int off = 1; off < 32; off <<= 1) {
                    const int a1 = __shfl_up_sync(0xffffffffu, a, off);
                    const int b1 = __shfl_up_sync(0xffffffffu, b, off);
                    if (lane >= off) {
                        b = max(addc(b1, a), b);
                        a = addc(a1, a);
                    }
                }
                F = max(addc(Fc, a), b);
                Fc = __shfl_sync(0xffffffffu, F, 31);
                Xc = __shfl_sync(0xffffffffu, X, 31);
            } else {
                // F(j) = max_{k<j} X(k) + go + sum_{k<t<=j} gapB(t)
                //      = PA(j) + (go - gop) + max_{k<j} (X(k) - PA(k)),
                // a prefix maximum over the lanes (inactive lanes: X = NEG)
                const int pa = PAX(gbc, j);
                const int v = X - pa;
                int w = __shfl_up_sync(0xffffffffu, v, 1);
                if (lane == 0) w = Pc;
#pragma unroll
                for (int off = 1; off < 32; off <<= 1) w = max(w, __shfl_up_sync(0xffffffffu, w, off));
                F = w + pa + gdel;
                Pc = __shfl_sync(0xffffffffu, max(w, v), 31);
            }
            const int M = norm(max(X, F));
            if (act) {
                CURR(rj) = M;
                Mrow[j] = M;
                if (TOP && local_top && i >= ra && j >= rb && M > best) {
                    best = M;
                    bi = i;
                    bj = j;
                }
            }
        }
        __syncwarp();
        if (DWRITE && i == dw_row) {
            // fill_D_entries for arc matches whose inner corner is in row i;
            // without lonely pairs (P.dwn set) fill_D_entries_noLP: the
            // better of the corner and the inner arc match's own D
            while (dwp < ndw) {
                const int q = dwp + lane;
                int4 e = make_int4(0, -1, 0, 0);
                if (q < ndw) e = dw[q];
                const bool mine = q < ndw && e.y == i;
                if (mine) {
                    int v = CUR(e.z) + e.w;
                    if (INNER && (P.flags & (PF_NOLP | PF_STACK)))
                        v = max(v, inner_term<WAIT>(P, dw + q, status, abort_flag));
                    st_volatile(Dp + e.x, norm(v));
                }
                const int cnt = __popc(__ballot_sync(0xffffffffu, mine));
                dwp += cnt;
                if (cnt < 32) break;
            }
            dw_row = dwp < ndw ? dw[dwp].y : INT_MAX;  // next row with D writes
        }
        if (i + 1 < ar) {
            // columns entering the band with row i+1: M above them is -inf,
            // their E starts at -inf, their gap cost is staged
            const int Ln = min(br, rnxt.y + 1);
            for (int j = max(hi + 1, bl + 1) + lane; j < Ln; j += 32) {
                CUR(j) = NEG;
                E[RG(j)] = NEG;
                gBs[RG(j)] = P.gbc[j];
            }
        }
        __syncwarp();
        const int tp = pv;
        pv = cu;
        cu = tp;
        // no per-row poll of the abort flag: every wait polls it, and the
        // dequeue loop stops on it after the group
    }
#undef PREV
#undef CUR
#undef PREVR
#undef CURR
#undef RG
#undef PAX
    if (TOP) {
        tout->best = best;
        tout->bi = bi;
        tout->bj = bj;
    }
    if (COUNT) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            n_terms += __shfl_xor_sync(0xffffffffu, n_terms, off);
            n_visits += __shfl_xor_sync(0xffffffffu, n_visits, off);
        }
        if (lane == 0) {
            atomicAdd(counters, n_terms);
            atomicAdd(counters + 1, n_visits);
        }
    }
}

// All groups use the same routine, specialised for pairs without anchor
// constraints; `cpl` (columns per lane in an earlier design) is ignored.
// Shared memory per warp (smem_warp_ints): 5 ring rows of `ringn` ints from
// `sbase` (previous and current M row, E, gap cost << 4 | sigma column class,
// arc-term maxima), indexed by column j mod ringn, and the 256-entry sigma
// class table; ringn (a multiple of 32) exceeds the column span of any two
// consecutive band rows. Gap costs stay below 2^27 (host check), so the
// packed value does not overflow.
// FAST: every pair of the launch has a sigma class table, no anchors, no
// lonely-pair or stacking terms (INNER = false: the D writes are the plain
// fill_D_entries, so this hot instantiation carries no inner-term code).
template <bool TOP, bool WAIT, bool DWRITE, bool COUNT = false, bool FAST = false, bool MOD = false>
__device__ __forceinline__ void run_group(const PairDev &P, int cpl, int al, int ar, int bl, int br,
                                          int *__restrict__ Mg, int pitch, int sbase, int ringn,
                                          const int4 *__restrict__ dw, int ndw,
                                          bool globalA, bool globalB, bool local_top, int *status,
                                          volatile int *abort_flag, TopOut *tout,
                                          unsigned long long *counters = nullptr, int lam = 0) {
    if (FAST)
        run_group_c<4, false, true, TOP, WAIT, DWRITE, COUNT, MOD, false>(P, al, ar, bl, br, Mg, pitch, sbase, ringn,
                                                                          dw, ndw, globalA, globalB, local_top, status,
                                                                          abort_flag, tout, counters, lam);
    else if ((P.flags & PF_ANCHORS) && (P.flags & PF_SCLS))
        run_group_c<4, true, true, TOP, WAIT, DWRITE, COUNT, MOD>(P, al, ar, bl, br, Mg, pitch, sbase, ringn, dw, ndw,
                                                             globalA, globalB, local_top, status, abort_flag,
                                                             tout, counters, lam);
    else if (P.flags & PF_ANCHORS)
        run_group_c<4, true, false, TOP, WAIT, DWRITE, COUNT, MOD>(P, al, ar, bl, br, Mg, pitch, sbase, ringn, dw, ndw,
                                                              globalA, globalB, local_top, status, abort_flag,
                                                              tout, counters, lam);
    else if (P.flags & PF_SCLS)
        run_group_c<4, false, true, TOP, WAIT, DWRITE, COUNT, MOD>(P, al, ar, bl, br, Mg, pitch, sbase, ringn, dw, ndw,
                                                              globalA, globalB, local_top, status, abort_flag,
                                                              tout, counters, lam);
    else
        run_group_c<4, false, false, TOP, WAIT, DWRITE, COUNT, MOD>(P, al, ar, bl, br, Mg, pitch, sbase, ringn, dw, ndw,
                                                               globalA, globalB, local_top, status, abort_flag,
                                                               tout, counters, lam);
}

static __device__ __forceinline__ void warp_argmax(int &v, int &k1, int &k2) {
    // max v; ties -> smallest (k1,k2) lexicographically
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        int v2 = __shfl_xor_sync(0xffffffffu, v, off);
        int a2 = __shfl_xor_sync(0xffffffffu, k1, off);
        int b2 = __shfl_xor_sync(0xffffffffu, k2, off);
        bool take = v2 > v || (v2 == v && (a2 < k1 || (a2 == k1 && b2 < k2)));
        if (take) {
            v = v2;
            k1 = a2;
            k2 = b2;
        }
    }
}

// top level + final argmax: align_top_level_free_endgaps (aligner.cc:736-819)
// and align_top_level_locally (aligner.cc:823-880)
template <bool COUNT, bool FAST = false, bool MOD = false>
__device__ __forceinline__ void run_top(const PairDev &P, int cpl, int sbase, int ringn,
                                     int *status, volatile int *abort_flag,
                                     unsigned long long *counters, int lam = 0,
                                     const int4 *rst = nullptr) {
    const int lane = threadIdx.x & 31;
    const int m1 = P.m + 1;
    // AlignerRestriction (aligner_restriction.hh): the top level aligns
    // A[sA..n] with B[sB..m]; the whole sequences unless rst is given (the
    // intervals of k-best alignment, checked on the host)
    const int sA = rst ? rst->x : 1, sB = rst ? rst->y : 1;
    const int n = rst ? rst->z : P.n, m = rst ? rst->w : P.m;
    int *const Mg = P.topM + (size_t)(sA - 1) * m1 + (sB - 1);  // M(sA-1, sB-1)
    const bool local = P.flags & PF_SEQU_LOCAL;
    const int fe = P.free_endgaps;
    TopOut to;
    if (local) {
        run_group<true, !MOD, false, COUNT, FAST, MOD>(P, cpl, sA - 1, n + 1, sB - 1, m + 1, Mg, m1, sbase, ringn,
                                                      nullptr, 0, false, false, true, status, abort_flag,
                                                      &to, counters, lam);
        int v = to.best, i = to.bi, j = to.bj;
        if (v <= 0) {
            v = 0;
            i = sA - 1;
            j = sB - 1;
        }
        warp_argmax(v, i, j);
        if (lane == 0) {
            if (v <= 0) {
                v = 0;
                i = sA - 1;
                j = sB - 1;
            }
            P.res[R_SCORE] = v;
            P.res[R_MAXI] = i;
            P.res[R_MAXJ] = j;
        }
        return;
    }
    run_group<true, !MOD, false, COUNT, FAST, MOD>(P, cpl, sA - 1, n + 1, sB - 1, m + 1, Mg, m1, sbase, ringn,
                                                  nullptr, 0, !(fe & 4), !(fe & 1), false, status, abort_flag,
                                                  &to, counters, lam);
    __syncwarp();
    // The argmax reads M(n,m) and, with free right end gaps, column m of the
    // rows whose band reaches m (aligner.cc:771-799). On an interval of
    // k-best alignment such a cell can lie outside the band, where the
    // reference reads whatever its reused matrix holds; here it counts as
    // -inf. On the whole sequences every cell read is in the band.
    if (!(fe & (2 | 8))) {
        if (lane == 0) {
            const bool inb = (P.min_col[n] <= m && m <= P.max_col[n]) || (n == sA - 1 && m == sB - 1);
            P.res[R_SCORE] = inb ? P.topM[(size_t)n * m1 + m] : NEG;
            P.res[R_MAXI] = n;
            P.res[R_MAXJ] = m;
        }
        return;
    }
    // free right end gaps: first strict maximum over column m (i ascending),
    // then over row n (j ascending); order key = position in that scan
    int v = NEG, k1 = INT32_MAX, k2 = 0;
    if (fe & 8) {
        for (int i = max(P.ra + 1, sA) + lane; i <= n; i += 32) {
            if (P.max_col[i] >= m && P.min_col[i] <= m) {
                int x = P.topM[(size_t)i * m1 + m];
                if (x > v) {
                    v = x;
                    k1 = i;
                    k2 = 0;
                }
            }
        }
    }
    if (fe & 2) {
        int lo = max(max(P.rb + 1, sB), P.min_col[n]), hi = min(m, P.max_col[n]);
        for (int j = lo + lane; j <= hi; j += 32) {
            int x = P.topM[(size_t)n * m1 + j];
            if (x > v) {
                v = x;
                k1 = n + 1 + j;  // after every column-m entry
                k2 = 0;
            }
        }
    }
    warp_argmax(v, k1, k2);
    if (lane == 0) {
        int mi = sA - 1, mj = sB - 1;
        if (v > NEG) {
            if (k1 <= n) {
                mi = k1;
                mj = m;
            } else {
                mi = n;
                mj = k1 - n - 1;
            }
        } else {
            v = NEG;
        }
        P.res[R_SCORE] = v;
        P.res[R_MAXI] = mi;
        P.res[R_MAXJ] = mj;
    }
}

// ---------------------------------------------------------------- traceback

struct Walker {
    const PairDev &P;
    int ntok, qtail;
    bool ok;
    __device__ Walker(const PairDev &p) : P(p), ntok(0), qtail(0), ok(true) {}
    __device__ void emit(int a, int b) {
        if (ntok < P.token_cap) P.tokens[ntok] = make_int2(a, b);
        else ok = false;
        ++ntok;
    }
    __device__ bool valid(int i, int j) const {
        return i >= 0 && i <= P.n && P.min_col[i] <= j && j <= P.max_col[i];
    }
};

// Traceback queue entries: (am, aux, a.l | b.l << 16 | mode, a.r | b.r << 16).
// Mode TQ_CHAIN (no lonely pairs): trace_arcmatch_noLP of am, aux = its D
// index. Otherwise the interior of am is recomputed and walked; aux = its D
// index, or, for the inner arc match of a no-lonely-pairs stack, the value
// its interior's corner must have (D(outer) - score(outer) - score(am)).
constexpr int TQ_CHAIN = INT32_MIN;
__device__ __forceinline__ int4 trace_entry(const PairDev &P, int am, int dpos, int al, int ar, int bl, int br) {
    return make_int4(am, dpos, al | (bl << 16) | ((P.flags & PF_NOLP) ? TQ_CHAIN : 0), ar | (br << 16));
}
// (a.l, a.r, b.l, b.r) of a queue entry
__device__ __forceinline__ int4 trace_ends(int lefts, int rights) {
    return make_int4(lefts & 0xffff, rights & 0xffff, (lefts >> 16) & 0x7fff, rights >> 16);
}

// Arc match k's segment when k is traced through its inner arc match:
// the inner arc match's two edges around its arc-match token
__device__ __forceinline__ void emit_inner(Walker &w, int in, int4 ends) {
    w.emit(ends.y - 1, ends.w - 1);
    w.emit(-2, in);
    w.emit(ends.x + 1, ends.z + 1);
}

// trace_arcmatch_noLP (aligner.cc:1030-1079) for arc match k (D index kpos):
// the inner arc match's two edges and its arc-match token form k's segment;
// the inner arc match is queued to continue the stack (TQ_CHAIN) when
// D(k) == D(inner) + score'(k), else to have its interior recomputed and
// walked (aligner.cc:1057-1075); score' is the stacked score with stacking.
static __device__ __noinline__ void trace_chain(Walker &w, int k, int kpos, int4 ends, int &nseg,
                                                int *status) {
    const PairDev &P = w.P;
    const int2 in = P.inner[k];
    const int start = w.ntok;
    if (in.x < 0) {
        atomicOr(status, ST_INTERNAL);
    } else {
        const int ial = ends.x + 1, iar = ends.y - 1, ibl = ends.z + 1, ibr = ends.w - 1;
        emit_inner(w, in.x, ends);
        const int dk = P.D[kpos], sk = (P.flags & PF_STACK) ? P.am_sscore[k] : P.am_score[k];
        const int din = in.y >= 0 ? P.D[in.y] : NEG;
        int4 e;
        if (in.y >= 0 && dk == din + sk)
            e = make_int4(in.x, in.y, ial | (ibl << 16) | TQ_CHAIN, iar | (ibr << 16));
        else
            e = make_int4(in.x, dk - sk - P.am_score[in.x], ial | (ibl << 16), iar | (ibr << 16));
        if (w.qtail < P.tq_cap) P.tq[w.qtail] = e;
        else w.ok = false;
        ++w.qtail;
    }
    if (nseg < P.tq_cap + 1) P.segs[nseg] = make_int4(k, start, w.ntok, 0);
    ++nseg;
}

// trace_arcmatch with stacking (aligner.cc:986-1006): if arc match k (D index
// kpos) is explained by its inner arc match, D(k) == D(inner) + stacked
// score(k), k's segment is the inner arc match's edges and token, the inner
// arc match is queued in the same mode, and this returns true; else k's
// interior is traced as without stacking.
static __device__ __noinline__ bool trace_stack(Walker &w, int k, int kpos, int4 ends, int &nseg) {
    const PairDev &P = w.P;
    const int2 in = P.inner[k];
    if (in.x < 0 || in.y < 0 || P.D[kpos] != P.D[in.y] + P.am_sscore[k]) return false;
    const int start = w.ntok;
    emit_inner(w, in.x, ends);
    if (w.qtail < P.tq_cap)
        P.tq[w.qtail] = make_int4(in.x, in.y, (ends.x + 1) | ((ends.z + 1) << 16), (ends.y - 1) | ((ends.w - 1) << 16));
    else
        w.ok = false;
    ++w.qtail;
    if (nseg < P.tq_cap + 1) P.segs[nseg] = make_int4(k, start, w.ntok, 0);
    ++nseg;
    return true;
}

// Walk back from (i,j) inside the rectangle with origin (al,bl) whose M is
// Mg (pitch), emitting tokens in reverse append order. Arc-match tokens are
// (-2, am); each traced arc match is queued for its own walk. On the top level
// (tl) lam is the penalty of the modified scoring view of normalized and
// penalized alignment (0 otherwise).
static __device__ __noinline__ void walk(Walker &w, const int *Mg, int pitch, int al, int bl, int i, int j, bool tl,
                     int *status, int lam = 0) {
    const PairDev &P = w.P;
    const int tlam = tl ? lam : 0;
    const bool local = P.flags & PF_SEQU_LOCAL;
    const int fe = P.free_endgaps;
    const int go = P.go;
#define MM(x, y) Mg[(size_t)((x) - al) * pitch + ((y) - bl)]
    for (int guard = 0; guard < 4 * (P.n + P.m + 4); ++guard) {
        const int Mij = MM(i, j);
        if (tl && local && Mij == 0) {
            P.res[R_MINI] = i;
            P.res[R_MINJ] = j;
            return;
        }
        if (i <= al) {
            if (!(tl && (local || (fe & 1))))
                for (int k = j; k > bl; --k) w.emit(-1, k);
            return;
        }
        if (j <= bl) {
            if (!(tl && (local || (fe & 4))))
                for (int k = i; k > al; --k) w.emit(k, -1);
            return;
        }
        if (a_match(P, i, j) && w.valid(i - 1, j - 1) &&
            Mij == MM(i - 1, j - 1) + sigma_at(P, i, j) - 2 * tlam) {
            w.emit(i, j);
            --i;
            --j;
            continue;
        }
        bool found = false;
        if (go == 0) {
            if (a_del(P, i, j) && w.valid(i - 1, j) && Mij == MM(i - 1, j) + P.gapA[i] - tlam) {
                w.emit(i, -1);
                --i;
                continue;
            }
            if (a_ins(P, i, j) && w.valid(i, j - 1) && Mij == MM(i, j - 1) + P.gapB[j] - tlam) {
                w.emit(-1, j);
                --j;
                continue;
            }
        } else {
            int gap = go;
            for (int k = 1; i >= al + k && a_del(P, i - k + 1, j); ++k) {
                if (!w.valid(i - k, j)) break;
                gap += P.gapA[i - k + 1] - tlam;
                if (Mij == MM(i - k, j) + gap) {
                    for (int l = 1; l <= k; ++l) w.emit(i - l + 1, -1);
                    i -= k;
                    found = true;
                    break;
                }
            }
            if (found) continue;
            gap = go;
            for (int k = 1; j >= bl + k && a_ins(P, i, j - k + 1); ++k) {
                if (!w.valid(i, j - k)) break;
                gap += P.gapB[j - k + 1] - tlam;
                if (Mij == MM(i, j - k) + gap) {
                    for (int l = 1; l <= k; ++l) w.emit(-1, j - l + 1);
                    j -= k;
                    found = true;
                    break;
                }
            }
            if (found) continue;
        }
        if (!(a_match(P, i, j) && w.valid(i - 1, j - 1))) return;
        const int cell = P.bandoff[i] + j - P.min_col[i];
        for (int q = P.cre_start[cell]; q < P.cre_start[cell + 1]; ++q) {
            const int4 ent = P.cre[q];
            const int alq = ent.y + 1, blq = ent.z + 1;
            if (alq <= al || blq <= bl) continue;
            if (Mij == MM(alq - 1, blq - 1) + P.D[ent.x] - tlam * ((i - alq + 1) + (j - blq + 1))) {
                w.emit(i, j);
                w.emit(-2, ent.w);
                w.emit(alq, blq);
                if (w.qtail < P.tq_cap) P.tq[w.qtail] = trace_entry(P, ent.w, ent.x, alq, i, blq, j);
                else w.ok = false;
                ++w.qtail;
                i = alq - 1;
                j = blq - 1;
                found = true;
                break;
            }
        }
        if (!found) return;
    }
    atomicOr(status, ST_INTERNAL);
#undef MM
}


}  // namespace lcg
