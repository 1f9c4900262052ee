// Structure-local Sankoff (--struct-local): the eight exclusion states of the
// reference (aligner_impl.hh:113-122) inside each left-end group.
//
//   sankoff_sl_fill_kernel   like sankoff_fill_kernel, but each group sweeps
//                            the eight state matrices of align_in_arcmatch
//                            with allow_exclusion (aligner.cc:373-565) and
//                            fills D with the best non-open state
//                            (fill_D_entries, aligner.cc:574-597); the top
//                            level is the plain one (state NO_NO).
//   sankoff_sl_trace_kernel  traceback through the state switch of
//                            trace_in_arcmatch (aligner.cc:1233-1343).
//
// The reference computes the eight matrices one after another over the whole
// rectangle. Every dependency between them is either on the same cell of an
// earlier state, on the previous row of the same state, or on the previous
// column of the same state, so this build evaluates all eight states row by
// row in the order NO_NO, OP_NO, NO_OP, NO_X, OP_X, X_NO, X_OP, X_X, which
// respects every dependency and gives the same values. Row-chained states use
// the same warp max-plus scan as the F chain:
//   NO_OP(i,j) = max(NO_OP(i,j-1) [if ins allowed], NO_NO(i,j))
//   X_OP (i,j) = max(X_OP (i,j-1) [if ins allowed], X_NO (i,j)).
#include <cuda_runtime.h>
#include <stdint.h>

#include "sankoff_group.cuh"

namespace lcg {

enum { S_NO_NO = 0, S_X_NO = 1, S_NO_X = 2, S_X_X = 3, S_OP_NO = 4, S_NO_OP = 5, S_OP_X = 6, S_X_OP = 7 };

constexpr int SL_FILL_WARPS = 4;
// shared-memory rows per warp: prev/cur of states 0,1,2,3,4,6 and E of 0..3
constexpr int SL_ROWS = 16;
// shared ints per warp of the fill kernel: SL_ROWS rows of sw for the group
// states, and room for the plain row sweep of the top level (smem_warp_ints)
__host__ __device__ inline int sl_warp_ints(int sw, int rb) {
    return SL_ROWS * sw > smem_warp_ints(rb) ? SL_ROWS * sw : smem_warp_ints(rb);
}

// slot of a state's prev row in shared memory (states 5 and 7 keep no row)
__device__ __forceinline__ int sl_slot(int s) { return s < 4 ? s : (s == 4 ? 4 : 5); }

// warp inclusive max-plus scan of maps x -> max(x + a, b), applied to x0
__device__ __forceinline__ int maxplus_scan(int a, int b, int x0, int lane) {
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        int a1 = __shfl_up_sync(0xffffffffu, a, off);
        int b1 = __shfl_up_sync(0xffffffffu, b, off);
        if (lane >= off) {
            b = max(addc(b1, a), b);
            a = addc(a1, a);
        }
    }
    return max(addc(x0, a), b);
}

// One left-end group with exclusions. Mg holds NS state matrices, state s at
// Mg + s*mstride (NS = 4 in the fill: the states arc terms read; 8 in the
// traceback recomputation).
template <bool WAIT, bool DWRITE, int NS>
__device__ void run_group_sl(const PairDev &P, int al, int ar, int bl, int br, int *__restrict__ Mg,
                             long long mstride, int pitch, int *sm, int sw,
                             const int4 *__restrict__ dw, int ndw, int *status,
                             volatile int *abort_flag) {
    const int lane = threadIdx.x & 31;
    const int go = P.go, X = P.excl;
    const int W = br - bl;
    int *prev[6], *cur[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        prev[k] = sm + k * sw;
        cur[k] = sm + (6 + k) * sw;
    }
    int *E[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) E[k] = sm + (12 + k) * sw;
    for (int c = lane; c < W; c += 32) {
#pragma unroll
        for (int k = 0; k < 4; ++k) E[k][c] = NEG;
    }
    // init_state per state (aligner.cc:264-368): row al patterns by (globalB,exclB)
    //  (1,0): states 0,1,4 -> go + prefix gapB ; (1,1): 2,3,6 -> exclusion ;
    //  (0,0): states 5,7   -> 0 ; all become -inf once an insertion is forbidden
    const int L0 = min(br, P.max_col[al] + 1);
    {
        int carry = go;
        bool blocked_carry = false;
        for (int base = bl + 1; base < L0; base += 32) {
            int j = base + lane;
            bool act = j < L0;
            bool blk = act && !a_ins(P, al, j);
            int s = act ? P.gapB[j] : 0;
            unsigned bm = __ballot_sync(0xffffffffu, blk);
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                int t = __shfl_up_sync(0xffffffffu, s, off);
                if (lane >= off) s += t;
            }
            bool anyblk = blocked_carry || (bm & (0xffffffffu >> (31 - lane)));
            int vg = anyblk ? NEG : carry + s, vx = anyblk ? NEG : X, v0 = anyblk ? NEG : 0;
            if (act) {
                const int c = j - bl;
                prev[0][c] = vg; prev[1][c] = vg; prev[4][c] = vg;
                prev[2][c] = vx; prev[3][c] = vx; prev[5][c] = vx;
                int vals[8] = {vg, vg, vx, vx, vg, v0, vx, v0};
#pragma unroll
                for (int s2 = 0; s2 < NS; ++s2) Mg[s2 * mstride + c] = vals[s2];
            }
            carry += __shfl_sync(0xffffffffu, s, 31);
            blocked_carry = blocked_carry || bm != 0;
        }
        if (lane == 0) {
#pragma unroll
            for (int k = 0; k < 6; ++k) prev[k][0] = 0;
#pragma unroll
            for (int s2 = 0; s2 < NS; ++s2) Mg[s2 * mstride] = 0;
        }
        if (al + 1 < ar) {
            int L1 = min(br, P.max_col[al + 1] + 1);
            for (int j = L0 + lane; j < L1; j += 32) {
#pragma unroll
                for (int k = 0; k < 6; ++k) prev[k][j - bl] = NEG;
            }
        }
    }
    __syncwarp();

    // column bl patterns by (globalA,exclA): (1,0): 0,2,5 ; (1,1): 1,3,7 ; (0,0): 4,6
    int colg = go;
    bool colblocked = false;
    int dwp = 0;
    for (int i = al + 1; i < ar; ++i) {
        const int minc = P.min_col[i];
        const int maxc = P.max_col[i];
        const int lo = max(bl + 1, minc);
        const int hi = min(br - 1, maxc);
        const int gAi = P.gapA[i];
        int Bs[8];
        if (minc <= bl) {
            if (!colblocked) {
                if (!a_del(P, i, bl)) colblocked = true;
                else colg += gAi;
            }
            const int bg = colblocked ? NEG : colg, bx = colblocked ? NEG : X, b0 = colblocked ? NEG : 0;
            Bs[0] = bg; Bs[2] = bg; Bs[5] = bg;
            Bs[1] = bx; Bs[3] = bx; Bs[7] = bx;
            Bs[4] = b0; Bs[6] = b0;
            if (lane == 0) {
#pragma unroll
                for (int s2 = 0; s2 < NS; ++s2) Mg[s2 * mstride + (long long)(i - al) * pitch] = Bs[s2];
            }
        } else {
#pragma unroll
            for (int s2 = 0; s2 < 8; ++s2) Bs[s2] = NEG;
        }
        if (lane == 0 && lo - 1 - bl < W) {
            cur[0][lo - 1 - bl] = Bs[0];
            cur[1][lo - 1 - bl] = Bs[1];
            cur[2][lo - 1 - bl] = Bs[2];
            cur[3][lo - 1 - bl] = Bs[3];
            cur[4][lo - 1 - bl] = Bs[4];
            cur[5][lo - 1 - bl] = Bs[6];
        }
        const long long roff = (long long)(i - al) * pitch - bl;
        const int cell0 = P.bandoff[i] - minc;
        // carries across chunks: F of states 0..3, X' of states 0..3, NO_OP, X_OP
        int Fc[4] = {NEG, NEG, NEG, NEG};
        int Xc[4] = {Bs[0], Bs[1], Bs[2], Bs[3]};
        int C5 = Bs[5], C7 = Bs[7];
        for (int base = lo; base <= hi; base += 32) {
            const int j = base + lane;
            const bool act = j <= hi;
            const int c = j - bl;
            bool mok = false, dok = false, iok = false;
            int sg = 0, gb = 0;
            int arcv[4] = {NEG, NEG, NEG, NEG};
            if (act) {
                mok = a_match(P, i, j);
                dok = a_del(P, i, j);
                iok = a_ins(P, i, j);
                sg = sigma_at(P, i, j);
                gb = P.gapB[j];
                if (mok) {
                    const int cell = cell0 + j;
                    const int q1 = P.cre_start[cell + 1];
                    for (int q = P.cre_start[cell]; q < q1; ++q) {
                        const int4 ent = P.cre[q];
                        const int alq = ent.y + 1, blq = ent.z + 1;
                        if (alq <= al) break;
                        if (blq <= bl) continue;
                        const int dv = WAIT ? wait_D(P.D, ent.x, status, abort_flag) : P.D[ent.x];
                        const long long o = (long long)(alq - 1 - al) * pitch + (blq - 1 - bl);
#pragma unroll
                        for (int s2 = 0; s2 < 4; ++s2) arcv[s2] = max(arcv[s2], Mg[s2 * mstride + o] + dv);
                    }
                }
            }
            // noex part of a state: diagonal, vertical gap, arc terms
            auto noex_x = [&](int s2) {
                int v = NEG;
                if (act) {
                    int d = mok ? prev[s2][c - 1] + sg : NEG;
                    int e = dok ? max(E[s2][c] + gAi, prev[s2][c] + gAi + go) : NEG;
                    e = norm(e);
                    E[s2][c] = e;
                    v = max(max(d, e), arcv[s2]);
                }
                return v;
            };
            auto fscan = [&](int s2, int Xs) {
                int Xp = __shfl_up_sync(0xffffffffu, Xs, 1);
                if (lane == 0) Xp = Xc[s2];
                int a = 0, b = NEG;
                if (act) {
                    if (iok) {
                        a = gb + max(go, 0);
                        b = addc(Xp, gb + go);
                    } else {
                        a = NEG;
                    }
                }
                const int F = maxplus_scan(a, b, Fc[s2], lane);
                Fc[s2] = __shfl_sync(0xffffffffu, F, 31);
                Xc[s2] = __shfl_sync(0xffffffffu, Xs, 31);
                return norm(max(Xs, F));
            };
            auto rowscan = [&](int &carry, int bval) {
                int a = act ? (iok ? 0 : NEG) : 0;
                int b = act ? bval : NEG;
                const int v = norm(maxplus_scan(a, b, carry, lane));
                carry = __shfl_sync(0xffffffffu, v, 31);
                return v;
            };
            // NO_NO
            const int M0 = fscan(0, noex_x(0));
            // OP_NO
            const int M4 = act ? norm(max(dok ? prev[4][c] : NEG, M0)) : NEG;
            // NO_OP
            const int M5 = rowscan(C5, M0);
            // NO_X
            int x2 = noex_x(2);
            if (act) x2 = max(x2, M5 + X);
            const int M2 = fscan(2, x2);
            // OP_X
            const int M6 = act ? norm(max(dok ? prev[5][c] : NEG, M2)) : NEG;
            // X_NO
            int x1 = noex_x(1);
            if (act) x1 = max(x1, M4 + X);
            const int M1 = fscan(1, x1);
            // X_OP
            const int M7 = rowscan(C7, M1);
            // X_X
            int x3 = noex_x(3);
            if (act) x3 = max(x3, max(M6 + X, M7 + X));
            const int M3 = fscan(3, x3);
            if (act) {
                cur[0][c] = M0;
                cur[1][c] = M1;
                cur[2][c] = M2;
                cur[3][c] = M3;
                cur[4][c] = M4;
                cur[5][c] = M6;
                const int vals[8] = {M0, M1, M2, M3, M4, M5, M6, M7};
#pragma unroll
                for (int s2 = 0; s2 < NS; ++s2) Mg[s2 * mstride + roff + j] = vals[s2];
            }
        }
        __syncwarp();
        if (DWRITE) {
            // fill_D_entries (struct-local: maximum over the non-open
            // states); without lonely pairs (P.dwn set) fill_D_entries_noLP
            while (dwp < ndw) {
                const int q = dwp + lane;
                int4 e = make_int4(0, -1, 0, 0);
                if (q < ndw) e = dw[q];
                const bool mine = q < ndw && e.y == i;
                if (mine) {
                    const int c2 = e.z - bl;
                    const int mv = max(max(cur[0][c2], cur[1][c2]), max(cur[2][c2], cur[3][c2]));
                    int v = mv + e.w;
                    if (P.flags & (PF_NOLP | PF_STACK)) v = max(v, inner_term<WAIT>(P, dw + q, status, abort_flag));
                    st_volatile(P.D + e.x, norm(v));
                }
                const int cnt = __popc(__ballot_sync(0xffffffffu, mine));
                dwp += cnt;
                if (cnt < 32) break;
            }
        }
        if (i + 1 < ar) {
            const int Ln = min(br, P.max_col[i + 1] + 1);
            for (int j = max(hi + 1, bl + 1) + lane; j < Ln; j += 32) {
#pragma unroll
                for (int k = 0; k < 6; ++k) cur[k][j - bl] = NEG;
            }
        }
        __syncwarp();
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            int *t = prev[k];
            prev[k] = cur[k];
            cur[k] = t;
        }
        if (WAIT && *abort_flag) return;
    }
}

// shared ints per warp of the fast fill (run_group_slf) for ring size rb:
// 15 rows of rb and the 16 x 16 sigma class table
__host__ __device__ inline int slf_warp_ints(int rb) { return 15 * rb + 256; }

// warp inclusive prefix maximum of v, started from the carry c (in: the
// previous chunk's, out: this chunk's last lane's), normalised
__device__ __forceinline__ int prefix_max_carry(int v, int &c, int lane) {
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) v = max(v, __shfl_up_sync(0xffffffffu, v, off));
    v = norm(max(v, c));
    c = __shfl_sync(0xffffffffu, v, 31);
    return v;
}

// F of one state by the prefix-sum form: F(j) = PA(j) + (go - max(go,0)) +
// max_{k<j} (X(k) - PA(k)), Pc the running maximum of X(k) - PA(k) over the
// earlier chunks (in) and through this one (out); returns norm(max(X, F)).
__device__ __forceinline__ int fscan_prefix(int x, int pa, int gdel, int &Pc, int lane) {
    const int v = x - pa;
    int w = __shfl_up_sync(0xffffffffu, v, 1);
    if (lane == 0) w = Pc;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) w = max(w, __shfl_up_sync(0xffffffffu, w, off));
    Pc = __shfl_sync(0xffffffffu, max(w, v), 31);
    return norm(max(x, w + pa + gdel));
}

// One left-end group with exclusions, fast path: pairs without anchor
// constraints and with a sigma class table (PF_SCLS). Writes NS state
// matrices to Mg (state s at Mg + s*mstride; NS = 4 in the fill: the states
// arc terms read; 8 in the traceback recomputation) and, with DWRITE, the
// group's D entries.
// The states, their order and values are those of run_group_sl; what
// differs is how they are computed:
//  * shared-memory rows are indexed by ring position (column j at j mod
//    ringn, as in the plain fill) and kept in place: a lane reads its
//    column's row i-1 value before writing row i's, and the diagonal comes
//    from the lane to its left by a shuffle (the chunk's last lane carries it
//    to the next chunk, the old value at lo-1 starts the row);
//  * the arc-match terms of row i come from the row's candidate list
//    (PairDev::crow, a.l descending), 32 entries per step for the whole warp,
//    each valid term M_s(a.l-1, b.l-1) + D(a,b) reduced into its column b.r
//    of state s with a shared-memory atomicMax;
//  * with every insertion allowed, the horizontal chains are prefix maxima:
//    F of NO_NO / X_NO / NO_X / X_X by the prefix-sum form of the plain fill
//    (PairDev::gbc holds PA(j)), NO_OP / X_OP by a plain prefix maximum.
// Shared rows (ring length ringn): 0-3 M of NO_NO, X_NO, NO_X, X_X; 4 M of
// OP_NO; 5 M of OP_X; 6-9 E of 0-3; 10 gap prefix << 4 | column class;
// 11-14 arc-term maxima of 0-3; then the class table.
template <bool WAIT, bool DWRITE, int NS>
__device__ void run_group_slf(const PairDev &P, int al, int ar, int bl, int br, int *__restrict__ Mg,
                              long long mstride, int pitch, int sbase, int ringn,
                              const int4 *__restrict__ dw, int ndw, int *status, volatile int *abort_flag) {
    const int lane = threadIdx.x & 31;
    const int go = P.go, X = P.excl;
    const int gop = max(go, 0), gdel = go - gop;
    const unsigned rmagic = 0xFFFFFFFFu / (unsigned)ringn + 1u;  // j / ringn = umulhi(j, rmagic), j < 2^20
    int *const R = lcg_smem + sbase;
#define ROW(k) (R + (k) * ringn)
#define RG(j) ((j) - ringn * (int)__umulhi((unsigned)(j), rmagic))
    int *const gBs = ROW(10);
    int *const Stab = R + 15 * ringn;
    const int4 *__restrict__ rowinfo = P.rowinfo;
    const int2 *__restrict__ rowarc = P.rowarc;
    const int2 *__restrict__ crow = P.crow;
    int *const Dp = P.D;
    // E rows and the arc-term maxima start at -inf; the cell sweep puts -inf
    // back into every maxima column it reads
    for (int c = lane; c < ringn; c += 32) {
#pragma unroll
        for (int s = 0; s < 4; ++s) {
            ROW(6 + s)[c] = NEG;
            ROW(11 + s)[c] = NEG;
        }
    }
    for (int k = lane; k < 256; k += 32) Stab[k] = P.scls[k];

    // ---- row al (init_state, aligner.cc:264-368): NO_NO, X_NO, OP_NO get
    // go + the gap prefix, NO_X, X_X, OP_X the exclusion X; (al, bl) is 0
    const int L0 = min(br, rowinfo[al].y + 1);
    const int PAbl = P.gbc[bl] >> 4;
    for (int j = bl + 1 + lane; j < L0; j += 32) {
        const int gbcj = P.gbc[j];
        const int rj = RG(j);
        gBs[rj] = gbcj;
        const int vg = go + (gbcj >> 4) - PAbl - (j - bl) * gop;
        ROW(0)[rj] = vg;
        ROW(1)[rj] = vg;
        ROW(4)[rj] = vg;
        ROW(2)[rj] = X;
        ROW(3)[rj] = X;
        ROW(5)[rj] = X;
        const int c = j - bl;
        Mg[c] = vg;
        Mg[mstride + c] = vg;
        Mg[2 * mstride + c] = X;
        Mg[3 * mstride + c] = X;
        if (NS == 8) {
            Mg[4 * mstride + c] = vg;
            Mg[5 * mstride + c] = 0;
            Mg[6 * mstride + c] = X;
            Mg[7 * mstride + c] = 0;
        }
    }
    if (lane == 0) {
        const int r0 = RG(bl);
#pragma unroll
        for (int k = 0; k < 6; ++k) ROW(k)[r0] = 0;
#pragma unroll
        for (int s = 0; s < NS; ++s) Mg[s * mstride] = 0;
    }
    // cells above the band of row al+1
    if (al + 1 < ar) {
        const int L1 = min(br, rowinfo[al + 1].y + 1);
        for (int j = L0 + lane; j < L1; j += 32) {
            const int rj = RG(j);
#pragma unroll
            for (int k = 0; k < 6; ++k) ROW(k)[rj] = NEG;
            gBs[rj] = P.gbc[j];
        }
    }
    __syncwarp();

    int colg = go;  // M(i, bl) of the gap states
    int dwp = 0;
    int dw_row = (DWRITE && ndw > 0) ? dw[0].y : INT_MAX;  // D-write lists are by row ascending
    int4 rnxt = rowinfo[min(al + 1, P.n + 1)];
    int2 anxt = rowarc[min(al + 1, P.n + 1)];
    int cnxt = P.rcls[min(al + 1, P.n + 1)];
    for (int i = al + 1; i < ar; ++i) {
        const int4 rcur = rnxt;
        const int2 acur = anxt;
        const int rcl16 = cnxt * 16;
        rnxt = rowinfo[min(i + 1, P.n + 1)];
        anxt = rowarc[min(i + 1, P.n + 1)];
        cnxt = P.rcls[min(i + 1, P.n + 1)];
        const int minc = rcur.x;
        const int gAi = rcur.z;
        const int lo = max(bl + 1, minc);
        const int hi = min(br - 1, rcur.y);

        // ---- arc-match terms of row i into rows 11-14 at columns lo..hi
        bool rowarcs = false;
        for (int e0 = acur.x; e0 < acur.y; e0 += 32) {
            const int e = e0 + lane;
            const int2 en = e < acur.y ? crow[e] : make_int2(0xffff, 0);
            const int ca = en.x & 0xffff, cbl = en.x >> 16;  // inner corner (a.l-1, b.l-1)
            const bool okA = ca >= al && ca != 0xffff;       // a.l > al
            const unsigned ball = __ballot_sync(0xffffffffu, okA);
            if (ball == 0u) break;
            rowarcs = true;
            if (okA && cbl >= bl && en.y >= lo && en.y <= hi) {
                int dv = WAIT ? ld_volatile(Dp + e) : Dp[e];
                const long long o = (long long)(ca - al) * pitch + (cbl - bl);
                int mv[4];
#pragma unroll
                for (int s = 0; s < 4; ++s) mv[s] = Mg[s * mstride + o];
                if (WAIT && dv == NOT_READY) dv = wait_D(Dp, e, status, abort_flag);
                const int rr = RG(en.y);
#pragma unroll
                for (int s = 0; s < 4; ++s) atomicMax(&ROW(11 + s)[rr], mv[s] + dv);
            }
            if (ball != 0xffffffffu) break;
        }
        __syncwarp();

        // ---- column bl (aligner.cc:264-368 by state) and the row's start
        int B0 = NEG, B1 = NEG, B4 = NEG;  // NO_NO / NO_X / NO_OP; X_NO / X_X / X_OP; OP_NO / OP_X
        if (minc <= bl) {
            colg += gAi;
            B0 = colg;
            B1 = X;
            B4 = 0;
            if (lane == 0) {
                const long long r = (long long)(i - al) * pitch;
                Mg[r] = B0;
                Mg[mstride + r] = B1;
                Mg[2 * mstride + r] = B0;
                Mg[3 * mstride + r] = B1;
                if (NS == 8) {
                    Mg[4 * mstride + r] = B4;
                    Mg[5 * mstride + r] = B0;
                    Mg[6 * mstride + r] = B4;
                    Mg[7 * mstride + r] = B1;
                }
            }
        }
        // lane 0: the diagonal carries (row i-1 at column lo-1), then column
        // lo-1 of row i
        int dc0 = NEG, dc1 = NEG, dc2 = NEG, dc3 = NEG;
        if (lane == 0 && lo - 1 < br) {
            const int r = RG(lo - 1);
            dc0 = ROW(0)[r];
            dc1 = ROW(1)[r];
            dc2 = ROW(2)[r];
            dc3 = ROW(3)[r];
            ROW(0)[r] = B0;
            ROW(1)[r] = B1;
            ROW(2)[r] = B0;
            ROW(3)[r] = B1;
            ROW(4)[r] = B4;
            ROW(5)[r] = B4;
        }
        const int palo = lo - 1 == bl ? PAbl : (gBs[RG(lo - 1)] >> 4);
        int Pc0 = B0 - palo, Pc1 = B1 - palo, Pc2 = B0 - palo, Pc3 = B1 - palo;
        int C5 = B0, C7 = B1;  // NO_OP, X_OP carries
        const long long roff = (long long)(i - al) * pitch - bl;
        int rbase = RG(lo);
        for (int base = lo; base <= hi; base += 32) {
            const int j = base + lane;
            const bool act = j <= hi;
            int rj = rbase + lane;  // ring index of column j
            if (rj >= ringn) rj -= ringn;
            rbase += 32;
            if (rbase >= ringn) rbase -= ringn;
            int gbc = 0, sg = 0;
            int p0 = NEG, p1 = NEG, p2 = NEG, p3 = NEG, p4 = NEG, p6 = NEG;
            int x0 = NEG, x1 = NEG, x2 = NEG, x3 = NEG;
            int e0v = NEG, e1v = NEG, e2v = NEG, e3v = NEG;
            if (act) {
                gbc = gBs[rj];
                sg = Stab[rcl16 + (gbc & 15)];
                p0 = ROW(0)[rj];
                p1 = ROW(1)[rj];
                p2 = ROW(2)[rj];
                p3 = ROW(3)[rj];
                p4 = ROW(4)[rj];
                p6 = ROW(5)[rj];
                e0v = ROW(6)[rj];
                e1v = ROW(7)[rj];
                e2v = ROW(8)[rj];
                e3v = ROW(9)[rj];
            }
            // diagonal M(i-1, j-1) of states 0-3
            int d0 = __shfl_up_sync(0xffffffffu, p0, 1);
            int d1 = __shfl_up_sync(0xffffffffu, p1, 1);
            int d2 = __shfl_up_sync(0xffffffffu, p2, 1);
            int d3 = __shfl_up_sync(0xffffffffu, p3, 1);
            if (lane == 0) {
                d0 = dc0;
                d1 = dc1;
                d2 = dc2;
                d3 = dc3;
            }
            dc0 = __shfl_sync(0xffffffffu, p0, 31);
            dc1 = __shfl_sync(0xffffffffu, p1, 31);
            dc2 = __shfl_sync(0xffffffffu, p2, 31);
            dc3 = __shfl_sync(0xffffffffu, p3, 31);
            if (act) {
                // vertical gaps and the no-exclusion part of states 0-3
                e0v = norm(__viaddmax_s32(e0v, gAi, p0 + gAi + go));
                e1v = norm(__viaddmax_s32(e1v, gAi, p1 + gAi + go));
                e2v = norm(__viaddmax_s32(e2v, gAi, p2 + gAi + go));
                e3v = norm(__viaddmax_s32(e3v, gAi, p3 + gAi + go));
                ROW(6)[rj] = e0v;
                ROW(7)[rj] = e1v;
                ROW(8)[rj] = e2v;
                ROW(9)[rj] = e3v;
                x0 = max(d0 + sg, e0v);
                x1 = max(d1 + sg, e1v);
                x2 = max(d2 + sg, e2v);
                x3 = max(d3 + sg, e3v);
                if (rowarcs) {
                    x0 = max(x0, ROW(11)[rj]);
                    x1 = max(x1, ROW(12)[rj]);
                    x2 = max(x2, ROW(13)[rj]);
                    x3 = max(x3, ROW(14)[rj]);
                    ROW(11)[rj] = NEG;
                    ROW(12)[rj] = NEG;
                    ROW(13)[rj] = NEG;
                    ROW(14)[rj] = NEG;
                }
            }
            const int pa = gbc >> 4;
            // NO_NO; OP_NO = max(OP_NO above, NO_NO); NO_OP = prefix max of NO_NO
            const int M0 = fscan_prefix(x0, pa, gdel, Pc0, lane);
            const int M4 = act ? norm(max(p4, M0)) : NEG;
            const int M5 = prefix_max_carry(act ? M0 : NEG, C5, lane);
            // NO_X with NO_OP + X; OP_X = max(OP_X above, NO_X)
            const int M2 = fscan_prefix(act ? max(x2, M5 + X) : NEG, pa, gdel, Pc2, lane);
            const int M6 = act ? norm(max(p6, M2)) : NEG;
            // X_NO with OP_NO + X; X_OP = prefix max of X_NO
            const int M1 = fscan_prefix(act ? max(x1, M4 + X) : NEG, pa, gdel, Pc1, lane);
            const int M7 = prefix_max_carry(act ? M1 : NEG, C7, lane);
            // X_X with OP_X + X and X_OP + X
            const int M3 = fscan_prefix(act ? max(x3, max(M6 + X, M7 + X)) : NEG, pa, gdel, Pc3, lane);
            if (act) {
                ROW(0)[rj] = M0;
                ROW(1)[rj] = M1;
                ROW(2)[rj] = M2;
                ROW(3)[rj] = M3;
                ROW(4)[rj] = M4;
                ROW(5)[rj] = M6;
                Mg[roff + j] = M0;
                Mg[mstride + roff + j] = M1;
                Mg[2 * mstride + roff + j] = M2;
                Mg[3 * mstride + roff + j] = M3;
                if (NS == 8) {
                    Mg[4 * mstride + roff + j] = M4;
                    Mg[5 * mstride + roff + j] = M5;
                    Mg[6 * mstride + roff + j] = M6;
                    Mg[7 * mstride + roff + j] = M7;
                }
            }
        }
        __syncwarp();
        if (DWRITE && i == dw_row) {
            // fill_D_entries (struct-local: the best non-open state); without
            // lonely pairs or with stacking also the inner arc match's term
            while (dwp < ndw) {
                const int q = dwp + lane;
                int4 e = make_int4(0, -1, 0, 0);
                if (q < ndw) e = dw[q];
                const bool mine = q < ndw && e.y == i;
                if (mine) {
                    const int rz = RG(e.z);
                    const int mv = max(max(ROW(0)[rz], ROW(1)[rz]), max(ROW(2)[rz], ROW(3)[rz]));
                    int v = mv + e.w;
                    if (P.flags & (PF_NOLP | PF_STACK)) v = max(v, inner_term<WAIT>(P, dw + q, status, abort_flag));
                    st_volatile(Dp + e.x, norm(v));
                }
                const int cnt = __popc(__ballot_sync(0xffffffffu, mine));
                dwp += cnt;
                if (cnt < 32) break;
            }
            dw_row = dwp < ndw ? dw[dwp].y : INT_MAX;
        }
        if (i + 1 < ar) {
            // columns entering the band with row i+1: M above them is -inf,
            // their E starts at -inf, their gap prefix is staged
            const int Ln = min(br, rnxt.y + 1);
            for (int j = max(hi + 1, bl + 1) + lane; j < Ln; j += 32) {
                const int rj = RG(j);
#pragma unroll
                for (int k = 0; k < 10; ++k) ROW(k)[rj] = NEG;
                gBs[rj] = P.gbc[j];
            }
        }
        __syncwarp();
    }
#undef ROW
#undef RG
}

// KEEP: the chunk keeps its group rectangles (PairDev::rect); a group with
// a kept rectangle writes all eight states there, interleaved by row (row
// i-al of state s at rect + 8 rect_off + (i-al) 8w + s w, w = br - bl), so
// that the traceback walks it instead of recomputing it.
template <bool FAST, bool KEEP>
__global__ void __launch_bounds__(SL_FILL_WARPS * 32)
    sankoff_sl_fill_kernel(const PairDev *__restrict__ pairs, const int2 *__restrict__ queue,
                           int nitems, int *scratch,
                           long long scratch_stride, int sw, int rb, unsigned int *qhead, int *status,
                           int *abort_flag_ptr) {
    extern __shared__ int smem[];
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    int *sm = smem + warp * (FAST ? slf_warp_ints(rb) : sl_warp_ints(sw, rb));
    // 4 state matrices per warp slot
    int *Mg = scratch + ((long long)blockIdx.x * SL_FILL_WARPS + warp) * scratch_stride * 4;
    volatile int *abort_flag = abort_flag_ptr;
    while (true) {
        int idx = 0;
        if (lane == 0) idx = (int)atomicAdd(qhead, 1u);
        idx = __shfl_sync(0xffffffffu, idx, 0);
        if (idx >= nitems || *abort_flag) break;
        const int2 qi = queue[idx];  // (pair, group)
        const PairDev &P = pairs[qi.x];
        const GroupItem it = P.groups[qi.y];
        const int4 *__restrict__ dw = P.dw;
        if (it.top) {
            const int base = (int)(sm - smem);
            run_top<false>(P, it.cpl, base, rb, status, abort_flag, nullptr);
        } else if (KEEP && P.rect && it.rect_off >= 0) {
            const int w = it.br - it.bl;
            int *Mk = P.rect + 8ll * it.rect_off;
            if (FAST)
                run_group_slf<true, true, 8>(P, it.al, it.ar, it.bl, it.br, Mk, w, 8 * w, (int)(sm - smem), rb,
                                             dw + it.dw_start, it.dw_count, status, abort_flag);
            else
                run_group_sl<true, true, 8>(P, it.al, it.ar, it.bl, it.br, Mk, w, 8 * w, sm, sw,
                                            dw + it.dw_start, it.dw_count, status, abort_flag);
        } else if (FAST) {
            run_group_slf<true, true, 4>(P, it.al, it.ar, it.bl, it.br, Mg, scratch_stride, sw, (int)(sm - smem), rb,
                                dw + it.dw_start, it.dw_count, status, abort_flag);
        } else {
            run_group_sl<true, true, 4>(P, it.al, it.ar, it.bl, it.br, Mg, scratch_stride, sw, sm, sw,
                                        dw + it.dw_start, it.dw_count, status, abort_flag);
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------- traceback

// trace_in_arcmatch (aligner.cc:1233-1343) as a loop over (state, i, j);
// M of state s is Mg + s*mstride (the top level has only state NO_NO).
static __device__ __noinline__ void walk_sl(Walker &w, const int *Mg, long long mstride, int pitch,
                                            int al, int bl, int state, int i, int j, bool tl,
                                            int *status, int lam = 0) {
    const PairDev &P = w.P;
    const int tlam = tl ? lam : 0;  // top level of normalized / penalized alignment
    const bool local = P.flags & PF_SEQU_LOCAL;
    const int fe = P.free_endgaps;
    const int go = P.go, X = P.excl;
#define MS(s, x, y) Mg[(long long)(s) * mstride + (long long)((x) - al) * pitch + ((y) - bl)]
    for (int guard = 0; guard < 8 * (P.n + P.m + 4); ++guard) {
        const int Mij = MS(state, i, j);
        if (tl && local && Mij == 0) {
            P.res[R_MINI] = i;
            P.res[R_MINJ] = j;
            return;
        }
        if (i <= al) {
            if (state == S_NO_NO || state == S_OP_NO || state == S_X_NO)
                if (!(tl && (local || (fe & 1))))
                    for (int k = j; k > bl; --k) w.emit(-1, k);
            return;
        }
        if (j <= bl) {
            if (state == S_NO_NO || state == S_NO_OP || state == S_NO_X)
                if (!(tl && (local || (fe & 4))))
                    for (int k = i; k > al; --k) w.emit(k, -1);
            return;
        }
        bool noex = false;
        switch (state) {
        case S_NO_NO: noex = true; break;
        case S_OP_NO:
            if (Mij == MS(state, i - 1, j)) { --i; continue; }
            if (Mij == MS(S_NO_NO, i, j)) { state = S_NO_NO; continue; }
            return;
        case S_NO_OP:
            if (Mij == MS(state, i, j - 1)) { --j; continue; }
            if (Mij == MS(S_NO_NO, i, j)) { state = S_NO_NO; continue; }
            return;
        case S_NO_X:
            if (Mij == MS(S_NO_OP, i, j) + X) { state = S_NO_OP; continue; }
            noex = true;
            break;
        case S_OP_X:
            if (Mij == MS(state, i - 1, j)) { --i; continue; }
            if (Mij == MS(S_NO_X, i, j)) { state = S_NO_X; continue; }
            return;
        case S_X_NO:
            if (Mij == MS(S_OP_NO, i, j) + X) { state = S_OP_NO; continue; }
            noex = true;
            break;
        case S_X_OP:
            if (Mij == MS(state, i, j - 1)) { --j; continue; }
            if (Mij == MS(S_X_NO, i, j)) { state = S_X_NO; continue; }
            return;
        case S_X_X:
            if (Mij == MS(S_OP_X, i, j) + X) { state = S_OP_X; continue; }
            if (Mij == MS(S_X_OP, i, j) + X) { state = S_X_OP; continue; }
            noex = true;
            break;
        }
        if (!noex) return;
        // trace_noex (aligner.cc:1082-1229) in `state`
        if (a_match(P, i, j) && w.valid(i - 1, j - 1) &&
            Mij == MS(state, i - 1, j - 1) + sigma_at(P, i, j) - 2 * tlam) {
            w.emit(i, j);
            --i;
            --j;
            continue;
        }
        bool found = false;
        if (go == 0) {
            if (a_del(P, i, j) && w.valid(i - 1, j) && Mij == MS(state, i - 1, j) + P.gapA[i] - tlam) {
                w.emit(i, -1);
                --i;
                continue;
            }
            if (a_ins(P, i, j) && w.valid(i, j - 1) && Mij == MS(state, i, j - 1) + P.gapB[j] - tlam) {
                w.emit(-1, j);
                --j;
                continue;
            }
        } else {
            int gap = go;
            for (int k = 1; i >= al + k && a_del(P, i - k + 1, j); ++k) {
                if (!w.valid(i - k, j)) break;
                gap += P.gapA[i - k + 1] - tlam;
                if (Mij == MS(state, i - k, j) + gap) {
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
                if (Mij == MS(state, i, j - k) + gap) {
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
            if (Mij == MS(state, alq - 1, blq - 1) + P.D[ent.x] - tlam * ((i - alq + 1) + (j - blq + 1))) {
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
#undef MS
}

template <bool FAST>
__global__ void __launch_bounds__(TRACE_WARPS * 32)
    sankoff_sl_trace_kernel(const PairDev *__restrict__ pairs, int npairs, int *scratch,
                            long long scratch_stride, int sw, int rb, int *status, TraceSel sel) {
    extern __shared__ int smem[];
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const int wi = blockIdx.x * TRACE_WARPS + warp;
    if (wi >= (sel.items ? sel.nitems : npairs)) return;
    const int pair = sel.items ? sel.items[wi] : wi;
    const PairDev &P = pairs[pair];
    if (!(P.flags & PF_TRACE)) return;
    // a fill that gave up (bounded wait) left the matrices incomplete: no walk
    if (*(volatile int *)status & ST_TIMEOUT) return;
    const int lam = sel.lam ? sel.lam[pair] : 0;
    int *sm = smem + warp * (FAST ? slf_warp_ints(rb) : SL_ROWS * sw);
    int *Mg = scratch + (long long)pair * scratch_stride * 8;
    int dummy_abort = 0;
    Walker w(P);
    int nseg = 0;
    int qhead = 0;
    if (lane == 0) {
        if (!(sel.flags & TRACE_KEEP_MIN)) {
            P.res[R_MINI] = 1;
            P.res[R_MINJ] = 1;
        }
        const int sA = sel.rst ? sel.rst[pair].x : 1, sB = sel.rst ? sel.rst[pair].y : 1;
        walk_sl(w, P.topM + (size_t)(sA - 1) * (P.m + 1) + (sB - 1), 0, P.m + 1, sA - 1, sB - 1, S_NO_NO,
                P.res[R_MAXI], P.res[R_MAXJ], true, status, lam);
        P.segs[nseg++] = make_int4(-1, 0, w.ntok, 0);
    }
    if (sel.flags & TRACE_TOP_ONLY) return;
    int qtail = __shfl_sync(0xffffffffu, w.qtail, 0);
    while (qhead < qtail) {
        int4 qe = make_int4(-1, 0, 0, 0);
        if (lane == 0 && qhead < P.tq_cap) qe = P.tq[qhead];
        const int k = __shfl_sync(0xffffffffu, qe.x, 0), kpos = __shfl_sync(0xffffffffu, qe.y, 0);
        const int lefts = __shfl_sync(0xffffffffu, qe.z, 0), rights = __shfl_sync(0xffffffffu, qe.w, 0);
        ++qhead;
        if (k < 0) break;
        const int4 ends = trace_ends(lefts, rights);  // a.l, a.r, b.l, b.r
        if (lefts & TQ_CHAIN) {
            if (lane == 0) trace_chain(w, k, kpos, ends, nseg, status);
            __syncwarp();
            qtail = __shfl_sync(0xffffffffu, w.qtail, 0);
            continue;
        }
        if ((P.flags & (PF_STACK | PF_NOLP)) == PF_STACK) {
            int stacked = 0;
            if (lane == 0) stacked = trace_stack(w, k, kpos, ends, nseg);
            if (__shfl_sync(0xffffffffu, stacked, 0)) {
                qtail = __shfl_sync(0xffffffffu, w.qtail, 0);
                continue;
            }
        }
        // the arc match's eight state matrices: its group's kept rectangle
        // from the fill, else recomputed into the pair's scratch slot
        const int2 kr = P.am_rect ? P.am_rect[k] : make_int2(-1, 0);
        const int *Mw = Mg;
        long long ms = scratch_stride;
        int pw = sw;
        if (kr.x >= 0) {
            Mw = P.rect + 8ll * kr.x;
            ms = kr.y;
            pw = 8 * kr.y;
        } else if (FAST) {
            run_group_slf<false, false, 8>(P, ends.x, ends.y, ends.z, ends.w, Mg, scratch_stride, sw,
                                           (int)(sm - smem), rb, nullptr, 0, status, (volatile int *)&dummy_abort);
        } else {
            run_group_sl<false, false, 8>(P, ends.x, ends.y, ends.z, ends.w, Mg, scratch_stride, sw, sm, sw,
                                          nullptr, 0, status, (volatile int *)&dummy_abort);
        }
        __syncwarp();
        if (lane == 0) {
            // trace_arcmatch, struct-local branch (aligner.cc:1014-1026): first
            // non-open state whose value explains D(am); for the inner arc
            // match of a no-lonely-pairs stack (aligner.cc:1062-1074) the
            // queue entry carries D(outer) - score(outer) - score(am)
            const int ar = ends.y, br = ends.w;
            const long long o = (long long)(ar - 1 - ends.x) * pw + (br - 1 - ends.z);
            const bool nolp = P.flags & PF_NOLP;
            const int dv = nolp ? kpos : P.D[kpos], sc = nolp ? 0 : P.am_score[k];
            const int start = w.ntok;
            for (int s2 = 0; s2 < 4; ++s2) {
                if (dv == Mw[s2 * ms + o] + sc) {
                    walk_sl(w, Mw, ms, pw, ends.x, ends.z, s2, ar - 1, br - 1, false, status);
                    break;
                }
            }
            if (nseg < P.tq_cap + 1) P.segs[nseg] = make_int4(k, start, w.ntok, 0);
            ++nseg;
        }
        __syncwarp();
        qtail = __shfl_sync(0xffffffffu, w.qtail, 0);
    }
    if (lane == 0) {
        P.res[R_NTOK] = w.ntok;
        P.res[R_NSEG] = nseg;
        if (!w.ok) atomicOr(status, ST_OVERFLOW);
    }
}

// ---------------------------------------------------------------- launchers

static size_t sl_fill_smem(int sw, int rb, bool fast) {
    return (size_t)SL_FILL_WARPS * (fast ? slf_warp_ints(rb) : sl_warp_ints(sw, rb)) * sizeof(int);
}
static size_t sl_trace_smem(int sw, int rb, bool fast) {
    return (size_t)TRACE_WARPS * (fast ? slf_warp_ints(rb) : SL_ROWS * sw) * sizeof(int);
}

cudaError_t sl_prepare(int sw, int rb, bool fast, bool keep, int *blocks_per_sm) {
    const size_t smem = sl_fill_smem(sw, rb, fast);
    const size_t smem_t = sl_trace_smem(sw, rb, fast);
    int optin = 0, dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e != cudaSuccess) return e;
    if (smem > (size_t)optin || smem_t > (size_t)optin) {
        *blocks_per_sm = 0;  // does not fit: the caller reports it
        return cudaSuccess;
    }
    const void *k = fast ? (const void *)sankoff_sl_fill_kernel<true, false>
                         : (const void *)sankoff_sl_fill_kernel<false, false>;
    const void *kk = fast ? (const void *)sankoff_sl_fill_kernel<true, true>
                          : (const void *)sankoff_sl_fill_kernel<false, true>;
    e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(kk, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const void *kt = fast ? (const void *)sankoff_sl_trace_kernel<true> : (const void *)sankoff_sl_trace_kernel<false>;
    e = cudaFuncSetAttribute(kt, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_t);
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, keep ? kk : k, SL_FILL_WARPS * 32, smem);
}

int sl_fill_warps_per_block() { return SL_FILL_WARPS; }

cudaError_t launch_sl_fill(const PairDev *pairs, const int2 *queue, int nitems,
                           int *scratch, long long scratch_stride, int sw, int rb, bool fast, bool keep,
                           unsigned int *qhead, int *status, int *abort_flag, int blocks, cudaStream_t st) {
    const size_t smem = sl_fill_smem(sw, rb, fast);
    auto kern = fast ? (keep ? sankoff_sl_fill_kernel<true, true> : sankoff_sl_fill_kernel<true, false>)
                     : (keep ? sankoff_sl_fill_kernel<false, true> : sankoff_sl_fill_kernel<false, false>);
    kern<<<blocks, SL_FILL_WARPS * 32, smem, st>>>(pairs, queue, nitems, scratch, scratch_stride, sw, rb, qhead,
                                                   status, abort_flag);
    return cudaGetLastError();
}

cudaError_t launch_sl_trace(const PairDev *pairs, int npairs, int *scratch, long long scratch_stride, int sw,
                            int rb, bool fast, int *status, cudaStream_t st, TraceSel sel) {
    const size_t smem = sl_trace_smem(sw, rb, fast);
    const int nw = sel.items ? sel.nitems : npairs;
    if (nw <= 0) return cudaSuccess;
    const int blocks = (nw + TRACE_WARPS - 1) / TRACE_WARPS;
    if (fast)
        sankoff_sl_trace_kernel<true><<<blocks, TRACE_WARPS * 32, smem, st>>>(pairs, npairs, scratch, scratch_stride,
                                                                           sw, rb, status, sel);
    else
        sankoff_sl_trace_kernel<false><<<blocks, TRACE_WARPS * 32, smem, st>>>(pairs, npairs, scratch,
                                                                            scratch_stride, sw, rb, status, sel);
    return cudaGetLastError();
}

}  // namespace lcg
