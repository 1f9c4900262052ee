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

__global__ void __launch_bounds__(SL_FILL_WARPS * 32)
    sankoff_sl_fill_kernel(const PairDev *__restrict__ pairs, const int2 *__restrict__ queue,
                           int nitems, int *scratch,
                           long long scratch_stride, int sw, int rb, unsigned int *qhead, int *status,
                           int *abort_flag_ptr) {
    extern __shared__ int smem[];
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    int *sm = smem + warp * sl_warp_ints(sw, rb);
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

__global__ void __launch_bounds__(TRACE_WARPS * 32)
    sankoff_sl_trace_kernel(const PairDev *__restrict__ pairs, int npairs, int *scratch,
                            long long scratch_stride, int sw, int *status, TraceSel sel) {
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
    int *sm = smem + warp * SL_ROWS * sw;
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
        run_group_sl<false, false, 8>(P, ends.x, ends.y, ends.z, ends.w, Mg, scratch_stride, sw, sm, sw,
                                      nullptr, 0, status, (volatile int *)&dummy_abort);
        __syncwarp();
        if (lane == 0) {
            // trace_arcmatch, struct-local branch (aligner.cc:1014-1026): first
            // non-open state whose value explains D(am); for the inner arc
            // match of a no-lonely-pairs stack (aligner.cc:1062-1074) the
            // queue entry carries D(outer) - score(outer) - score(am)
            const int ar = ends.y, br = ends.w;
            const long long o = (long long)(ar - 1 - ends.x) * sw + (br - 1 - ends.z);
            const bool nolp = P.flags & PF_NOLP;
            const int dv = nolp ? kpos : P.D[kpos], sc = nolp ? 0 : P.am_score[k];
            const int start = w.ntok;
            for (int s2 = 0; s2 < 4; ++s2) {
                if (dv == Mg[s2 * scratch_stride + o] + sc) {
                    walk_sl(w, Mg, scratch_stride, sw, ends.x, ends.z, s2, ar - 1, br - 1, false, status);
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

cudaError_t sl_prepare(int sw, int rb, int *blocks_per_sm) {
    size_t smem = (size_t)SL_FILL_WARPS * sl_warp_ints(sw, rb) * sizeof(int);
    size_t smem_t = (size_t)TRACE_WARPS * SL_ROWS * sw * sizeof(int);
    cudaError_t e = cudaFuncSetAttribute(sankoff_sl_fill_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(sankoff_sl_trace_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem_t);
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, sankoff_sl_fill_kernel,
                                                         SL_FILL_WARPS * 32, smem);
}

int sl_fill_warps_per_block() { return SL_FILL_WARPS; }

cudaError_t launch_sl_fill(const PairDev *pairs, const int2 *queue, int nitems,
                           int *scratch, long long scratch_stride, int sw, int rb, unsigned int *qhead,
                           int *status, int *abort_flag, int blocks, cudaStream_t st) {
    size_t smem = (size_t)SL_FILL_WARPS * sl_warp_ints(sw, rb) * sizeof(int);
    sankoff_sl_fill_kernel<<<blocks, SL_FILL_WARPS * 32, smem, st>>>(
        pairs, queue, nitems, scratch, scratch_stride, sw, rb, qhead, status, abort_flag);
    return cudaGetLastError();
}

cudaError_t launch_sl_trace(const PairDev *pairs, int npairs, int *scratch,
                            long long scratch_stride, int sw, int *status, cudaStream_t st, TraceSel sel) {
    size_t smem = (size_t)TRACE_WARPS * SL_ROWS * sw * sizeof(int);
    const int nw = sel.items ? sel.nitems : npairs;
    if (nw <= 0) return cudaSuccess;
    int blocks = (nw + TRACE_WARPS - 1) / TRACE_WARPS;
    sankoff_sl_trace_kernel<<<blocks, TRACE_WARPS * 32, smem, st>>>(pairs, npairs, scratch,
                                                                    scratch_stride, sw, status, sel);
    return cudaGetLastError();
}

}  // namespace lcg
