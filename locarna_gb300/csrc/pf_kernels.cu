// LocARNA-P partition function on the GPU: the inside (forward) pass as a
// persistent dataflow kernel over left-end groups, and its hand-written
// adjoint (backward) pass, which yields arc-match and base-match
// probabilities and the derivatives of log Z with respect to the Boltzmann
// weights in one sweep.
//
// Reference: AlignerP<T>::align_inside (src/LocARNA/aligner_p.icc:148-438)
// for the forward recursions; the outside algorithm and the probability
// computations (aligner_p.icc:450-1399) are replaced by the adjoint of the
// forward DAG: d Z / d D(am) plays the role of the outside value D'(am)
// (am prob = D * dZ/dD / Z, aligner_p.icc:1177-1180), and the expected number
// of uses of a base match (i,j) is the base-match probability
// (aligner_p.icc:1201-1399 with min_am_prob 0).
//
// Recursions per group (al,bl), split so that no term is subtracted
// (the reference computes E*g + (M-E)*g*o, aligner_p.icc:209-229):
//   X(i,j) = M(i-1,j-1) bm(i,j) + sum_am M(a.l-1,b.l-1) D(am) s
//   E(i,j) = E(i-1,j) gA(i) + N(i-1,j) gA(i) o        N = X + F  (= M - E)
//   F(i,j) = F(i,j-1) gB(j) + Q(i,j-1) gB(j) o        Q = X + E  (= M - F)
//   M = X + E + F,  D(am) = M(ar-1,br-1) w(am)
// F is a linear recurrence along the row and is evaluated with a warp scan.
//
// Scaling. With a per-position factor c, every group's values are kept
// relative to its own left ends: M'(i,j) = M(i,j) c^-((i-al)+(j-bl)). This is
// the same recursion with bm/c^2, gA/c, gB/c and the arc factor s/c^4, and
// Z = Z' c^(n+m); probabilities are unchanged. The FP32 path uses c from a
// host estimate so values stay well inside the float range; FP64 uses c = 1.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstdlib>
#include <stdint.h>

#include "lcg_device.cuh"
#include "pf_device.cuh"

namespace lcg {

constexpr int PF_WARPS = 4;
// resident blocks per SM the register budget targets: 8 (32 warps) in FP32;
// FP64 rows take twice the shared memory, 5 blocks fit
template <typename T>
__host__ __device__ constexpr int pf_min_blocks() {
    return sizeof(T) == 4 ? 8 : 5;
}
constexpr long long PF_SPIN_LIMIT = 1ll << 22;

__device__ __forceinline__ bool pf_not_ready(double v) {
    return __double_as_longlong(v) == PF_NOT_READY_F64;
}
__device__ __forceinline__ bool pf_not_ready(float v) { return __float_as_int(v) == PF_NOT_READY_F32; }
__device__ __forceinline__ double pf_ld(const double *p) { return *(const volatile double *)p; }
__device__ __forceinline__ float pf_ld(const float *p) { return *(const volatile float *)p; }

template <typename T>
__device__ __forceinline__ T pf_wait(const T *p, int *status, volatile int *abort_flag) {
    T v = pf_ld(p);
    long long spins = 0;
    while (pf_not_ready(v)) {
        __nanosleep(64);
        v = pf_ld(p);
        if (++spins > PF_SPIN_LIMIT || *abort_flag) {
            atomicOr(status, ST_TIMEOUT);
            *abort_flag = 1;
            return T(0);
        }
    }
    return v;
}

extern __shared__ unsigned char pf_smem_raw[];

// Shared-memory rows per warp (T each), ring buffers of rb entries (a
// multiple of 32) indexed by column j mod rb: M and N of the previous / current row, E, and
// the arc-term sums of the current row. RB exceeds the span of any two
// consecutive band rows, so live columns never alias. The backward pass
// reuses E as E_bar and Ar as the row's X_bar.
template <typename T>
struct PFRows {
    T *Mp, *Mc, *Np, *Nc, *E, *Ar;
    int rb;
    unsigned magic;  // j / rb = umulhi(j, magic) for 0 <= j < 2^20
};

constexpr int PF_RING_ROWS = 6;

template <typename T>
__device__ __forceinline__ PFRows<T> pf_rows(int warp, int rb) {
    T *base = reinterpret_cast<T *>(pf_smem_raw) + (size_t)warp * PF_RING_ROWS * rb;
    PFRows<T> r;
    r.Mp = base;
    r.Mc = base + rb;
    r.Np = base + 2 * rb;
    r.Nc = base + 3 * rb;
    r.E = base + 4 * rb;
    r.Ar = base + 5 * rb;
    r.rb = rb;
    r.magic = 0xFFFFFFFFu / (unsigned)rb + 1u;
    return r;
}

// Sum-product sweep of one group (or the top level) in the scaled frame; M of
// the rectangle goes to Mg (row i-al, column j-bl, pitch `pitch`), with SAVE
// also the cells around the band the adjoint reads, and with SAVE and SAVEEF
// E and F (Eg, Fg; only the gap gradients read them).
// Arc terms per row: the row's candidates (arc matches with a.r = i, a.l
// descending) are read 32 at a time until the first a.l <= al, and each term
// M(a.l-1,b.l-1) D(am) s is summed into its column with a shared-memory
// atomicAdd. COUNTU counts the uses of every D entry (for the backward pass).
template <typename T, bool WAIT, bool DWRITE, bool COUNTU, bool SAVE, bool SAVEEF = true>
__device__ void pf_group_sweep(const PFPair<T> &P, int al, int ar, int bl, int br, T *__restrict__ Mg,
                               T *__restrict__ Eg, T *__restrict__ Fg, int pitch, PFRows<T> R,
                               const int4 *__restrict__ dw, int ndw, int *status, volatile int *abort_flag) {
    const int lane = threadIdx.x & 31;
    const int m1 = P.m + 1;
    const T o = P.o, arcf = P.arcf;
#define RG(j) ((j) - R.rb * (int)__umulhi((unsigned)(j), R.magic))
    // E and the arc-term sums start at zero; the cell sweep puts zero back
    // into every arc-term column it reads, so no row needs a clearing pass
    for (int c = lane; c < R.rb; c += 32) {
        R.E[c] = T(0);
        R.Ar[c] = T(0);
    }
    // row al: M(al,bl) = 1/s, M(al,j) = (o/s) prod gB (aligner_p.icc:149-190)
    const int L0 = min(br, P.rowinfo[al].y + 1);
    {
        T carry = o * P.inv_s;
        for (int base = bl + 1; base < L0; base += 32) {
            const int j = base + lane;
            T v = j < L0 ? P.gB[j] : T(1);
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                T t = __shfl_up_sync(0xffffffffu, v, off);
                if (lane >= off) v *= t;
            }
            const T val = carry * v;
            if (j < L0) {
                R.Mp[RG(j)] = val;
                R.Np[RG(j)] = val;
                Mg[j - bl] = val;
                if (SAVE && SAVEEF) {
                    Eg[j - bl] = T(0);
                    Fg[j - bl] = T(0);
                }
            }
            carry = __shfl_sync(0xffffffffu, val, 31);
        }
        if (lane == 0) {
            R.Mp[RG(bl)] = P.inv_s;
            R.Np[RG(bl)] = P.inv_s;
            Mg[0] = P.inv_s;
            if (SAVE && SAVEEF) {
                Eg[0] = T(0);
                Fg[0] = T(0);
            }
        }
        if (al + 1 < ar) {
            const int L1 = min(br, P.rowinfo[al + 1].y + 1);
            for (int j = L0 + lane; j < L1; j += 32) {
                R.Mp[RG(j)] = T(0);
                R.Np[RG(j)] = T(0);
                if (SAVE) {
                    Mg[j - bl] = T(0);
                    if (SAVEEF) {
                        Eg[j - bl] = T(0);
                        Fg[j - bl] = T(0);
                    }
                }
            }
        }
    }
    __syncwarp();
    T colval = o * P.inv_s;
    int dwp = 0;
    for (int i = al + 1; i < ar; ++i) {
        const int4 ri = P.rowinfo[i];
        const int2 ra = P.rowarc[i];
        const int minc = ri.x;
        const int lo = max(bl + 1, minc), hi = min(br - 1, ri.y);
        const T gAi = P.gA[i];
        // ---- arc-match terms of row i into Ar[lo..hi]: two batches of 32
        // entries per step, their loads issued together
        bool rowarcs = false;
        for (int e0 = ra.x; e0 < ra.y; e0 += 64) {
            int2 en[2];
            bool okA[2];
            unsigned ball[2];
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int e = e0 + 32 * u + lane;
                en[u] = e < ra.y ? P.crow[e] : make_int2(0xffff, 0);
            }
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int ca = en[u].x & 0xffff;
                okA[u] = ca >= al && ca != 0xffff;  // a.l > al
                ball[u] = __ballot_sync(0xffffffffu, okA[u]);
            }
            if (ball[0] == 0u) break;
            rowarcs = true;
            bool ok[2];
            T dv[2], mv[2];
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int ca = en[u].x & 0xffff, cbl = en[u].x >> 16;  // inner corner (a.l-1, b.l-1)
                ok[u] = okA[u] && cbl >= bl && en[u].y >= lo && en[u].y <= hi;
                const int e = e0 + 32 * u + lane;
                dv[u] = ok[u] ? pf_ld(P.D + e) : T(0);
                mv[u] = ok[u] ? Mg[(size_t)(ca - al) * pitch + (cbl - bl)] : T(0);
            }
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                if (ok[u]) {
                    const int e = e0 + 32 * u + lane;
                    if (WAIT && pf_not_ready(dv[u])) dv[u] = pf_wait(P.D + e, status, abort_flag);
                    atomicAdd(&R.Ar[RG(en[u].y)], mv[u] * dv[u] * arcf);
                    if (COUNTU) atomicAdd(P.cnt + e, 1);
                }
            }
            if (ball[0] != 0xffffffffu || ball[1] != 0xffffffffu) break;
        }
        __syncwarp();
        T B = T(0);
        if (minc <= bl) {
            colval *= gAi;
            B = colval;
            if (lane == 0) Mg[(size_t)(i - al) * pitch] = B;
        }
        if (lane == 0) {
            R.Mc[RG(lo - 1)] = B;
            R.Nc[RG(lo - 1)] = B;
            if (SAVE) {
                // the cell left of the row's band (column bl, or a zero cell)
                Mg[(size_t)(i - al) * pitch + (lo - 1 - bl)] = B;
                if (SAVEEF) {
                    Eg[(size_t)(i - al) * pitch + (lo - 1 - bl)] = T(0);
                    Fg[(size_t)(i - al) * pitch + (lo - 1 - bl)] = T(0);
                }
            }
        }
        const T *bmrow = P.bm + (size_t)i * m1;
        const size_t roff = (size_t)(i - al) * pitch - bl;
        T Fc = T(0), Qc = B;
        for (int base = lo; base <= hi; base += 32) {
            const int j = base + lane;
            const bool act = j <= hi;
            T X = T(0), Ei = T(0), g = T(0);
            if (act) {
                Ei = R.E[RG(j)] * gAi + R.Np[RG(j)] * gAi * o;
                X = R.Mp[RG(j - 1)] * bmrow[j];
                if (rowarcs) {
                    X += R.Ar[RG(j)];
                    R.Ar[RG(j)] = T(0);
                }
                g = P.gB[j];
            }
            // F(j) = gB(j) F(j-1) + gB(j) o Q(j-1): linear warp scan
            const T Q = X + Ei;
            T Qp = __shfl_up_sync(0xffffffffu, Q, 1);
            if (lane == 0) Qp = Qc;
            T a = T(1), b = T(0);
            if (act) {
                a = g;
                b = g * o * Qp;
            }
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const T a1 = __shfl_up_sync(0xffffffffu, a, off);
                const T b1 = __shfl_up_sync(0xffffffffu, b, off);
                if (lane >= off) {
                    b = a * b1 + b;
                    a = a * a1;
                }
            }
            const T F = a * Fc + b;
            if (act) {
                const T M = X + Ei + F;
                R.E[RG(j)] = Ei;
                R.Mc[RG(j)] = M;
                R.Nc[RG(j)] = X + F;
                Mg[roff + j] = M;
                if (SAVE && SAVEEF) {
                    Eg[roff + j] = Ei;
                    Fg[roff + j] = F;
                }
            }
            Fc = __shfl_sync(0xffffffffu, F, 31);
            Qc = __shfl_sync(0xffffffffu, Q, 31);
        }
        __syncwarp();
        if (DWRITE) {
            while (dwp < ndw) {
                const int qq = dwp + lane;
                int4 e = make_int4(0, -1, 0, 0);
                if (qq < ndw) e = dw[qq];
                const bool mine = qq < ndw && e.y == i;
                if (mine) {
                    const T v = R.Mc[RG(e.z)] * P.w[e.x];
                    *(volatile T *)(P.D + e.x) = v;
                }
                const int cnt = __popc(__ballot_sync(0xffffffffu, mine));
                dwp += cnt;
                if (cnt < 32) break;
            }
        }
        if (i + 1 < ar) {
            // columns entering the band with row i+1 start from zero
            const int Ln = min(br, P.rowinfo[i + 1].y + 1);
            for (int j = max(hi + 1, bl + 1) + lane; j < Ln; j += 32) {
                R.Mc[RG(j)] = T(0);
                R.Nc[RG(j)] = T(0);
                R.E[RG(j)] = T(0);
                if (SAVE) {
                    Mg[(size_t)(i - al) * pitch + (j - bl)] = T(0);
                    if (SAVEEF) {
                        Eg[(size_t)(i - al) * pitch + (j - bl)] = T(0);
                        Fg[(size_t)(i - al) * pitch + (j - bl)] = T(0);
                    }
                }
            }
        }
        __syncwarp();
        T *t;
        t = R.Mp; R.Mp = R.Mc; R.Mc = t;
        t = R.Np; R.Np = R.Nc; R.Nc = t;
    }
#undef RG
}

// KEEP: 0, or the pairs' rect_states (the groups' rectangles are kept for
// the backward pass, M alone or M, E and F)
template <typename T, bool COUNTU, int KEEP = 0>
__global__ void __launch_bounds__(PF_WARPS * 32, pf_min_blocks<T>())
    pf_fwd_kernel(const PFPair<T> *__restrict__ pairs, const int2 *__restrict__ queue, int nitems,
                  T *scratch, long long stride, int pitch, int rb,
                  unsigned int *qhead, int *status, int *abort_ptr) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    PFRows<T> R = pf_rows<T>(warp, rb);
    T *Mg = scratch + ((long long)blockIdx.x * PF_WARPS + warp) * stride;
    volatile int *abort_flag = abort_ptr;
    while (true) {
        int idx = 0;
        if (lane == 0) idx = (int)atomicAdd(qhead, 1u);
        idx = __shfl_sync(0xffffffffu, idx, 0);
        if (idx >= nitems || *abort_flag) break;
        const int2 qi = queue[idx];  // (pair, group)
        const PFPair<T> &P = pairs[qi.x];
        const GroupItem it = P.groups[qi.y];
        if (it.top) {
            pf_group_sweep<T, true, false, COUNTU, false>(P, 0, P.n + 1, 0, P.m + 1, P.topM, nullptr, nullptr,
                                                          P.m + 1, R, nullptr, 0, status, abort_flag);
            __syncwarp();
            if (lane == 0) {
                const T z = P.topM[(size_t)P.n * (P.m + 1) + P.m];
                P.res[0] = log((double)z);
            }
        } else if (KEEP > 0 && P.rect && it.rect_off >= 0) {
            const int w = it.br - it.bl;
            const size_t sz = (size_t)(it.ar - it.al) * w;
            T *Mk = P.rect + (size_t)KEEP * it.rect_off;
            pf_group_sweep<T, true, true, COUNTU, true, KEEP == 3>(P, it.al, it.ar, it.bl, it.br, Mk, Mk + sz,
                                                                   Mk + 2 * sz, w, R, P.dw + it.dw_start,
                                                                   it.dw_count, status, abort_flag);
        } else {
            pf_group_sweep<T, true, true, COUNTU, false>(P, it.al, it.ar, it.bl, it.br, Mg, nullptr, nullptr,
                                                         pitch, R, P.dw + it.dw_start, it.dw_count, status,
                                                         abort_flag);
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------- backward

template <typename T>
__device__ __forceinline__ T ld_cg(const T *p) { return __ldcg(p); }

// Adjoint of one group's forward sweep, on Mg, Eg, Fg as the forward kept
// them or as pf_group_sweep<SAVE> recomputed them. Mb (same layout as Mg)
// accumulates dZ'/dM for every cell of the rectangle, boundaries included.
// Seeds: the group's own D
// entries (dZ'/dD(am) w(am) into M(ar-1,br-1)) or, for the top level,
// dZ'/dM(n,m) = 1. Propagates into D_bar of nested arc matches, the per-pair
// base-match accumulator and the gap counts. Rows bottom-up, chunks right to
// left; E_bar of the row below lives in the E ring, the row's X_bar in Ar.
// TRUNC: the base-match sums of compute_basematch_probabilities with a
// positive min_am_prob (aligner_p.icc:1201-1327): D_bar is final (from the
// full pass), only the group's arc matches with probability D D_bar / Z' >
// theta seed M_bar, and nothing propagates out of the group (no D_bar, no use
// counters, no gap counts); the per-band-cell sums go to bmacc. GRADS: the
// gap counts (ext_acc / open_acc) are accumulated, which reads E and F;
// without, only M of the recomputed rectangle is read.
template <typename T, bool TRUNC = false, bool GRADS = true>
__device__ void pf_group_back(const PFPair<T> &P, int al, int ar, int bl, int br, bool top,
                              const T *__restrict__ Mg, const T *__restrict__ Eg, const T *__restrict__ Fg,
                              T *__restrict__ Mb, int pitch, PFRows<T> R, const int4 *__restrict__ dw, int ndw,
                              int *status, volatile int *abort_flag, double *ext_acc, double *open_acc,
                              double theta_z = 0.0) {
    const int lane = threadIdx.x & 31;
    const int m1 = P.m + 1;
    const T o = P.o, arcf = P.arcf;
    T *const Eb = R.E;
    T *const Xb = R.Ar;
    // diagonal adjoint contributions X_bar(i,j) bm(i,j) to M_bar(i-1,j-1):
    // row i writes them into one ring (each target column once), row i-1
    // reads them (and clears the entry) from it; the two rings alternate.
    // Targets outside row i-1's columns, and row al, take the global atomic.
    T *Dn = R.Mp, *Dc = R.Mc;
#define RG(j) ((j) - R.rb * (int)__umulhi((unsigned)(j), R.magic))
    const int rows = ar - al;
    // clear the adjoint rectangle (band cells and boundaries)
    for (int r = 0; r < rows; ++r) {
        const int i = al + r;
        const int4 ri = P.rowinfo[i];
        const int lo = max(bl, ri.x - 1), hi = min(br - 1, max(ri.y, (i + 1 < ar) ? P.rowinfo[i + 1].y : ri.y));
        for (int j = lo + lane; j <= hi; j += 32) Mb[(size_t)r * pitch + (j - bl)] = T(0);
        if (lane == 0) Mb[(size_t)r * pitch] = T(0);
    }
    for (int c = lane; c < R.rb; c += 32) {
        Eb[c] = T(0);
        Dn[c] = T(0);
        Dc[c] = T(0);
    }
    __syncwarp();
    if (top && lane == 0) Mb[(size_t)(P.n - al) * pitch + (P.m - bl)] = T(1);
    __syncwarp();
    double ext = 0.0, opn = 0.0;
    int dwp = ndw - 1;  // D entries by ar descending
    for (int i = ar - 1; i > al; --i) {
        const int4 ri = P.rowinfo[i];
        const int2 ra = P.rowarc[i];
        const int minc = ri.x;
        const int lo = max(bl + 1, minc), hi = min(br - 1, ri.y);
        const T gAi = P.gA[i];
        const T gAn = (i + 1 < ar) ? P.gA[i + 1] : T(0);
        // seeds: dZ'/dD(am) w(am) into M(ar-1, br-1) once every use of D(am)
        // has been back-propagated
        while (dwp >= 0) {
            const int qq = dwp - lane;
            int4 e = make_int4(0, -1, 0, 0);
            if (qq >= 0) e = dw[qq];
            const bool mine = qq >= 0 && e.y == i;
            if (mine && TRUNC) {
                const double db = P.Dbar[e.x];
                if ((double)P.D[e.x] * db > theta_z)
                    atomicAdd(Mb + (size_t)(i - al) * pitch + (e.z - bl), (T)db * P.w[e.x]);
            } else if (mine) {
                long long spins = 0;
                while (*(const volatile int *)(P.cnt + e.x) > 0) {
                    __nanosleep(64);
                    if (++spins > PF_SPIN_LIMIT || *abort_flag) {
                        atomicOr(status, ST_TIMEOUT);
                        *abort_flag = 1;
                        break;
                    }
                }
                __threadfence();
                const T db = (T)ld_cg(P.Dbar + e.x);
                atomicAdd(Mb + (size_t)(i - al) * pitch + (e.z - bl), db * P.w[e.x]);
            }
            const int cnt = __popc(__ballot_sync(0xffffffffu, mine));
            dwp -= cnt;
            if (cnt < 32) break;
        }
        __syncwarp();
        const T *bmrow = P.bm + (size_t)i * m1;
        const size_t roff = (size_t)(i - al) * pitch;
        const int cb = ri.w - minc;
        // columns of row i-1 whose diagonal contributions go through the ring
        const int4 rup = P.rowinfo[i - 1];
        const int dlo = i - 1 > al ? max(bl + 1, rup.x) : INT_MAX;
        const int dhi = min(br - 1, rup.y);
        // chunks right to left
        const int nchunks = hi >= lo ? (hi - lo) / 32 + 1 : 0;
        T Fbc = T(0);  // F_bar(i, base+32) carried from the chunk to the right
        for (int k = nchunks - 1; k >= 0; --k) {
            const int base = lo + 32 * k;
            const int j = base + lane;
            const bool act = j <= hi;
            const int c = j - bl;
            // every load of the chunk first (none depends on the scan); left
            // neighbours and gB(j+1) come from the adjacent lanes
            T Mbar = T(0), Ebn = T(0), g = T(0), Ev = T(0), Fv = T(0), Mv = T(0), Mup = T(0), Eup = T(0),
              bmj = T(0);
            if (act) {
                Mbar = ld_cg(Mb + roff + c) + Dc[RG(j)];
                Dc[RG(j)] = T(0);
                Ebn = Eb[RG(j)];  // E_bar(i+1, j)
                g = P.gB[j];
                if (GRADS) {
                    Ev = Eg[roff + c];
                    Fv = Fg[roff + c];
                    Mv = Mg[roff + c];
                    Eup = Eg[roff - pitch + c];
                }
                Mup = Mg[roff - pitch + c];
                bmj = bmrow[j];
            }
            T gn = __shfl_down_sync(0xffffffffu, g, 1);  // gB(j+1); 0 past the row's end
            T Ml = __shfl_up_sync(0xffffffffu, Mv, 1), Fl = __shfl_up_sync(0xffffffffu, Fv, 1);
            T Md = __shfl_up_sync(0xffffffffu, Mup, 1);
            if (lane == 31 && act) gn = (j + 1 <= hi) ? P.gB[j + 1] : T(0);
            if (lane == 0 && act) {
                if (GRADS) {
                    Ml = Mg[roff + c - 1];
                    Fl = Fg[roff + c - 1];
                }
                Md = Mg[roff - pitch + c - 1];
            }
            const T Nbar = act ? Ebn * gAn * o : T(0);  // N(i,j) feeds E(i+1,j)
            // F_bar(j) = gB(j+1) F_bar(j+1) + (M_bar + N_bar)(j), right to left
            T a = T(1), b = T(0);
            if (act) {
                a = gn;
                b = Mbar + Nbar;
            }
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const T a2 = __shfl_down_sync(0xffffffffu, a, off);
                const T b2 = __shfl_down_sync(0xffffffffu, b, off);
                if (lane + off < 32) {
                    b = a * b2 + b;
                    a = a * a2;
                }
            }
            const T Fb = a * Fbc + b;
            T Fbr = __shfl_down_sync(0xffffffffu, Fb, 1);  // F_bar(i, j+1)
            if (lane == 31) Fbr = Fbc;
            if (act) {
                const T Qbar = Fbr * gn * o;
                const T Ebar = Mbar + Qbar + Ebn * gAn;
                const T Xbar = Mbar + Nbar + Qbar;
                Eb[RG(j)] = Ebar;
                Xb[RG(j)] = Xbar;
                // gap derivatives: E(i,j) = gA(i) (E(i-1,j) + N(i-1,j) o)
                if (GRADS) {
                    ext += (double)(Ebar * Ev + Fb * Fv);
                    opn += (double)(Ebar * (Mup - Eup) * gAi * o + Fb * (Ml - Fl) * g * o);
                }
                // diagonal
                if (j - 1 >= dlo && j - 1 <= dhi)
                    Dn[RG(j - 1)] = Xbar * bmj;
                else
                    atomicAdd(Mb + roff - pitch + c - 1, Xbar * bmj);
                atomicAdd(P.bmacc + cb + j, (double)(Xbar * Md * bmj));
                // E(i,j) reads N(i-1,j) = M(i-1,j) - E(i-1,j); F(i,j) reads Q(i,j-1)
                if (i - 1 == al || rup.x > j || rup.y < j)
                    atomicAdd(Mb + roff - pitch + c, Ebar * gAi * o);
                if (j == lo) atomicAdd(Mb + roff + c - 1, Fb * g * o);
            }
            Fbc = __shfl_sync(0xffffffffu, Fb, 0);
        }
        __syncwarp();
        // arc terms of row i: M_bar(corner) += X_bar D s', D_bar(am) += X_bar M(corner) s'
        // (two batches of 32 entries per step, loads issued together). The
        // use counters of the row's entries drop after one fence per row:
        // bit 2k+u of `pend` stands for entry ebase + 64k + 32u + lane.
        unsigned long long pend = 0;
        int ebase = ra.x, kb = 0;
        auto drop_uses = [&]() {
            if (pend) {
                __threadfence();  // the D_bar updates are visible before the counters drop
                do {
                    const int b = __ffsll((long long)pend) - 1;
                    pend &= pend - 1;
                    atomicSub(P.cnt + ebase + 64 * (b >> 1) + 32 * (b & 1) + lane, 1);
                } while (pend);
            }
        };
        for (int e0 = ra.x; e0 < ra.y; e0 += 64, ++kb) {
            if (kb == 32) {
                drop_uses();
                ebase = e0;
                kb = 0;
            }
            int2 en[2];
            bool okA[2];
            unsigned ball[2];
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int e = e0 + 32 * u + lane;
                en[u] = e < ra.y ? P.crow[e] : make_int2(0xffff, 0);
                const int ca = en[u].x & 0xffff;
                okA[u] = ca >= al && ca != 0xffff;
                ball[u] = __ballot_sync(0xffffffffu, okA[u]);
            }
            if (ball[0] == 0u) break;
            bool ok[2];
            T dv[2], mv[2], xb[2];
            size_t co[2];
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int ca = en[u].x & 0xffff, cbl = en[u].x >> 16;
                ok[u] = okA[u] && cbl >= bl && en[u].y >= lo && en[u].y <= hi;
                const int e = e0 + 32 * u + lane;
                co[u] = ok[u] ? (size_t)(ca - al) * pitch + (cbl - bl) : 0;
                xb[u] = ok[u] ? Xb[RG(en[u].y)] : T(0);
                dv[u] = ok[u] ? P.D[e] : T(0);
                mv[u] = ok[u] ? Mg[co[u]] : T(0);
            }
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                if (ok[u]) {
                    atomicAdd(Mb + co[u], xb[u] * dv[u] * arcf);
                    if (!TRUNC) atomicAdd(P.Dbar + e0 + 32 * u + lane, (double)(xb[u] * mv[u] * arcf));
                }
            }
#pragma unroll
            for (int u = 0; u < 2; ++u)
                if (ok[u] && !TRUNC) pend |= 1ull << (2 * kb + u);
            if (ball[0] != 0xffffffffu || ball[1] != 0xffffffffu) break;
        }
        drop_uses();
        // E_bar of row i at columns row i-1 has but row i does not is zero
        if (i - 1 > al) {
            const int lp = max(bl + 1, P.rowinfo[i - 1].x);
            for (int j = lp + lane; j < lo; j += 32) Eb[RG(j)] = T(0);
        }
        __syncwarp();
        T *const dt = Dn;  // row i-1 reads what row i wrote
        Dn = Dc;
        Dc = dt;
        if (*abort_flag) return;
    }
    // boundary values: M(al,j) = (o/s) prod gB, M(i,bl) = (o/s) prod gA
    if (GRADS) {
        const int L0 = min(br, P.rowinfo[al].y + 1);
        for (int j = bl + 1 + lane; j < L0; j += 32) {
            const T v = ld_cg(Mb + (j - bl)) * Mg[j - bl];
            ext += (double)v * (j - bl);
            opn += (double)v;
        }
        for (int i = al + 1 + lane; i < ar; i += 32) {
            if (P.rowinfo[i].x > bl) continue;
            const T v = ld_cg(Mb + (size_t)(i - al) * pitch) * Mg[(size_t)(i - al) * pitch];
            ext += (double)v * (i - al);
            opn += (double)v;
        }
    }
#undef RG
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        ext += __shfl_xor_sync(0xffffffffu, ext, off);
        opn += __shfl_xor_sync(0xffffffffu, opn, off);
    }
    if (lane == 0 && !TRUNC && GRADS) {
        atomicAdd(ext_acc, ext);
        atomicAdd(open_acc, opn);
    }
}

template <typename T, bool TRUNC, bool GRADS>
__global__ void __launch_bounds__(PF_WARPS * 32, pf_min_blocks<T>())
    pf_back_kernel(const PFPair<T> *__restrict__ pairs, const int2 *__restrict__ queue, int nitems,
                   T *scratch, long long stride, int pitch, int rb,
                   unsigned int *qhead, int *status, int *abort_ptr, double theta) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    PFRows<T> R = pf_rows<T>(warp, rb);
    T *Mg = scratch + ((long long)blockIdx.x * PF_WARPS + warp) * stride * 4;
    T *Eg = Mg + stride, *Fg = Eg + stride, *Mb = Fg + stride;
    volatile int *abort_flag = abort_ptr;
    while (true) {
        int idx = 0;
        if (lane == 0) idx = (int)atomicAdd(qhead, 1u);
        idx = __shfl_sync(0xffffffffu, idx, 0);
        if (idx >= nitems || *abort_flag) break;
        // items in reverse: the consumers of a group's D entries come first
        const int2 qi = queue[nitems - 1 - idx];
        const PFPair<T> &P = pairs[qi.x];
        const GroupItem it = P.groups[qi.y];
        const int al = it.top ? 0 : it.al, ar = it.top ? P.n + 1 : it.ar;
        const int bl = it.top ? 0 : it.bl, br = it.top ? P.m + 1 : it.br;
        // TRUNC: theta Z' (scaled frame); a group none of whose arc matches
        // passes the threshold contributes nothing
        const double theta_z = TRUNC ? theta * exp(P.res[0]) : 0.0;
        if (TRUNC && !it.top) {
            bool any = false;
            for (int k = lane; k < it.dw_count && !any; k += 32) {
                const int pos = P.dw[it.dw_start + k].x;
                any = (double)P.D[pos] * P.Dbar[pos] > theta_z;
            }
            if (!__any_sync(0xffffffffu, any)) continue;
        }
        // the group's rectangles: kept by the forward pass, else recomputed
        // into the warp's slot (the adjoint rectangle Mb takes the same pitch)
        const T *Mw = Mg, *Ew = Eg, *Fw = Fg;
        int pw = pitch;
        if (!it.top && P.rect && it.rect_off >= 0 && (!GRADS || P.rect_states == 3)) {
            pw = br - bl;
            const size_t sz = (size_t)(ar - al) * pw;
            Mw = P.rect + (size_t)P.rect_states * it.rect_off;
            Ew = Mw + sz;
            Fw = Ew + sz;
        } else {
            pf_group_sweep<T, false, false, false, true, GRADS>(P, al, ar, bl, br, Mg, Eg, Fg, pitch, R, nullptr,
                                                                0, status, abort_flag);
        }
        __syncwarp();
        pf_group_back<T, TRUNC, GRADS>(P, al, ar, bl, br, it.top != 0, Mw, Ew, Fw, Mb, pw, R,
                                it.top ? nullptr : P.dw + it.dw_start, it.top ? 0 : it.dw_count, status, abort_flag,
                                P.res + 1, P.res + 2, theta_z);
        __syncwarp();
    }
}

// ---------------------------------------------------------------- launchers

template <typename T>
static size_t pf_smem(int rb) {
    return (size_t)PF_WARPS * PF_RING_ROWS * rb * sizeof(T);
}

template <typename T>
cudaError_t pf_launch_fwd(const void *pairs, const int2 *queue, int nitems, void *scratch,
                          long long stride, int pitch, int rb, unsigned int *qhead, int *status, int *abort_flag,
                          int blocks, bool count_uses, cudaStream_t st, int keep_states) {
    const size_t smem = pf_smem<T>(rb);
    cudaError_t e;
    if (count_uses && keep_states > 0) {
        auto k = keep_states == 3 ? pf_fwd_kernel<T, true, 3> : pf_fwd_kernel<T, true, 1>;
        e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k<<<blocks, PF_WARPS * 32, smem, st>>>((const PFPair<T> *)pairs, queue, nitems, (T *)scratch, stride, pitch,
                                               rb, qhead, status, abort_flag);
    } else if (count_uses) {
        e = cudaFuncSetAttribute(pf_fwd_kernel<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        pf_fwd_kernel<T, true><<<blocks, PF_WARPS * 32, smem, st>>>(
            (const PFPair<T> *)pairs, queue, nitems, (T *)scratch, stride, pitch, rb, qhead,
            status, abort_flag);
    } else {
        e = cudaFuncSetAttribute(pf_fwd_kernel<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        pf_fwd_kernel<T, false><<<blocks, PF_WARPS * 32, smem, st>>>(
            (const PFPair<T> *)pairs, queue, nitems, (T *)scratch, stride, pitch, rb, qhead,
            status, abort_flag);
    }
    return cudaGetLastError();
}

// Resident blocks per SM for a kernel that could hold `occ`: the cap from
// the environment variable `var` (tuning runs), else `occ`. A cap below occ
// also asks for a shared-memory carveout that fits only the capped blocks, so
// that the rest of the SM's unified memory serves as L1 cache.
template <typename K>
static cudaError_t pf_cap_blocks(K kernel, const char *var, size_t smem, int *blocks_per_sm) {
    const char *v = std::getenv(var);
    const int cap = v ? std::atoi(v) : 0;
    cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, -1);
    if (cap <= 0 || cap >= *blocks_per_sm) return cudaSuccess;
    *blocks_per_sm = cap;
    int dev = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    const size_t want = (size_t)cap * (smem + 1024);
    const int pct = (int)std::min<size_t>(100, (want * 100 + per_sm - 1) / (size_t)std::max(per_sm, 1));
    return cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, pct);
}

template <typename T>
cudaError_t pf_fwd_occupancy(int rb, int *blocks_per_sm) {
    const size_t smem = pf_smem<T>(rb);
    cudaError_t e = cudaFuncSetAttribute(pf_fwd_kernel<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, pf_fwd_kernel<T, true>, PF_WARPS * 32, smem);
    if (e != cudaSuccess) return e;
    return pf_cap_blocks(pf_fwd_kernel<T, true>, "LCG_PF_FWD_BPS", smem, blocks_per_sm);
}

template <typename T, bool TRUNC, bool GRADS>
static cudaError_t pf_launch_back_k(const void *pairs, const int2 *queue, int nitems, void *scratch, long long stride,
                                    int pitch, int rb, unsigned int *qhead, int *status, int *abort_flag, int blocks,
                                    cudaStream_t st, double theta) {
    const size_t smem = pf_smem<T>(rb);
    cudaError_t e = cudaFuncSetAttribute(pf_back_kernel<T, TRUNC, GRADS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    pf_back_kernel<T, TRUNC, GRADS><<<blocks, PF_WARPS * 32, smem, st>>>(
        (const PFPair<T> *)pairs, queue, nitems, (T *)scratch, stride, pitch, rb, qhead, status, abort_flag, theta);
    return cudaGetLastError();
}

template <typename T>
cudaError_t pf_launch_back(const void *pairs, const int2 *queue, int nitems, void *scratch,
                           long long stride, int pitch, int rb, unsigned int *qhead, int *status, int *abort_flag,
                           int blocks, cudaStream_t st, double theta, bool grads) {
    if (theta > 0.0)
        return pf_launch_back_k<T, true, false>(pairs, queue, nitems, scratch, stride, pitch, rb, qhead, status,
                                                abort_flag, blocks, st, theta);
    if (grads)
        return pf_launch_back_k<T, false, true>(pairs, queue, nitems, scratch, stride, pitch, rb, qhead, status,
                                                abort_flag, blocks, st, 0.0);
    return pf_launch_back_k<T, false, false>(pairs, queue, nitems, scratch, stride, pitch, rb, qhead, status,
                                             abort_flag, blocks, st, 0.0);
}

template <typename T>
cudaError_t pf_back_occupancy(int rb, int *blocks_per_sm) {
    const size_t smem = pf_smem<T>(rb);
    cudaError_t e = cudaFuncSetAttribute(pf_back_kernel<T, false, true>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, pf_back_kernel<T, false, true>, PF_WARPS * 32,
                                                      smem);
    if (e != cudaSuccess) return e;
    return pf_cap_blocks(pf_back_kernel<T, false, true>, "LCG_PF_BACK_BPS", smem, blocks_per_sm);
}

int pf_warps_per_block() { return PF_WARPS; }

template cudaError_t pf_launch_fwd<double>(const void *, const int2 *, int, void *, long long, int,
                                           int, unsigned int *, int *, int *, int, bool, cudaStream_t, int);
template cudaError_t pf_launch_fwd<float>(const void *, const int2 *, int, void *, long long, int,
                                          int, unsigned int *, int *, int *, int, bool, cudaStream_t, int);
template cudaError_t pf_fwd_occupancy<double>(int, int *);
template cudaError_t pf_fwd_occupancy<float>(int, int *);
template cudaError_t pf_launch_back<double>(const void *, const int2 *, int, void *, long long, int,
                                            int, unsigned int *, int *, int *, int, cudaStream_t, double, bool);
template cudaError_t pf_launch_back<float>(const void *, const int2 *, int, void *, long long, int,
                                           int, unsigned int *, int *, int *, int, cudaStream_t, double, bool);
template cudaError_t pf_back_occupancy<double>(int, int *);
template cudaError_t pf_back_occupancy<float>(int, int *);

}  // namespace lcg
