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
#include <stdint.h>

#include "lcg_device.cuh"
#include "pf_device.cuh"

namespace lcg {

constexpr int PF_WARPS = 4;
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

// Shared-memory rows per warp (T each): Mprev, Mcur, Nprev, Ncur, E, gB, and
// 32 slots for the arc terms of a chunk.
template <typename T>
struct PFRows {
    T *Mp, *Mc, *Np, *Nc, *E, *gB, *A;
};

template <typename T>
__device__ __forceinline__ PFRows<T> pf_rows(int warp, int sw) {
    T *base = reinterpret_cast<T *>(pf_smem_raw) + (size_t)warp * (6 * sw + 32);
    PFRows<T> r;
    r.Mp = base;
    r.Mc = base + sw;
    r.Np = base + 2 * sw;
    r.Nc = base + 3 * sw;
    r.E = base + 4 * sw;
    r.gB = base + 5 * sw;
    r.A = base + 6 * sw;
    return r;
}

// Forward sweep of one group (or the top level) in the scaled frame; M of the
// rectangle goes to Mg (row i-al, column j-bl, pitch `pitch`).
// COUNTU: count the uses of every D entry (for the backward pass).
template <typename T, bool WAIT, bool DWRITE, bool COUNTU>
__device__ void pf_group_fwd(const PFPair<T> &P, int al, int ar, int bl, int br, T *__restrict__ Mg,
                             int pitch, PFRows<T> R, const int4 *__restrict__ dw, int ndw, int *status,
                             volatile int *abort_flag) {
    const int lane = threadIdx.x & 31;
    const int m1 = P.m + 1;
    const T o = P.o, arcf = P.arcf;
    const int W = br - bl;
    for (int c = lane; c < W; c += 32) {
        R.E[c] = T(0);
        R.gB[c] = c > 0 ? P.gB[bl + c] : T(0);
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
                R.Mp[j - bl] = val;
                R.Np[j - bl] = val;
                Mg[j - bl] = val;
            }
            carry = __shfl_sync(0xffffffffu, val, 31);
        }
        if (lane == 0) {
            R.Mp[0] = P.inv_s;
            R.Np[0] = P.inv_s;
            Mg[0] = P.inv_s;
        }
        if (al + 1 < ar) {
            const int L1 = min(br, P.rowinfo[al + 1].y + 1);
            for (int j = L0 + lane; j < L1; j += 32) {
                R.Mp[j - bl] = T(0);
                R.Np[j - bl] = T(0);
            }
        }
    }
    __syncwarp();
    T colval = o * P.inv_s;
    int dwp = 0;
    for (int i = al + 1; i < ar; ++i) {
        const int4 ri = P.rowinfo[i];
        const int minc = ri.x;
        const int lo = max(bl + 1, minc), hi = min(br - 1, ri.y);
        const T gAi = P.gA[i];
        T B = T(0);
        if (minc <= bl) {
            colval *= gAi;
            B = colval;
            if (lane == 0) Mg[(size_t)(i - al) * pitch] = B;
        }
        if (lane == 0 && lo - 1 - bl < W) {
            R.Mc[lo - 1 - bl] = B;
            R.Nc[lo - 1 - bl] = B;
        }
        const T *bmrow = P.bm + (size_t)i * m1;
        T *Mrow = Mg + (size_t)(i - al) * pitch - bl;
        const int cb = ri.w - minc;
        T Fc = T(0), Qc = B;
        for (int base = lo; base <= hi; base += 32) {
            const int j = base + lane;
            const bool act = j <= hi;
            const int c = j - bl;
            T X = T(0), Ei = T(0);
            int q = 0, qe = 0;
            if (act) {
                Ei = R.E[c] * gAi + R.Np[c] * gAi * o;
                X = R.Mp[c - 1] * bmrow[j];
                q = P.cre_start[cb + j];
                qe = P.cre_start[cb + j + 1];
            }
            // arc-match terms, warp-cooperative over the chunk's candidates
            {
                const int last = min(base + 31, hi) - base;
                const int Qs = __shfl_sync(0xffffffffu, q, 0);
                const int Qe = __shfl_sync(0xffffffffu, qe, last);
                R.A[lane] = T(0);
                __syncwarp();
                for (int e = Qs + lane; e < Qe; e += 32) {
                    const int4 en = P.cre[e];
                    if (en.y >= al && en.z >= bl) {
                        T dv = pf_ld(P.D + en.x);
                        if (WAIT && pf_not_ready(dv)) dv = pf_wait(P.D + en.x, status, abort_flag);
                        const T mv = Mg[(size_t)(en.y - al) * pitch + (en.z - bl)];
                        atomicAdd(&R.A[en.w - base], mv * dv * arcf);
                        if (COUNTU) atomicAdd(P.cnt + en.x, 1);
                    }
                }
                __syncwarp();
                X += R.A[lane];
            }
            // F(j) = gB(j) F(j-1) + gB(j) o Q(j-1): linear warp scan
            const T Q = X + Ei;
            T Qp = __shfl_up_sync(0xffffffffu, Q, 1);
            if (lane == 0) Qp = Qc;
            T a = T(1), b = T(0);
            if (act) {
                const T g = R.gB[c];
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
                R.E[c] = Ei;
                R.Mc[c] = M;
                R.Nc[c] = X + F;
                Mrow[j] = M;
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
                    const T v = R.Mc[e.z - bl] * P.w[e.x];
                    *(volatile T *)(P.D + e.x) = v;
                }
                const int cnt = __popc(__ballot_sync(0xffffffffu, mine));
                dwp += cnt;
                if (cnt < 32) break;
            }
        }
        if (i + 1 < ar) {
            const int Ln = min(br, P.rowinfo[i + 1].y + 1);
            for (int j = max(hi + 1, bl + 1) + lane; j < Ln; j += 32) {
                R.Mc[j - bl] = T(0);
                R.Nc[j - bl] = T(0);
            }
        }
        __syncwarp();
        T *t;
        t = R.Mp; R.Mp = R.Mc; R.Mc = t;
        t = R.Np; R.Np = R.Nc; R.Nc = t;
        if (WAIT && *abort_flag) return;
    }
}

template <typename T, bool COUNTU>
__global__ void __launch_bounds__(PF_WARPS * 32)
    pf_fwd_kernel(const PFPair<T> *__restrict__ pairs, const PFItem<T> *__restrict__ items, int nitems,
                  const int4 *__restrict__ dw, T *scratch, long long stride, int sw, unsigned int *qhead,
                  int *status, int *abort_ptr) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    PFRows<T> R = pf_rows<T>(warp, sw);
    T *Mg = scratch + ((long long)blockIdx.x * PF_WARPS + warp) * stride;
    volatile int *abort_flag = abort_ptr;
    while (true) {
        int idx = 0;
        if (lane == 0) idx = (int)atomicAdd(qhead, 1u);
        idx = __shfl_sync(0xffffffffu, idx, 0);
        if (idx >= nitems || *abort_flag) break;
        const PFItem<T> it = items[idx];
        const PFPair<T> &P = pairs[it.pair];
        if (it.top) {
            pf_group_fwd<T, true, false, COUNTU>(P, 0, P.n + 1, 0, P.m + 1, P.topM, P.m + 1, R, nullptr, 0,
                                                 status, abort_flag);
            __syncwarp();
            if (lane == 0) {
                const T z = P.topM[(size_t)P.n * (P.m + 1) + P.m];
                P.res[0] = log((double)z);
            }
        } else {
            pf_group_fwd<T, true, true, COUNTU>(P, it.al, it.ar, it.bl, it.br, Mg, sw, R, dw + it.dw_start,
                                                it.dw_count, status, abort_flag);
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------- backward

// Forward recomputation for the backward pass: like pf_group_fwd (D entries
// are final) but it also keeps E and F of every cell (Eg, Fg, same layout as
// Mg), which the gap-count derivatives need.
template <typename T>
__device__ void pf_group_recompute(const PFPair<T> &P, int al, int ar, int bl, int br, T *__restrict__ Mg,
                                   T *__restrict__ Eg, T *__restrict__ Fg, int pitch, PFRows<T> R) {
    const int lane = threadIdx.x & 31;
    const int m1 = P.m + 1;
    const T o = P.o, arcf = P.arcf;
    const int W = br - bl;
    for (int c = lane; c < W; c += 32) {
        R.E[c] = T(0);
        R.gB[c] = c > 0 ? P.gB[bl + c] : T(0);
    }
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
                R.Mp[j - bl] = val;
                R.Np[j - bl] = val;
                Mg[j - bl] = val;
                Eg[j - bl] = T(0);
                Fg[j - bl] = T(0);
            }
            carry = __shfl_sync(0xffffffffu, val, 31);
        }
        if (lane == 0) {
            R.Mp[0] = P.inv_s;
            R.Np[0] = P.inv_s;
            Mg[0] = P.inv_s;
            Eg[0] = T(0);
            Fg[0] = T(0);
        }
        if (al + 1 < ar) {
            const int L1 = min(br, P.rowinfo[al + 1].y + 1);
            for (int j = L0 + lane; j < L1; j += 32) {
                R.Mp[j - bl] = T(0);
                R.Np[j - bl] = T(0);
                Mg[j - bl] = T(0);
                Eg[j - bl] = T(0);
                Fg[j - bl] = T(0);
            }
        }
    }
    __syncwarp();
    T colval = o * P.inv_s;
    for (int i = al + 1; i < ar; ++i) {
        const int4 ri = P.rowinfo[i];
        const int minc = ri.x;
        const int lo = max(bl + 1, minc), hi = min(br - 1, ri.y);
        const T gAi = P.gA[i];
        T B = T(0);
        if (minc <= bl) {
            colval *= gAi;
            B = colval;
            if (lane == 0) {
                Mg[(size_t)(i - al) * pitch] = B;
                Eg[(size_t)(i - al) * pitch] = T(0);
                Fg[(size_t)(i - al) * pitch] = T(0);
            }
        }
        if (lane == 0 && lo - 1 - bl < W) {
            R.Mc[lo - 1 - bl] = B;
            R.Nc[lo - 1 - bl] = B;
            // the cell left of the row's band (column bl, or a zero cell)
            Mg[(size_t)(i - al) * pitch + (lo - 1 - bl)] = B;
            Eg[(size_t)(i - al) * pitch + (lo - 1 - bl)] = T(0);
            Fg[(size_t)(i - al) * pitch + (lo - 1 - bl)] = T(0);
        }
        const T *bmrow = P.bm + (size_t)i * m1;
        const size_t roff = (size_t)(i - al) * pitch - bl;
        const int cb = ri.w - minc;
        T Fc = T(0), Qc = B;
        for (int base = lo; base <= hi; base += 32) {
            const int j = base + lane;
            const bool act = j <= hi;
            const int c = j - bl;
            T X = T(0), Ei = T(0);
            int q = 0, qe = 0;
            if (act) {
                Ei = R.E[c] * gAi + R.Np[c] * gAi * o;
                X = R.Mp[c - 1] * bmrow[j];
                q = P.cre_start[cb + j];
                qe = P.cre_start[cb + j + 1];
            }
            {
                const int last = min(base + 31, hi) - base;
                const int Qs = __shfl_sync(0xffffffffu, q, 0);
                const int Qe = __shfl_sync(0xffffffffu, qe, last);
                R.A[lane] = T(0);
                __syncwarp();
                for (int e = Qs + lane; e < Qe; e += 32) {
                    const int4 en = P.cre[e];
                    if (en.y >= al && en.z >= bl) {
                        const T mv = Mg[(size_t)(en.y - al) * pitch + (en.z - bl)];
                        atomicAdd(&R.A[en.w - base], mv * P.D[en.x] * arcf);
                    }
                }
                __syncwarp();
                X += R.A[lane];
            }
            const T Q = X + Ei;
            T Qp = __shfl_up_sync(0xffffffffu, Q, 1);
            if (lane == 0) Qp = Qc;
            T a = T(1), b = T(0);
            if (act) {
                const T g = R.gB[c];
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
                R.E[c] = Ei;
                R.Mc[c] = M;
                R.Nc[c] = X + F;
                Mg[roff + j] = M;
                Eg[roff + j] = Ei;
                Fg[roff + j] = F;
            }
            Fc = __shfl_sync(0xffffffffu, F, 31);
            Qc = __shfl_sync(0xffffffffu, Q, 31);
        }
        __syncwarp();
        if (i + 1 < ar) {
            const int Ln = min(br, P.rowinfo[i + 1].y + 1);
            for (int j = max(hi + 1, bl + 1) + lane; j < Ln; j += 32) {
                R.Mc[j - bl] = T(0);
                R.Nc[j - bl] = T(0);
                Mg[(size_t)(i - al) * pitch + (j - bl)] = T(0);
                Eg[(size_t)(i - al) * pitch + (j - bl)] = T(0);
                Fg[(size_t)(i - al) * pitch + (j - bl)] = T(0);
            }
        }
        __syncwarp();
        T *t;
        t = R.Mp; R.Mp = R.Mc; R.Mc = t;
        t = R.Np; R.Np = R.Nc; R.Nc = t;
    }
}

template <typename T>
__device__ __forceinline__ T ld_cg(const T *p) { return __ldcg(p); }

// Adjoint of one group's forward sweep. Mb (same layout as Mg) accumulates
// dZ'/dM for every cell of the rectangle, boundaries included. Seeds: the
// group's own D entries (dZ'/dD(am) w(am) into M(ar-1,br-1)) or, for the top
// level, dZ'/dM(n,m) = 1. Propagates into D_bar of nested arc matches, the
// per-pair base-match accumulator and the gap counts.
template <typename T>
__device__ void pf_group_back(const PFPair<T> &P, int al, int ar, int bl, int br, bool top,
                              const T *__restrict__ Mg, const T *__restrict__ Eg, const T *__restrict__ Fg,
                              T *__restrict__ Mb, int pitch, T *Eb, T *gBs, T *A, const int4 *__restrict__ dw,
                              int ndw, int *status, volatile int *abort_flag, double *ext_acc, double *open_acc) {
    const int lane = threadIdx.x & 31;
    const int m1 = P.m + 1;
    const T o = P.o, arcf = P.arcf;
    const int W = br - bl;
    const int rows = ar - al;
    // clear the adjoint rectangle (band cells and boundaries)
    for (int r = 0; r < rows; ++r) {
        const int i = al + r;
        const int4 ri = P.rowinfo[i];
        const int lo = max(bl, ri.x - 1), hi = min(br - 1, max(ri.y, (i + 1 < ar) ? P.rowinfo[i + 1].y : ri.y));
        for (int j = lo + lane; j <= hi; j += 32) Mb[(size_t)r * pitch + (j - bl)] = T(0);
        if (lane == 0) Mb[(size_t)r * pitch] = T(0);
    }
    for (int c = lane; c < W; c += 32) {
        Eb[c] = T(0);
        gBs[c] = c > 0 ? P.gB[bl + c] : T(0);
    }
    __syncwarp();
    if (top && lane == 0) Mb[(size_t)(P.n - al) * pitch + (P.m - bl)] = T(1);
    __syncwarp();
    double ext = 0.0, opn = 0.0;
    int dwp = ndw - 1;  // D entries by ar descending
    for (int i = ar - 1; i > al; --i) {
        const int4 ri = P.rowinfo[i];
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
            if (mine) {
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
                const T db = ld_cg(P.Dbar + e.x);
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
        // chunks right to left
        const int nchunks = hi >= lo ? (hi - lo) / 32 + 1 : 0;
        T Fbc = T(0);  // F_bar(i, base+32) carried from the chunk to the right
        for (int k = nchunks - 1; k >= 0; --k) {
            const int base = lo + 32 * k;
            const int j = base + lane;
            const bool act = j <= hi;
            const int c = j - bl;
            T Mbar = T(0), Nbar = T(0), Ebn = T(0);
            if (act) {
                Mbar = ld_cg(Mb + roff + c);
                Ebn = Eb[c];                 // E_bar(i+1, j)
                Nbar = Ebn * gAn * o;        // N(i,j) feeds E(i+1,j)
            }
            // F_bar(j) = gB(j+1) F_bar(j+1) + (M_bar + N_bar)(j), right to left
            T a = T(1), b = T(0);
            if (act) {
                a = (j + 1 <= hi) ? gBs[c + 1] : T(0);
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
            T Qbar = T(0), Ebar = T(0), Xbar = T(0);
            if (act) {
                Qbar = (j + 1 <= hi) ? Fbr * gBs[c + 1] * o : T(0);
                Ebar = Mbar + Qbar + Ebn * gAn;
                Xbar = Mbar + Nbar + Qbar;
                Eb[c] = Ebar;
                // gap derivatives: E(i,j) = gA(i) (E(i-1,j) + N(i-1,j) o)
                const T Ev = Eg[roff + (c)], Fv = Fg[roff + (c)];
                ext += (double)(Ebar * Ev + Fb * Fv);
                const T Mup = Mg[roff - pitch + c], Eup = Eg[roff - pitch + c];
                const T Ml = Mg[roff + c - 1], Fl = Fg[roff + c - 1];
                opn += (double)(Ebar * (Mup - Eup) * gAi * o + Fb * (Ml - Fl) * gBs[c] * o);
                // diagonal
                const T Md = Mg[roff - pitch + c - 1];
                atomicAdd(Mb + roff - pitch + c - 1, Xbar * bmrow[j]);
                atomicAdd(P.bmacc + cb + j, Xbar * Md * bmrow[j]);
                // E(i,j) reads N(i-1,j) = M(i-1,j) - E(i-1,j); F(i,j) reads Q(i,j-1)
                if (i - 1 == al || P.rowinfo[i - 1].x > j || P.rowinfo[i - 1].y < j)
                    atomicAdd(Mb + roff - pitch + c, Ebar * gAi * o);
                if (j == lo) atomicAdd(Mb + roff + c - 1, Fb * gBs[c] * o);
            }
            // arc terms: M_bar(corner) += X_bar D s', D_bar(am) += X_bar M(corner) s'
            int q = 0, qe = 0;
            if (act) {
                q = P.cre_start[cb + j];
                qe = P.cre_start[cb + j + 1];
            }
            const int last = min(base + 31, hi) - base;
            const int Qs = __shfl_sync(0xffffffffu, q, 0);
            const int Qe = __shfl_sync(0xffffffffu, qe, last);
            A[lane] = Xbar;
            __syncwarp();
            for (int e = Qs + lane; e < Qe; e += 32) {
                const int4 en = P.cre[e];
                if (en.y >= al && en.z >= bl) {
                    const T xb = A[en.w - base];
                    const size_t co = (size_t)(en.y - al) * pitch + (en.z - bl);
                    atomicAdd(Mb + co, xb * P.D[en.x] * arcf);
                    atomicAdd(P.Dbar + en.x, xb * Mg[co] * arcf);
                    __threadfence();
                    atomicSub(P.cnt + en.x, 1);
                }
            }
            __syncwarp();
            Fbc = __shfl_sync(0xffffffffu, Fb, 0);
        }
        __syncwarp();
        if (*abort_flag) return;
    }
    // boundary values: M(al,j) = (o/s) prod gB, M(i,bl) = (o/s) prod gA
    {
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
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        ext += __shfl_xor_sync(0xffffffffu, ext, off);
        opn += __shfl_xor_sync(0xffffffffu, opn, off);
    }
    if (lane == 0) {
        atomicAdd(ext_acc, ext);
        atomicAdd(open_acc, opn);
    }
}

template <typename T>
__global__ void __launch_bounds__(PF_WARPS * 32)
    pf_back_kernel(const PFPair<T> *__restrict__ pairs, const PFItem<T> *__restrict__ items, int nitems,
                   const int4 *__restrict__ dw, T *scratch, long long stride, int sw, unsigned int *qhead,
                   int *status, int *abort_ptr) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    PFRows<T> R = pf_rows<T>(warp, sw);
    T *Mg = scratch + ((long long)blockIdx.x * PF_WARPS + warp) * stride * 4;
    T *Eg = Mg + stride, *Fg = Eg + stride, *Mb = Fg + stride;
    volatile int *abort_flag = abort_ptr;
    while (true) {
        int idx = 0;
        if (lane == 0) idx = (int)atomicAdd(qhead, 1u);
        idx = __shfl_sync(0xffffffffu, idx, 0);
        if (idx >= nitems || *abort_flag) break;
        // items in reverse: the consumers of a group's D entries come first
        const PFItem<T> it = items[nitems - 1 - idx];
        const PFPair<T> &P = pairs[it.pair];
        const int al = it.top ? 0 : it.al, ar = it.top ? P.n + 1 : it.ar;
        const int bl = it.top ? 0 : it.bl, br = it.top ? P.m + 1 : it.br;
        const int pitch = sw;
        pf_group_recompute<T>(P, al, ar, bl, br, Mg, Eg, Fg, pitch, R);
        __syncwarp();
        pf_group_back<T>(P, al, ar, bl, br, it.top != 0, Mg, Eg, Fg, Mb, pitch, R.Np, R.gB, R.A,
                         it.top ? nullptr : dw + it.dw_start, it.top ? 0 : it.dw_count, status, abort_flag,
                         P.res + 1, P.res + 2);
        __syncwarp();
    }
}

// ---------------------------------------------------------------- launchers

template <typename T>
cudaError_t pf_launch_fwd(const void *pairs, const void *items, int nitems, const int4 *dw, void *scratch,
                          long long stride, int sw, unsigned int *qhead, int *status, int *abort_flag,
                          int blocks, bool count_uses, cudaStream_t st) {
    size_t smem = (size_t)PF_WARPS * (6 * sw + 32) * sizeof(T);
    cudaError_t e;
    if (count_uses) {
        e = cudaFuncSetAttribute(pf_fwd_kernel<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        pf_fwd_kernel<T, true><<<blocks, PF_WARPS * 32, smem, st>>>(
            (const PFPair<T> *)pairs, (const PFItem<T> *)items, nitems, dw, (T *)scratch, stride, sw, qhead,
            status, abort_flag);
    } else {
        e = cudaFuncSetAttribute(pf_fwd_kernel<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        pf_fwd_kernel<T, false><<<blocks, PF_WARPS * 32, smem, st>>>(
            (const PFPair<T> *)pairs, (const PFItem<T> *)items, nitems, dw, (T *)scratch, stride, sw, qhead,
            status, abort_flag);
    }
    return cudaGetLastError();
}

template <typename T>
cudaError_t pf_fwd_occupancy(int sw, int *blocks_per_sm) {
    size_t smem = (size_t)PF_WARPS * (6 * sw + 32) * sizeof(T);
    cudaError_t e = cudaFuncSetAttribute(pf_fwd_kernel<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, pf_fwd_kernel<T, true>, PF_WARPS * 32, smem);
}

template <typename T>
cudaError_t pf_launch_back(const void *pairs, const void *items, int nitems, const int4 *dw, void *scratch,
                           long long stride, int sw, unsigned int *qhead, int *status, int *abort_flag, int blocks,
                           cudaStream_t st) {
    size_t smem = (size_t)PF_WARPS * (6 * sw + 32) * sizeof(T);
    cudaError_t e = cudaFuncSetAttribute(pf_back_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    pf_back_kernel<T><<<blocks, PF_WARPS * 32, smem, st>>>((const PFPair<T> *)pairs, (const PFItem<T> *)items,
                                                             nitems, dw, (T *)scratch, stride, sw, qhead, status,
                                                             abort_flag);
    return cudaGetLastError();
}

template <typename T>
cudaError_t pf_back_occupancy(int sw, int *blocks_per_sm) {
    size_t smem = (size_t)PF_WARPS * (6 * sw + 32) * sizeof(T);
    cudaError_t e = cudaFuncSetAttribute(pf_back_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, pf_back_kernel<T>, PF_WARPS * 32, smem);
}

int pf_warps_per_block() { return PF_WARPS; }

template cudaError_t pf_launch_fwd<double>(const void *, const void *, int, const int4 *, void *, long long, int,
                                           unsigned int *, int *, int *, int, bool, cudaStream_t);
template cudaError_t pf_launch_fwd<float>(const void *, const void *, int, const int4 *, void *, long long, int,
                                          unsigned int *, int *, int *, int, bool, cudaStream_t);
template cudaError_t pf_fwd_occupancy<double>(int, int *);
template cudaError_t pf_fwd_occupancy<float>(int, int *);
template cudaError_t pf_launch_back<double>(const void *, const void *, int, const int4 *, void *, long long, int,
                                            unsigned int *, int *, int *, int, cudaStream_t);
template cudaError_t pf_launch_back<float>(const void *, const void *, int, const int4 *, void *, long long, int,
                                           unsigned int *, int *, int *, int, cudaStream_t);
template cudaError_t pf_back_occupancy<double>(int, int *);
template cudaError_t pf_back_occupancy<float>(int, int *);

}  // namespace lcg
