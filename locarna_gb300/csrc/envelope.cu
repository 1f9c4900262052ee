// Sequence envelope on the GPU: the trace-probability band of the reference's
// TraceController (trace_controller.cc:565-597) from the PFGotoh forward and
// reverse partition functions (edge_probs.icc:76-162) and the edge
// probabilities of PFTraceProbs (edge_probs.icc:212-268), for a batch of
// pairs, one warp per pair.
//
// The reference evaluates the recursions in long double (locarna) or double
// (locarna_p) without scaling. Here every matrix row is kept in FP64 scaled by
// a power of two (exact), with its exponent alongside, so no row overflows.
// Only the threshold decision p(i,j) >= min_prob leaves the kernel: cells whose
// probability lies within a relative margin of the threshold (far above the
// FP64 and the reference's own rounding) are reported, and the host recomputes
// such a pair in the reference's precision when one of them could move a row
// bound. Pairs whose unscaled values would leave the range of the reference's
// float type are reported likewise (the reference's result there depends on
// its overflow behaviour).
//
// Matrices are full rows (n+1) x (m+1) as in the reference: out-of-band cells
// hold the values the reference leaves there (zero, or the free-end-gap and
// boundary initialisations of row 0 and column 0).
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/locarna_gb300.h"
#include "engine_state.hh"
#include "envelope.hh"

namespace {

constexpr int ENV_WARPS = 4;  // warps (pairs) per block

struct EnvDev {
    int n, m;
    const signed char *ca, *cb;
    const double *sdA, *suA, *sdB, *suB;
    const int *minc, *maxc;
    int *newmin, *newmax, *flag;
    double *fz;   // forward rows: (n+1) x [zM | zA | zB] x (m+1)
    int *fexp;    // forward row exponents
    double *rz;   // reverse rows, two alternating: 2 x [zM | zA | zB] x (m+1)
};

struct EnvConst {
    double sw, itemp, go, ge, gopen1, min_prob, mu;
    double score[16];
    int local, fe, rfe, exp_limit;
};

// value = v * 2^e, v kept in [1, 2) (or 0)
struct XAcc {
    double v;
    int e;
};

__device__ __forceinline__ void xadd(XAcc &a, double v, int e) {
    if (v == 0.0) return;
    if (a.v == 0.0) {
        a.v = v;
        a.e = e;
    } else if (e > a.e) {
        a.v = ldexp(a.v, a.e - e) + v;
        a.e = e;
    } else {
        a.v += ldexp(v, e - a.e);
    }
    const int d = ilogb(a.v);
    a.v = ldexp(a.v, -d);
    a.e += d;
}

__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, off));
    return v;
}
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

// band of row i in direction REV (the reverse band is TraceRange::reverse,
// trace_controller.cc:319-338)
template <bool REV>
__device__ __forceinline__ int band_lo(const EnvDev &P, int i) {
    return REV ? P.m - P.maxc[P.n - i] : P.minc[i];
}
template <bool REV>
__device__ __forceinline__ int band_hi(const EnvDev &P, int i) {
    return REV ? P.m - P.minc[P.n - i] : P.maxc[i];
}

// Boltzmann weight of the StralScore match (stral_score.cc:29-60) at (i, j)
// of direction REV; the reverse object mirrors both sequences and swaps the
// up/down probabilities, which leaves sqrt(dA dB) + sqrt(uA uB) unchanged.
template <bool REV>
__device__ __forceinline__ double match_weight(const EnvDev &P, const EnvConst &C, int i, int j) {
    const int ia = REV ? P.n + 1 - i : i, jb = REV ? P.m + 1 - j : j;
    const int a = P.ca[ia], b = P.cb[jb];
    const double seq = (a >= 0 && b >= 0) ? C.score[a * 4 + b] : 0.0;
    const double s = C.sw * (P.sdA[ia] * P.sdB[jb] + P.suA[ia] * P.suB[jb]) + seq;
    return exp(s * C.itemp);
}

// Row 0 of direction REV (PFGotoh::pf_gotoh initialisation, edge_probs.icc:
// 89-117): zM(0,0) = 1 (global) / 0 (local); zB(0,j) = g_open g_ext^j along
// the band; +1 on zB(0,j) with free end gaps at the start of B.
template <bool REV>
__device__ void env_row0(const EnvDev &P, const EnvConst &C, double *row, int fe) {
    const int lane = threadIdx.x & 31;
    const int m1 = P.m + 1;
    const int lo0 = band_lo<REV>(P, 0), hi0 = band_hi<REV>(P, 0);
    const bool chain = lo0 <= 1;
    for (int j = lane; j <= P.m; j += 32) {
        double zb = 0.0;
        if (j >= 1) {
            if (chain && j <= hi0) zb = C.go * C.ge * pow(C.ge, (double)(j - 1));
            if (fe & LCG_FREE_LEFT_1) zb += 1.0;
        }
        row[j] = (j == 0 && lo0 == 0 && !C.local) ? 1.0 : 0.0;
        row[m1 + j] = 0.0;
        row[2 * m1 + j] = zb;
    }
}

// Row i >= 1 of direction REV from row i-1 (`prev`, scaled by 2^-eprev) into
// `cur` in the same scale (edge_probs.icc:118-161); returns the row maximum
// and, through zsum, the sum of zM over the row.
template <bool REV>
__device__ double env_row(const EnvDev &P, const EnvConst &C, int i, const double *prev, double *cur, int eprev,
                          int fe, double *zsum) {
    const int lane = threadIdx.x & 31;
    const int m1 = P.m + 1;
    const int lo = band_lo<REV>(P, i), hi = band_hi<REV>(P, i);
    const int j0 = max(lo, 1), j1 = min(hi, P.m);
    // column 0: zA(i,0) = g_open g_ext^i while the band holds column 0 (from
    // row 1 on), +1 with free end gaps at the start of A
    double col0 = 0.0;
    if (band_lo<REV>(P, 1) == 0 && lo == 0) col0 = C.go * C.ge * pow(C.ge, (double)(i - 1));
    if (fe & LCG_FREE_LEFT_2) col0 += 1.0;
    col0 = ldexp(col0, -eprev);
    const double locw = C.local ? ldexp(1.0, -eprev) : 0.0;
    const double gog = C.go * C.ge;
    double carryB = 0.0, carryMA = 0.0;  // zB(i, base-1) and zM + zA at (i, base-1)
    double rmax = 0.0, rsum = 0.0;
    for (int base = 0; base <= P.m; base += 32) {
        const int j = base + lane;
        const bool act = j <= P.m;
        const bool inb = act && j >= j0 && j <= j1;
        double zm = 0.0, za = (j == 0) ? col0 : 0.0;
        if (inb) {
            const double w = match_weight<REV>(P, C, i, j);
            const double pm1 = prev[j - 1] + prev[m1 + j - 1] + prev[2 * m1 + j - 1];
            zm = pm1 * w + w * locw;
            za = prev[m1 + j] * C.ge + prev[j] * gog + prev[2 * m1 + j] * gog;
        }
        // zB(j) = g_ext zB(j-1) + (zM + zA)(j-1) g_open g_ext inside the band,
        // 0 outside: a first-order linear recurrence, scanned over the lanes
        double ma = zm + za;
        double mal = __shfl_up_sync(0xffffffffu, ma, 1);
        if (lane == 0) mal = carryMA;
        double a = inb ? C.ge : 0.0;
        double b = inb ? mal * gog : 0.0;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const double a2 = __shfl_up_sync(0xffffffffu, a, off);
            const double b2 = __shfl_up_sync(0xffffffffu, b, off);
            if (lane >= off) {
                b = a * b2 + b;
                a = a * a2;
            }
        }
        const double zb = a * carryB + b;
        if (act) {
            cur[j] = zm;
            cur[m1 + j] = za;
            cur[2 * m1 + j] = zb;
            rmax = fmax(rmax, fmax(zm, fmax(za, zb)));
            rsum += zm;
        }
        carryB = __shfl_sync(0xffffffffu, zb, 31);
        carryMA = __shfl_sync(0xffffffffu, ma, 31);
    }
    *zsum = warp_sum(rsum);
    return warp_max(rmax);
}

// scale a row by 2^-d (exact)
__device__ void env_scale(double *row, int m1, int d) {
    if (d == 0) return;
    const int lane = threadIdx.x & 31;
    for (int k = lane; k < 3 * m1; k += 32) row[k] = ldexp(row[k], -d);
}

__device__ __forceinline__ int exp_of(double v) { return v > 0.0 ? ilogb(v) : 0; }

__global__ void __launch_bounds__(ENV_WARPS * 32) envelope_kernel(const EnvDev *__restrict__ pairs, int npairs,
                                                                    EnvConst C) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int q = blockIdx.x * ENV_WARPS + warp;
    if (q >= npairs) return;
    const EnvDev &P = pairs[q];
    const int n = P.n, m = P.m, m1 = m + 1;
    const size_t rowsz = 3 * (size_t)m1;
    int flag = 0;

    // ---- forward: every row kept
    env_row0<false>(P, C, P.fz, C.fe);
    if (lane == 0) P.fexp[0] = 0;
    __syncwarp();
    int e = 0;
    XAcc zloc{0.0, 0};
    if (C.local) {
        double s = 0.0;
        for (int j = lane; j <= m; j += 32) s += P.fz[j];
        xadd(zloc, warp_sum(s), 0);
    }
    for (int i = 1; i <= n; ++i) {
        double *cur = P.fz + (size_t)i * rowsz;
        double zs = 0.0;
        const double mx = env_row<false>(P, C, i, cur - rowsz, cur, e, C.fe, &zs);
        if (C.local) xadd(zloc, zs, e);
        __syncwarp();
        const int d = exp_of(mx);
        env_scale(cur, m1, d);
        e += d;
        if (e + 2 > C.exp_limit) flag = 2;
        if (lane == 0) P.fexp[i] = e;
        __syncwarp();
    }
    // total (edge_probs.icc:220-236)
    XAcc z{0.0, 0};
    if (C.local) {
        xadd(z, 1.0, 0);
        xadd(z, zloc.v, zloc.e);
    } else {
        const double *rn = P.fz + (size_t)n * rowsz;
        xadd(z, rn[m] + rn[m1 + m] + rn[2 * m1 + m], e);
        if (C.fe & LCG_FREE_LEFT_2)
            for (int i = 0; i <= n; ++i) xadd(z, P.fz[(size_t)i * rowsz + m1 + m], P.fexp[i]);
        if (C.fe & LCG_FREE_LEFT_1) {
            double s = 0.0;
            for (int j = lane; j <= m; j += 32) s += rn[2 * m1 + j];
            xadd(z, warp_sum(s), e);
        }
    }
    if (z.v == 0.0 || z.e + 2 > C.exp_limit || z.e < -C.exp_limit) flag = 2;
    const double zinv = z.v > 0.0 ? 1.0 / z.v : 0.0;

    // ---- reverse, combined row by row with the stored forward rows
    int er = 0;
    const double thr_hi = C.min_prob * (1.0 + C.mu), thr_lo = C.min_prob * (1.0 - C.mu);
    for (int r = 0; r <= n; ++r) {
        double *cur = P.rz + (size_t)(r & 1) * rowsz;
        if (r == 0) {
            env_row0<true>(P, C, cur, C.rfe);
        } else {
            double zs = 0.0;
            const double mx = env_row<true>(P, C, r, P.rz + (size_t)((r - 1) & 1) * rowsz, cur, er, C.rfe, &zs);
            __syncwarp();
            const int d = exp_of(mx);
            env_scale(cur, m1, d);
            er += d;
            if (er + 2 > C.exp_limit) flag = 2;
        }
        __syncwarp();
        // edge probabilities of forward row i = n - r (edge_probs.icc:238-262)
        // and the row's threshold (trace_controller.cc:568-579)
        const int i = n - r;
        const double *f = P.fz + (size_t)i * rowsz;
        const int ef = P.fexp[i];
        const double locs = C.local ? ldexp(1.0, -er) : 0.0;
        const int lo = P.minc[i], hi = P.maxc[i];
        int nmin = hi, nmax = lo, umin = INT_MAX, umax = INT_MIN;
        for (int j = max(lo, 0) + lane; j <= min(hi, m); j += 32) {
            const int jr = m - j;
            const double rM = cur[jr], rA = cur[m1 + jr], rB = cur[2 * m1 + jr];
            const double zij = f[j] * (rM + rA + rB + locs) + f[m1 + j] * (rM + rA / C.gopen1 + rB) +
                               f[2 * m1 + j] * (rM + rA + rB / C.gopen1);
            const double p = ldexp(zij * zinv, ef + er - z.e);
            if (p >= thr_hi) {
                nmin = min(nmin, j);
                nmax = max(nmax, j);
            } else if (p >= thr_lo) {
                umin = min(umin, j);
                umax = max(umax, j);
            }
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            nmin = min(nmin, __shfl_xor_sync(0xffffffffu, nmin, off));
            nmax = max(nmax, __shfl_xor_sync(0xffffffffu, nmax, off));
            umin = min(umin, __shfl_xor_sync(0xffffffffu, umin, off));
            umax = max(umax, __shfl_xor_sync(0xffffffffu, umax, off));
        }
        if (umin < nmin || umax > nmax) flag = flag ? flag : 1;
        if (lane == 0) {
            P.newmin[i] = nmin;
            P.newmax[i] = nmax;
        }
        __syncwarp();
    }
    if (lane == 0) *P.flag = flag;
}

size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

}  // namespace

namespace lcg_env {

void reset_transfer(lcg_engine eng) {
    eng->prep_h2d = 0;
    eng->prep_d2h = 0;
}

struct Pending {
    std::vector<std::pair<int, size_t>> outs;  // (pair, output offset in the pinned staging)
    PairOut *out = nullptr;
    const PairIn *in = nullptr;
    size_t out_begin = 0, out_end = 0;
    cudaEvent_t done = nullptr;
};

// One wave (pairs [q0, q1) whose rows fit the device budget) staged,
// enqueued and, with wait, finished; without wait the wave's outputs are
// described in *pend.
static lcg_status enqueue_wave(lcg_engine eng, const EnvConst &C, int q0, int q1, const PairIn *in, PairOut *out,
                               bool wait, Pending *pend, std::string &err);

static EnvConst make_const(const Params &Pm) {
    EnvConst C;
    C.sw = Pm.sw;
    C.itemp = 1.0 / Pm.temp;
    C.go = Pm.g_open;
    C.ge = Pm.g_ext;
    C.gopen1 = Pm.g_open;
    C.min_prob = Pm.min_prob;
    C.mu = 1e-7;  // relative margin around the threshold (FP64 rounding is below 1e-12 here)
    std::memcpy(C.score, Pm.score, sizeof C.score);
    C.local = Pm.local;
    C.fe = Pm.fe;
    int rfe = 0;  // FreeEndgaps::reverse (free_endgaps.hh:74-79)
    if (Pm.fe & LCG_FREE_LEFT_1) rfe |= LCG_FREE_RIGHT_1;
    if (Pm.fe & LCG_FREE_RIGHT_1) rfe |= LCG_FREE_LEFT_1;
    if (Pm.fe & LCG_FREE_LEFT_2) rfe |= LCG_FREE_RIGHT_2;
    if (Pm.fe & LCG_FREE_RIGHT_2) rfe |= LCG_FREE_LEFT_2;
    C.rfe = rfe;
    C.exp_limit = Pm.exp_limit;

    return C;
}

static size_t wave_end(const PairIn *in, int q0, int npairs) {
    // waves of pairs whose forward rows fit a device budget
    const size_t budget = (size_t)6 << 30;
    size_t fz_bytes = 0;
    int q1 = q0;
    for (; q1 < npairs; ++q1) {
        const size_t n1 = (size_t)in[q1].n + 1, m1 = (size_t)in[q1].m + 1;
        const size_t f = 8 * (3 * n1 * m1 + 6 * m1) + 4 * n1;
        if (q1 > q0 && fz_bytes + f > budget) break;
        fz_bytes += f;
    }
    return (size_t)q1;
}

lcg_status compute(lcg_engine eng, const Params &Pm, int npairs, const PairIn *in, PairOut *out, std::string &err) {
    if (npairs <= 0) return LCG_OK;
    cudaError_t ce = cudaSetDevice(eng->device);
    if (ce != cudaSuccess) {
        err = std::string("cudaSetDevice: ") + cudaGetErrorString(ce);
        return LCG_ERR_CUDA;
    }
    const EnvConst C = make_const(Pm);
    for (int q0 = 0; q0 < npairs;) {
        const int q1 = (int)wave_end(in, q0, npairs);
        lcg_status rc = enqueue_wave(eng, C, q0, q1, in, out, true, nullptr, err);
        if (rc != LCG_OK) return rc;
        q0 = q1;
    }
    return LCG_OK;
}

lcg_status compute_begin(lcg_engine eng, const Params &Pm, int npairs, const PairIn *in, PairOut *out,
                         Pending **pending, std::string &err) {
    *pending = nullptr;
    if (npairs <= 0) return LCG_OK;
    cudaError_t ce = cudaSetDevice(eng->device);
    if (ce != cudaSuccess) {
        err = std::string("cudaSetDevice: ") + cudaGetErrorString(ce);
        return LCG_ERR_CUDA;
    }
    // more than one wave: computed now (the pinned staging holds one wave)
    if ((int)wave_end(in, 0, npairs) < npairs) return compute(eng, Pm, npairs, in, out, err);
    auto *p = new Pending;
    lcg_status rc = enqueue_wave(eng, make_const(Pm), 0, npairs, in, out, false, p, err);
    if (rc != LCG_OK) {
        if (p->done) cudaEventDestroy(p->done);
        delete p;
        return rc;
    }
    *pending = p;
    return LCG_OK;
}

lcg_status compute_end(lcg_engine eng, Pending *p, std::string &err) {
    if (!p) return LCG_OK;
    const cudaError_t ce = cudaEventSynchronize(p->done);
    cudaEventDestroy(p->done);
    if (ce != cudaSuccess) {
        err = std::string("envelope kernel: ") + cudaGetErrorString(ce);
        delete p;
        return LCG_ERR_CUDA;
    }
    const char *H = eng->env_host;
    eng->prep_h2d += (long long)p->out_begin;
    eng->prep_d2h += (long long)(p->out_end - p->out_begin);
    for (auto &x : p->outs) {
        const int n1 = p->in[x.first].n + 1;
        const int *o = (const int *)(H + x.second);
        std::memcpy(p->out[x.first].newmin, o, 4ull * n1);
        std::memcpy(p->out[x.first].newmax, o + n1, 4ull * n1);
        p->out[x.first].flag = o[2 * n1];
    }
    delete p;
    return LCG_OK;
}

static lcg_status enqueue_wave(lcg_engine eng, const EnvConst &C, int q0, int q1, const PairIn *in, PairOut *out,
                               bool wait, Pending *pend, std::string &err) {
    cudaError_t ce;
    std::vector<size_t> in_off, out_off, dev_off;
    auto take = [](size_t &cur, size_t b) {
        size_t o = cur;
        cur = align16(cur + b);
        return o;
    };
    const int nq = q1 - q0;
    // host staging: [EnvDev x nq][per pair inputs][per pair outputs]
    size_t hs = 0;
    const size_t o_pairs = take(hs, sizeof(EnvDev) * nq);
    in_off.resize(nq);
    for (int k = 0; k < nq; ++k) {
        const PairIn &p = in[q0 + k];
        const size_t n1 = (size_t)p.n + 1, m1 = (size_t)p.m + 1;
        in_off[k] = take(hs, 4 * (2 * n1) + 8 * (2 * n1 + 2 * m1) + n1 + m1);
    }
    const size_t out_begin = hs;
    out_off.resize(nq);
    for (int k = 0; k < nq; ++k) out_off[k] = take(hs, 4 * (2 * ((size_t)in[q0 + k].n + 1) + 1));
    const size_t out_end = hs;
    size_t ds = hs;  // device-only section after the mirrored staging
    dev_off.resize(nq);
    for (int k = 0; k < nq; ++k) {
        const size_t n1 = (size_t)in[q0 + k].n + 1, m1 = (size_t)in[q0 + k].m + 1;
        dev_off[k] = take(ds, 8 * (3 * n1 * m1 + 6 * m1) + 4 * n1);
    }
    // the buffers are reused only after the previous computation ended
    // (compute waits; a pending one is ended before the next begins)
    if (ds > eng->env_dev_cap) {
        if (eng->env_dev) cudaFree(eng->env_dev);
        eng->env_dev = nullptr;
        eng->env_dev_cap = 0;
        if (cudaMalloc(&eng->env_dev, ds + ds / 4) != cudaSuccess) {
            err = "envelope device allocation failed";
            return LCG_ERR_NOMEM;
        }
        eng->env_dev_cap = ds + ds / 4;
    }
    if (out_end > eng->env_host_cap) {
        if (eng->env_host) cudaFreeHost(eng->env_host);
        eng->env_host = nullptr;
        eng->env_host_cap = 0;
        if (cudaMallocHost(&eng->env_host, out_end + out_end / 4) != cudaSuccess) {
            err = "envelope pinned allocation failed";
            return LCG_ERR_NOMEM;
        }
        eng->env_host_cap = out_end + out_end / 4;
    }
    char *H = eng->env_host, *D = eng->env_dev;
    EnvDev *hp = (EnvDev *)(H + o_pairs);
    for (int k = 0; k < nq; ++k) {
        const PairIn &p = in[q0 + k];
        const int n1 = p.n + 1, m1 = p.m + 1;
        char *h = H + in_off[k];
        char *d = D + in_off[k];
        int *minc = (int *)h, *maxc = minc + n1;
        std::memcpy(minc, p.minc, 4ull * n1);
        std::memcpy(maxc, p.maxc, 4ull * n1);
        double *sdA = (double *)(h + 8ull * n1), *suA = sdA + n1, *sdB = suA + n1, *suB = sdB + m1;
        std::memcpy(sdA, p.sdA, 8ull * n1);
        std::memcpy(suA, p.suA, 8ull * n1);
        std::memcpy(sdB, p.sdB, 8ull * m1);
        std::memcpy(suB, p.suB, 8ull * m1);
        signed char *ca = (signed char *)(suB + m1), *cb = ca + n1;
        std::memcpy(ca, p.ca, n1);
        std::memcpy(cb, p.cb, m1);
        EnvDev &v = hp[k];
        v.n = p.n;
        v.m = p.m;
        v.minc = (const int *)d;
        v.maxc = (const int *)d + n1;
        v.sdA = (const double *)(d + 8ull * n1);
        v.suA = v.sdA + n1;
        v.sdB = v.suA + n1;
        v.suB = v.sdB + m1;
        v.ca = (const signed char *)(v.suB + m1);
        v.cb = v.ca + n1;
        char *od = D + out_off[k];
        v.newmin = (int *)od;
        v.newmax = (int *)od + n1;
        v.flag = (int *)od + 2 * n1;
        char *dd = D + dev_off[k];
        v.fz = (double *)dd;
        v.rz = v.fz + 3ull * n1 * m1;
        v.fexp = (int *)(v.rz + 6ull * m1);
    }
    cudaStream_t st = eng->stream;
    auto fail_cuda = [&](cudaError_t x, const char *what) {
        err = std::string(what) + ": " + cudaGetErrorString(x);
        cudaStreamSynchronize(st);
        return LCG_ERR_CUDA;
    };
    if ((ce = cudaMemcpyAsync(D, H, out_begin, cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return fail_cuda(ce, "envelope upload");
    const int blocks = (nq + ENV_WARPS - 1) / ENV_WARPS;
    envelope_kernel<<<blocks, ENV_WARPS * 32, 0, st>>>((const EnvDev *)(D + o_pairs), nq, C);
    if ((ce = cudaGetLastError()) != cudaSuccess) return fail_cuda(ce, "envelope launch");
    if ((ce = cudaMemcpyAsync(H + out_begin, D + out_begin, out_end - out_begin, cudaMemcpyDeviceToHost, st)) !=
        cudaSuccess)
        return fail_cuda(ce, "envelope download");
    if (!wait) {
        // finished by compute_end: an event after the download
        if ((ce = cudaEventCreateWithFlags(&pend->done, cudaEventDisableTiming)) != cudaSuccess)
            return fail_cuda(ce, "envelope event");
        if ((ce = cudaEventRecord(pend->done, st)) != cudaSuccess) return fail_cuda(ce, "envelope event");
        pend->in = in;
        pend->out = out;
        pend->out_begin = out_begin;
        pend->out_end = out_end;
        for (int k = 0; k < nq; ++k) pend->outs.emplace_back(q0 + k, out_off[k]);
        return LCG_OK;
    }
    if ((ce = cudaStreamSynchronize(st)) != cudaSuccess) return fail_cuda(ce, "envelope kernel");
    eng->prep_h2d += (long long)out_begin;
    eng->prep_d2h += (long long)(out_end - out_begin);
    for (int k = 0; k < nq; ++k) {
        const int n1 = in[q0 + k].n + 1;
        const int *o = (const int *)(H + out_off[k]);
        std::memcpy(out[q0 + k].newmin, o, 4ull * n1);
        std::memcpy(out[q0 + k].newmax, o + n1, 4ull * n1);
        out[q0 + k].flag = o[2 * n1];
    }
    return LCG_OK;
}

}  // namespace lcg_env
