// Host side of the LocARNA-P engine: the forward (log Z) / backward
// (probabilities and weight derivatives) C-ABI pair of include/locarna_gb300.h.
//
// The forward keeps its device state in the engine so that the backward pass
// can run on it: D entries, the per-arc-match use counters, and the
// accumulators of the adjoint.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <limits>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/locarna_gb300.h"
#include "engine_prep.hh"
#include "engine_state.hh"
#include "lcg_device.cuh"
#include "pf_device.cuh"


using namespace lcg;

namespace {

lcg_status pf_fail(lcg_status c, const std::string &m) {
    lcg_host::set_error(m);
    return c;
}

#define PF_TRY(call)                                                                          \
    do {                                                                                      \
        cudaError_t _e = (call);                                                              \
        if (_e != cudaSuccess) return pf_fail(LCG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e)); \
    } while (0)

size_t up16(size_t x) { return (x + 15) / 16 * 16; }

struct PFLayout {
    int n, m, na, npos, bandcells;  // npos: D entries (arc matches with a band cell as right ends)
    size_t rowinfo, crow, rowarc, groups, dw, bm, gA, gB, w, D, Dbar, cnt, bmacc, res, topM, rect;
    double log_c_total;  // (n+m) log c
};

struct PFState {
    int precision = 64;
    int npairs = 0;
    char *d_arena = nullptr;
    size_t cap = 0;
    char *h_stage = nullptr;
    size_t hcap = 0;
    char *d_scratch = nullptr;
    size_t scratch_cap = 0;
    std::vector<PFLayout> lay;
    size_t off_pairs = 0, off_queue = 0, off_queue_back = 0, off_ctrl = 0, out_begin = 0, out_end = 0, total = 0;
    size_t nitems = 0;
    int sw = 0, rb = 0;
    long long stride = 0;
    bool have_forward = false;
    double fwd_ms = 0, back_ms = 0;
    double temperature = 300.0;
    double min_am_prob = 0.0;  // > 0: base-match probabilities truncated as AlignerP computes them
    bool gap_gradients = true;  // the backward pass accumulates the gap counts
    std::vector<double> log_z;
    std::vector<std::vector<int>> am_pos;  // per pair: D position of each arc match
};

PFState *state_of(lcg_engine e) {
    if (!e->pf) e->pf = new PFState();
    return (PFState *)e->pf;
}

// log of the sequence-only partition function (base matches and affine gaps,
// no arc matches) over the band, in double with per-row rescaling; its value
// per alignment position sets the FP32 scale factor.
double seq_log_pf(const lcg_pair_tables &t, const std::vector<double> &bm, const std::vector<double> &gA,
                  const std::vector<double> &gB, double o) {
    const int n = t.len_a, m = t.len_b;
    std::vector<double> Mp(m + 1, 0.0), Mc(m + 1, 0.0), Ep(m + 1, 0.0), Ec(m + 1, 0.0);
    double logscale = 0.0;
    Mp[0] = 1.0;
    double g = o;
    for (int j = 1; j <= std::min(m, t.max_col[0]); ++j) {
        g *= gB[j];
        Mp[j] = g;
    }
    double colv = o;
    for (int i = 1; i <= n; ++i) {
        std::fill(Mc.begin(), Mc.end(), 0.0);
        std::fill(Ec.begin(), Ec.end(), 0.0);
        colv *= gA[i];
        if (t.min_col[i] == 0) Mc[0] = colv;
        double F = 0.0;
        const int lo = std::max(1, t.min_col[i]), hi = std::min(m, t.max_col[i]);
        for (int j = lo; j <= hi; ++j) {
            const double E = Ep[j] * gA[i] + (Mp[j] - Ep[j]) * gA[i] * o;
            F = F * gB[j] + (Mc[j - 1] - F) * gB[j] * o;
            Ec[j] = E;
            Mc[j] = Mp[j - 1] * bm[(size_t)i * (m + 1) + j] + E + F;
        }
        double mx = 0.0;
        for (int j = 0; j <= m; ++j) mx = std::max(mx, Mc[j]);
        if (mx > 0.0) {
            for (int j = 0; j <= m; ++j) {
                Mc[j] /= mx;
                Ec[j] /= mx;
            }
            colv /= mx;
            logscale += std::log(mx);
        }
        std::swap(Mp, Mc);
        std::swap(Ep, Ec);
    }
    return logscale + std::log(std::max(Mp[m], 1e-300));
}

template <typename T>
lcg_status pf_forward_t(lcg_engine e, PFState *S, const lcg_pair_tables *pairs, int npairs, const lcg_pf_opts *o,
                        const lcg_pf_grad_spec *specs, double *log_z) {
    const double temp = o->temperature > 0 ? o->temperature : 300.0;
    const double pf_scale = o->pf_scale > 0 ? o->pf_scale : 1.0;
    lcg_align_opts ao{0, 0, 0, 0};
    std::vector<lcg_host::Prep> prep(npairs);
    lcg_host::parallel_for(npairs, [&](int q) { lcg_host::prep_pair(pairs[q], ao, prep[q]); });
    bool need_spec = false;
    for (int k = 2; k < 19; ++k) need_spec |= o->param_delta[k] != 0.0;
    if (need_spec && !specs) return pf_fail(LCG_ERR_ARG, "param_delta[2..18] needs grad specs");
    for (int q = 0; q < npairs; ++q) {
        if (prep[q].code != LCG_OK) return pf_fail(prep[q].code, "pair " + std::to_string(q) + ": " + prep[q].err);
        if (pairs[q].match_lo) return pf_fail(LCG_ERR_UNSUPPORTED, "LocARNA-P ignores anchors in the reference; pass none");
    }
    // layout
    S->lay.assign(npairs, PFLayout{});
    S->am_pos.assign(npairs, std::vector<int>());
    size_t up = 0;
    auto take = [](size_t &cur, size_t bytes) {
        size_t r = cur;
        cur = up16(cur + bytes);
        return r;
    };
    size_t nitems = 0;
    int sw = 0, rows_max = 1, span = 2;
    for (auto &p : prep) {
        nitems += p.groups.size();
        sw = std::max(sw, std::max(p.width_max + 1, p.m + 2));
        rows_max = std::max(rows_max, std::max(p.rows_max + 1, p.n + 1));
        // widest column range two consecutive band rows cover (plus the
        // cell left of the band)
        for (int i = 0; i < p.n; ++i) span = std::max(span, p.max_col[i + 1] - p.min_col[i] + 3);
    }
    S->off_pairs = take(up, sizeof(PFPair<T>) * npairs);
    S->off_queue = take(up, sizeof(int2) * nitems);
    S->off_queue_back = take(up, sizeof(int2) * nitems);
    S->off_ctrl = take(up, 64);
    for (int q = 0; q < npairs; ++q) {
        const auto &p = prep[q];
        PFLayout &L = S->lay[q];
        L.n = p.n;
        L.m = p.m;
        L.na = pairs[q].num_arcmatches;
        L.npos = p.num_pos;
        L.bandcells = p.bandcells;
        L.rowinfo = take(up, 16ull * (p.n + 2));
        L.crow = take(up, 4ull * std::max<size_t>(p.crow.size(), 4));
        L.rowarc = take(up, 4ull * p.rowarc.size());
        L.groups = take(up, sizeof(GroupItem) * p.groups.size());
        L.dw = take(up, sizeof(int4) * std::max<size_t>(p.dw.size(), 1));
        L.bm = take(up, sizeof(T) * (p.n + 1) * (p.m + 1));
        L.gA = take(up, sizeof(T) * (p.n + 1));
        L.gB = take(up, sizeof(T) * (p.m + 1));
        L.w = take(up, sizeof(T) * std::max(L.npos, 1));
        L.D = take(up, sizeof(T) * std::max(L.npos, 1));
    }
    // zero-initialised device section, then the output section
    const size_t zero_begin = up;
    for (int q = 0; q < npairs; ++q) S->lay[q].cnt = take(up, 4ull * std::max(S->lay[q].npos, 1));
    const size_t out_begin = up;
    for (int q = 0; q < npairs; ++q) {
        PFLayout &L = S->lay[q];
        L.res = take(up, 8ull * 4);
        L.Dbar = take(up, sizeof(double) * std::max(L.npos, 1));
        L.bmacc = take(up, sizeof(double) * std::max(L.bandcells, 1));
    }
    const size_t out_end = up;
    for (int q = 0; q < npairs; ++q) S->lay[q].topM = take(up, sizeof(T) * (S->lay[q].n + 1) * (S->lay[q].m + 1));
    // Kept group rectangles: the forward writes every group's M (and, for
    // the gap gradients, E and F) to a rectangle of its own and the backward
    // reads them instead of recomputing the groups, when the pairs'
    // rectangles fit the engine's budget (lcg_engine_set_rect_budget) -
    // single pairs and small batches. By default FP64 only: an FP32
    // recomputation into the warp's slot, read back from L2, is faster than
    // reading the kept rectangle from DRAM (200-nt pair: backward 3.37 ms
    // recomputing, 3.60 ms kept; FP64 7.51 against 6.06 ms).
    const int rect_states = o->gap_gradients ? 3 : 1;
    bool keep;
    {
        const long long budget =
            e->rect_budget >= 0 ? e->rect_budget : (sizeof(T) == 8 ? RECT_BUDGET_PLAIN : 0);
        keep = budget > 0;
        long long cells = 0;
        for (auto &p : prep) {
            if (p.rect_cells < 0) keep = false;
            cells += p.rect_cells;
        }
        keep = keep && (double)cells * rect_states * sizeof(T) <= (double)budget;
    }
    for (int q = 0; q < npairs; ++q)
        S->lay[q].rect = keep ? take(up, sizeof(T) * rect_states * std::max<long long>(prep[q].rect_cells, 1)) : 0;
    const size_t total = up;
    if (total > S->cap) {
        if (S->d_arena) cudaFree(S->d_arena);
        S->d_arena = nullptr;
        S->cap = 0;
        if (cudaMalloc(&S->d_arena, total + total / 4) != cudaSuccess) return pf_fail(LCG_ERR_NOMEM, "PF device arena allocation failed");
        S->cap = total + total / 4;
    }
    if (out_end > S->hcap) {
        if (S->h_stage) cudaFreeHost(S->h_stage);
        S->h_stage = nullptr;
        S->hcap = 0;
        if (cudaMallocHost(&S->h_stage, out_end + out_end / 4) != cudaSuccess) return pf_fail(LCG_ERR_NOMEM, "PF pinned staging allocation failed");
        S->hcap = out_end + out_end / 4;
    }
    char *H = S->h_stage, *Dv = S->d_arena;
    // pack
    PFPair<T> *hp = (PFPair<T> *)(H + S->off_pairs);
    {
        // forward: waves of pairs whose tables fit a share of L2, interleaved
        // by progress inside a wave (as for lcg_align_pairs). Backward (the
        // queue read in reverse): much larger waves, because a group's
        // backward waits for every consumer of its D entries, and more pairs
        // in flight hide those waits (32 pairs of 80-500 nt, one wave
        // against 8 MB ones: FP32 backward 335 -> 283 ms, FP64 841 -> 655 ms,
        // while the forward slows from 74 to 82 ms)
        std::vector<size_t> ng(npairs);
        for (int q = 0; q < npairs; ++q) ng[q] = prep[q].groups.size();
        auto bytes = [&](int q) {
            return (12.0 + 3.0 * sizeof(T)) * prep[q].num_pos + 3.0 * sizeof(T) * prep[q].bandcells;
        };
        auto pfor = [](int n, auto fn) { lcg_host::parallel_for(n, fn); };
        lcg_host::queue_order(ng, bytes, (int2 *)(H + S->off_queue), pfor);
        const char *v = std::getenv("LCG_PF_BACK_WAVE_MB");
        const double back_mb = v ? std::atof(v) : 256.0;
        lcg_host::queue_order(ng, bytes, (int2 *)(H + S->off_queue_back), pfor,
                              (back_mb > 0 ? back_mb : 1e9) * 1048576.0);
    }
    std::memset(H + S->off_ctrl, 0, 64);
    // per pair: Boltzmann weights, scale factor and packed tables (disjoint
    // staging regions, filled in parallel)
    auto pack = [&](int q) {
        const auto &p = prep[q];
        const auto &t = pairs[q];
        const PFLayout &L0 = S->lay[q];
        PFLayout &L = S->lay[q];
        const int n = p.n, m = p.m;
        // Boltzmann weights exp(score / temperature) (scoring.hh:857-860),
        // scores shifted by the continuous parameter offsets
        const double *dl = o->param_delta;
        const lcg_pf_grad_spec *sp = specs ? &specs[q] : nullptr;
        std::vector<double> bm((size_t)(n + 1) * (m + 1), 0.0), gA(n + 1, 0.0), gB(m + 1, 0.0);
        for (int i = 1; i <= n; ++i) {
            const int x = sp && sp->code_a ? sp->code_a[i] : -1;
            for (int j = 1; j <= m; ++j) {
                const int y = sp && sp->code_b ? sp->code_b[j] : -1;
                const double d = (x >= 0 && x < 4 && y >= 0 && y < 4) ? dl[3 + 4 * x + y] : 0.0;
                bm[(size_t)i * (m + 1) + j] = std::exp(((double)t.sigma[(size_t)i * (m + 1) + j] + d) / temp);
            }
        }
        for (int i = 1; i <= n; ++i) gA[i] = std::exp(((double)t.gap_a[i] + dl[0]) / temp);
        for (int j = 1; j <= m; ++j) gB[j] = std::exp(((double)t.gap_b[j] + dl[0]) / temp);
        const double ow = std::exp(((double)t.indel_opening + dl[1]) / temp);
        double logc = 0.0;
        if (sizeof(T) == 4) logc = seq_log_pf(t, bm, gA, gB, ow) / (double)(n + m);
        const double c = std::exp(logc), c2 = c * c;
        L.log_c_total = logc * (n + m);
        std::memcpy(H + L0.rowinfo, p.rowinfo.data(), 16ull * (n + 2));
        if (!p.crow.empty()) std::memcpy(H + L0.crow, p.crow.data(), 4ull * p.crow.size());
        std::memcpy(H + L0.groups, p.groups.data(), sizeof(GroupItem) * p.groups.size());
        if (!p.dw.empty()) std::memcpy(H + L0.dw, p.dw.data(), sizeof(int4) * p.dw.size());
        std::memcpy(H + L0.rowarc, p.rowarc.data(), 4ull * p.rowarc.size());
        T *hbm = (T *)(H + L0.bm);
        for (size_t k = 0; k < bm.size(); ++k) hbm[k] = (T)(bm[k] / c2);
        T *hgA = (T *)(H + L0.gA);
        for (int i = 0; i <= n; ++i) hgA[i] = (T)(gA[i] / c);
        T *hgB = (T *)(H + L0.gB);
        for (int j = 0; j <= m; ++j) hgB[j] = (T)(gB[j] / c);
        T *hw = (T *)(H + L0.w);
        T *hD = (T *)(H + L0.D);
        for (int k = 0; k < L.na; ++k) {
            const int pos = p.am_pos[k];
            if (pos < 0) continue;  // never a term: its right ends are not a band cell
            const double dsw = (sp && sp->am_dscore_dsw) ? dl[2] * sp->am_dscore_dsw[k] : 0.0;
            hw[pos] = (T)std::exp(((double)t.am_score[k] + dsw) / temp);
            if (p.Dinit[pos] == NOT_READY) {
                if (sizeof(T) == 8) {
                    long long bits = PF_NOT_READY_F64;
                    std::memcpy(&hD[pos], &bits, 8);
                } else {
                    int bits = PF_NOT_READY_F32;
                    std::memcpy(&hD[pos], &bits, 4);
                }
            } else {
                hD[pos] = T(0);
            }
        }
        S->am_pos[q] = p.am_pos;
        PFPair<T> &d = hp[q];
        std::memset(&d, 0, sizeof d);
        d.n = n;
        d.m = m;
        d.num_am = L.na;
        d.rowinfo = (const int4 *)(Dv + L0.rowinfo);
        d.crow = (const int2 *)(Dv + L0.crow);
        d.groups = (const GroupItem *)(Dv + L0.groups);
        d.dw = (const int4 *)(Dv + L0.dw);
        d.rowarc = (const int2 *)(Dv + L0.rowarc);
        d.bm = (const T *)(Dv + L0.bm);
        d.gA = (const T *)(Dv + L0.gA);
        d.gB = (const T *)(Dv + L0.gB);
        d.o = (T)ow;
        d.inv_s = (T)(1.0 / pf_scale);
        d.arcf = (T)(pf_scale / (c2 * c2));
        d.w = (const T *)(Dv + L0.w);
        d.D = (T *)(Dv + L0.D);
        d.Dbar = (double *)(Dv + L.Dbar);
        d.cnt = (int *)(Dv + L.cnt);
        d.topM = (T *)(Dv + L.topM);
        d.bmacc = (double *)(Dv + L.bmacc);
        d.res = (double *)(Dv + L.res);
        d.rect = keep ? (T *)(Dv + L.rect) : nullptr;
        d.rect_states = rect_states;
    };
    lcg_host::parallel_for(npairs, pack);
    // scratch: forward one rectangle per warp, backward four
    int bf = 0, bb = 0;
    const int rb = lcg_host::ring_size(span);
    PF_TRY(pf_fwd_occupancy<T>(rb, &bf));
    PF_TRY(pf_back_occupancy<T>(rb, &bb));
    if (bf < 1 || bb < 1) return pf_fail(LCG_ERR_UNSUPPORTED, "PF kernels do not fit on an SM");
    const long long stride = (long long)rows_max * sw;
    const size_t fwd_slots = (size_t)e->sms * bf * pf_warps_per_block();
    const size_t back_slots = (size_t)e->sms * bb * pf_warps_per_block() * 4;
    const size_t need = std::max(fwd_slots, back_slots) * (size_t)stride * sizeof(T);
    if (need > S->scratch_cap) {
        if (S->d_scratch) cudaFree(S->d_scratch);
        S->d_scratch = nullptr;
        S->scratch_cap = 0;
        if (cudaMalloc(&S->d_scratch, need) != cudaSuccess) return pf_fail(LCG_ERR_NOMEM, "PF scratch allocation failed");
        S->scratch_cap = need;
    }
    cudaStream_t st = e->stream;
    PF_TRY(cudaMemcpyAsync(Dv, H, zero_begin, cudaMemcpyHostToDevice, st));
    PF_TRY(cudaMemsetAsync(Dv + zero_begin, 0, out_end - zero_begin, st));
    unsigned int *qhead = (unsigned int *)(Dv + S->off_ctrl);
    int *status = (int *)(Dv + S->off_ctrl + 4);
    int *abort_flag = (int *)(Dv + S->off_ctrl + 8);
    PF_TRY(cudaEventRecord(e->ev0, st));
    PF_TRY(pf_launch_fwd<T>(Dv + S->off_pairs, (const int2 *)(Dv + S->off_queue), (int)nitems,
                            S->d_scratch, stride, sw, rb, qhead, status, abort_flag, e->sms * bf, true, st,
                            keep ? rect_states : 0));
    PF_TRY(cudaEventRecord(e->ev1, st));
    PF_TRY(cudaMemcpyAsync(H + S->off_ctrl, Dv + S->off_ctrl, 64, cudaMemcpyDeviceToHost, st));
    for (int q = 0; q < npairs; ++q)
        PF_TRY(cudaMemcpyAsync(H + S->lay[q].res, Dv + S->lay[q].res, 8, cudaMemcpyDeviceToHost, st));
    PF_TRY(cudaStreamSynchronize(st));
    float ms = 0;
    cudaEventElapsedTime(&ms, e->ev0, e->ev1);
    S->fwd_ms = ms;
    if (((int *)(H + S->off_ctrl))[1] & ST_TIMEOUT) return pf_fail(LCG_ERR_TIMEOUT, "a device wait timed out (PF forward)");
    S->log_z.resize(npairs);
    for (int q = 0; q < npairs; ++q) {
        log_z[q] = ((double *)(H + S->lay[q].res))[0] + S->lay[q].log_c_total;
        S->log_z[q] = log_z[q];
    }
    S->temperature = temp;
    S->min_am_prob = o->min_am_prob;
    S->gap_gradients = o->gap_gradients != 0;
    S->precision = sizeof(T) == 8 ? 64 : 32;
    S->npairs = npairs;
    S->nitems = nitems;
    S->sw = sw;
    S->rb = rb;
    S->stride = stride;
    S->out_begin = out_begin;
    S->out_end = out_end;
    S->total = total;
    S->have_forward = true;
    (void)bb;
    return LCG_OK;
}

template <typename T>
lcg_status pf_backward_t(lcg_engine e, PFState *S, const lcg_pf_grad_spec *grads, lcg_pf_result *results) {
    char *H = S->h_stage, *Dv = S->d_arena;
    cudaStream_t st = e->stream;
    int bb = 0;
    PF_TRY(pf_back_occupancy<T>(S->rb, &bb));
    PF_TRY(cudaMemsetAsync(Dv + S->off_ctrl, 0, 64, st));
    unsigned int *qhead = (unsigned int *)(Dv + S->off_ctrl);
    int *status = (int *)(Dv + S->off_ctrl + 4);
    int *abort_flag = (int *)(Dv + S->off_ctrl + 8);
    PF_TRY(cudaEventRecord(e->ev1, st));
    PF_TRY(pf_launch_back<T>(Dv + S->off_pairs, (const int2 *)(Dv + S->off_queue_back), (int)S->nitems,
                             S->d_scratch, S->stride, S->sw, S->rb, qhead, status, abort_flag, e->sms * bb, st, 0.0,
                             S->gap_gradients));
    PF_TRY(cudaEventRecord(e->ev2, st));
    PF_TRY(cudaMemcpyAsync(H + S->off_ctrl, Dv + S->off_ctrl, 64, cudaMemcpyDeviceToHost, st));
    PF_TRY(cudaMemcpyAsync(H + S->out_begin, Dv + S->out_begin, S->out_end - S->out_begin, cudaMemcpyDeviceToHost, st));
    // D values (for the arc-match probabilities)
    for (int q = 0; q < S->npairs; ++q)
        if (S->lay[q].npos > 0)
            PF_TRY(cudaMemcpyAsync(H + S->lay[q].D, Dv + S->lay[q].D, sizeof(T) * S->lay[q].npos,
                                   cudaMemcpyDeviceToHost, st));
    PF_TRY(cudaStreamSynchronize(st));
    float ms = 0;
    cudaEventElapsedTime(&ms, e->ev1, e->ev2);
    S->back_ms = ms;
    if (((int *)(H + S->off_ctrl))[1] & ST_TIMEOUT) return pf_fail(LCG_ERR_TIMEOUT, "a device wait timed out (PF backward)");
    const double invT = 1.0 / S->temperature;
    for (int q = 0; q < S->npairs; ++q) {
        const PFLayout &L = S->lay[q];
        lcg_pf_result &r = results[q];
        const double *res = (const double *)(H + L.res);
        const double Zs = std::exp(res[0]);  // Z in the scaled frame
        const T *D = (const T *)(H + L.D);
        const double *Db = (const double *)(H + L.Dbar);
        const double *acc = (const double *)(H + L.bmacc);
        const int4 *rowinfo = (const int4 *)(H + L.rowinfo);
        const lcg_pf_grad_spec *g = grads ? &grads[q] : nullptr;
        r.log_z = S->log_z[q];
        // without gap gradients the pass did not accumulate the gap counts
        const double nan = std::numeric_limits<double>::quiet_NaN();
        r.gap_ext_uses = S->gap_gradients ? res[1] / Zs : nan;
        r.gap_open_uses = S->gap_gradients ? res[2] / Zs : nan;
        r.dlogz_dindel = r.gap_ext_uses * invT;
        r.dlogz_dindel_opening = r.gap_open_uses * invT;
        r.dlogz_dstruct_weight = 0.0;
        for (int k = 0; k < 16; ++k) r.dlogz_dbasematch[k] = 0.0;
        const bool sw_grad = g && g->am_dscore_dsw;
        if (r.am_prob || sw_grad) {
            double dsw = 0.0;
            const std::vector<int> &pos = S->am_pos[q];
            for (int k = 0; k < L.na; ++k) {
                const double p = pos[k] >= 0 ? (double)D[pos[k]] * Db[pos[k]] / Zs : 0.0;
                if (r.am_prob) r.am_prob[k] = p;
                if (sw_grad) dsw += p * g->am_dscore_dsw[k];
            }
            r.dlogz_dstruct_weight = dsw * invT;
        }
        const bool bm_grad = g && g->code_a && g->code_b;
        if (r.bm_prob || bm_grad) {
            const int n = L.n, m = L.m;
            if (r.bm_prob) std::memset(r.bm_prob, 0, sizeof(double) * (size_t)(n + 1) * (m + 1));
            double cnt[16] = {0};
            for (int i = 1; i <= n; ++i) {
                const int lo = std::max(1, rowinfo[i].x), hi = std::min(m, rowinfo[i].y);
                for (int j = lo; j <= hi; ++j) {
                    const double p = (double)acc[rowinfo[i].w + j - rowinfo[i].x] / Zs;
                    if (r.bm_prob) r.bm_prob[(size_t)i * (m + 1) + j] = p;
                    if (bm_grad && g->code_a[i] >= 0 && g->code_a[i] < 4 && g->code_b[j] >= 0 && g->code_b[j] < 4)
                        cnt[4 * g->code_a[i] + g->code_b[j]] += p;
                }
            }
            if (bm_grad)
                for (int k = 0; k < 16; ++k) r.dlogz_dbasematch[k] = cnt[k] * invT;
        }
    }
    // base-match probabilities as AlignerP::compute_basematch_probabilities
    // reports them for min_am_prob > 0 (aligner_p.icc:1201-1327): inside an
    // arc match only the arc matches with probability > sqrt(min_am_prob)
    // contribute. A second pass over the groups with the final D_bar; the
    // gradients above keep the exact marginals.
    bool want_bm = false;
    for (int q = 0; q < S->npairs; ++q) want_bm |= results[q].bm_prob != nullptr;
    if (S->min_am_prob > 0.0 && want_bm) {
        for (int q = 0; q < S->npairs; ++q)
            PF_TRY(cudaMemsetAsync(Dv + S->lay[q].bmacc, 0, sizeof(double) * std::max(S->lay[q].bandcells, 1), st));
        PF_TRY(cudaMemsetAsync(Dv + S->off_ctrl, 0, 64, st));
        PF_TRY(pf_launch_back<T>(Dv + S->off_pairs, (const int2 *)(Dv + S->off_queue_back), (int)S->nitems,
                                 S->d_scratch, S->stride, S->sw, S->rb, qhead, status, abort_flag, e->sms * bb, st,
                                 std::sqrt(S->min_am_prob)));
        PF_TRY(cudaEventRecord(e->ev2, st));
        for (int q = 0; q < S->npairs; ++q)
            PF_TRY(cudaMemcpyAsync(H + S->lay[q].bmacc, Dv + S->lay[q].bmacc,
                                   sizeof(double) * std::max(S->lay[q].bandcells, 1), cudaMemcpyDeviceToHost, st));
        PF_TRY(cudaStreamSynchronize(st));
        cudaEventElapsedTime(&ms, e->ev1, e->ev2);
        S->back_ms = ms;
        for (int q = 0; q < S->npairs; ++q) {
            lcg_pf_result &r = results[q];
            if (!r.bm_prob) continue;
            const PFLayout &L = S->lay[q];
            const double Zs = std::exp(((const double *)(H + L.res))[0]);
            const double *acc = (const double *)(H + L.bmacc);
            const int4 *rowinfo = (const int4 *)(H + L.rowinfo);
            const int n = L.n, m = L.m;
            for (int i = 1; i <= n; ++i) {
                const int lo = std::max(1, rowinfo[i].x), hi = std::min(m, rowinfo[i].y);
                for (int j = lo; j <= hi; ++j)
                    r.bm_prob[(size_t)i * (m + 1) + j] = acc[rowinfo[i].w + j - rowinfo[i].x] / Zs;
            }
        }
    }
    return LCG_OK;
}

}  // namespace

namespace lcg_host {
void pf_release(lcg_engine_s *e) {
    PFState *S = (PFState *)e->pf;
    if (!S) return;
    if (S->d_arena) cudaFree(S->d_arena);
    if (S->h_stage) cudaFreeHost(S->h_stage);
    if (S->d_scratch) cudaFree(S->d_scratch);
    delete S;
    e->pf = nullptr;
}
}  // namespace lcg_host

extern "C" {

void lcg_pf_opts_default(lcg_pf_opts *o) {
    std::memset(o, 0, sizeof *o);
    o->temperature = 300.0;
    o->pf_scale = 1.0;
    o->precision = 64;
    o->min_am_prob = 0.001;  // locarna_p --min-am-prob / --min-bm-prob (src/locarna_p.cc:143-146)
    o->min_bm_prob = 0.001;
    o->gap_gradients = 1;
}

lcg_status lcg_pf_forward(lcg_engine e, const lcg_pair_tables *pairs, int32_t npairs, const lcg_pf_opts *opts,
                          const lcg_pf_grad_spec *specs, double *log_z) {
    if (!e || !pairs || !opts || !log_z || npairs < 1) return pf_fail(LCG_ERR_ARG, "bad argument");
    cudaError_t ce = cudaSetDevice(e->device);
    if (ce != cudaSuccess) return pf_fail(LCG_ERR_CUDA, cudaGetErrorString(ce));
    PFState *S = state_of(e);
    S->have_forward = false;
    if (opts->precision == 64) return pf_forward_t<double>(e, S, pairs, npairs, opts, specs, log_z);
    if (opts->precision == 32) return pf_forward_t<float>(e, S, pairs, npairs, opts, specs, log_z);
    return pf_fail(LCG_ERR_ARG, "precision must be 32 or 64");
}

lcg_status lcg_pf_backward(lcg_engine e, const lcg_pf_grad_spec *grads, lcg_pf_result *results) {
    if (!e || !results) return pf_fail(LCG_ERR_ARG, "bad argument");
    PFState *S = state_of(e);
    if (!S->have_forward) return pf_fail(LCG_ERR_ARG, "lcg_pf_backward needs a preceding lcg_pf_forward");
    cudaError_t ce = cudaSetDevice(e->device);
    if (ce != cudaSuccess) return pf_fail(LCG_ERR_CUDA, cudaGetErrorString(ce));
    lcg_status r = S->precision == 64 ? pf_backward_t<double>(e, S, grads, results)
                                       : pf_backward_t<float>(e, S, grads, results);
    S->have_forward = false;  // the backward consumes the use counters
    return r;
}

lcg_status lcg_pf_last_timing(lcg_engine e, double *forward_ms, double *backward_ms) {
    if (!e) return pf_fail(LCG_ERR_ARG, "engine is NULL");
    PFState *S = state_of(e);
    if (forward_ms) *forward_ms = S->fwd_ms;
    if (backward_ms) *backward_ms = S->back_ms;
    return LCG_OK;
}

}  // extern "C"
