// GB300 (sm_103a) kernels of the sparsified Sankoff aligner.
//
//   sankoff_fill_kernel  persistent, warp-per-work-item dataflow kernel that
//                        fills the arc-match table D for every left-end group
//                        of every pair and runs each pair's top level
//                        (reference: AlignerImpl::align_D, aligner.cc:660-732;
//                        align_in_arcmatch :373-437; align_noex :153-233;
//                        fill_D_entries :574-610; top levels :736-880).
//   sankoff_trace_kernel one warp per pair: traceback on the top-level matrix,
//                        recomputing M inside each traced arc match
//                        (trace :1345-1358, trace_in_arcmatch :1233-1343,
//                        trace_noex :1082-1229, trace_arcmatch :967-1028).
//
// Work decomposition. A left-end group (al,bl) sweeps the rows al+1..ar-1 of
// its rectangle; the 32 lanes of its warp cover the band-restricted columns of
// a row in chunks of 32. Per cell the diagonal, vertical-gap (E) and arc-match
// terms are independent across the row; the horizontal gap chain
//   F(j) = max(F(j-1) + gB(j), M(i,j-1) + gB(j) + go),  M = max(X, F)
// is rewritten as the max-plus affine recurrence
//   F(j) = max(F(j-1) + gB(j) + max(go,0), X(j-1) + gB(j) + go)
// and evaluated with a warp-wide max-plus scan (exact for integers).
//
// Dataflow. Items are dequeued in an order where every group precedes the
// groups that read its D entries (per pair: al descending, bl descending, the
// reference's own loop order). A D entry starts as NOT_READY; its producer
// writes it as soon as the cell (ar-1,br-1) is final, and a consumer reading it
// in its own row spins (bounded) until it is written. Because a consumer only
// waits on items dequeued before its own, the lowest unfinished item never
// waits, so the schedule always progresses; each spin is bounded and reports
// ST_TIMEOUT instead of hanging.
#include <cuda_runtime.h>
#include <stdint.h>

#include "sankoff_group.cuh"

namespace lcg {

template <bool COUNT, bool FAST>
__global__ void __launch_bounds__(FILL_WARPS * 32, FILL_MIN_BLOCKS)
    sankoff_fill_kernel(const PairDev *__restrict__ pairs, const int2 *__restrict__ queue,
                        int nitems, int *scratch,
                        long long scratch_stride, int sw, int rb, unsigned int *qhead, int *status,
                        int *abort_flag_ptr, unsigned long long *counters) {
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const int sbase = warp * smem_warp_ints(rb);
    int *Mg = scratch + ((long long)blockIdx.x * FILL_WARPS + warp) * scratch_stride;
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
            run_top<COUNT, FAST>(P, it.cpl, sbase, rb, status, abort_flag, counters);
        } else {
            // the group's own kept rectangle, or the warp's scratch slot
            const bool kept = P.rect && it.rect_off >= 0;
            run_group<false, true, true, COUNT, FAST>(P, it.cpl, it.al, it.ar, it.bl, it.br,
                                                kept ? P.rect + it.rect_off : Mg, kept ? it.br - it.bl : sw,
                                                sbase, rb, dw + it.dw_start, it.dw_count, true, true, false,
                                                status, abort_flag, nullptr, counters);
        }
        __syncwarp();
    }
}

__global__ void __launch_bounds__(TRACE_WARPS * 32)
    sankoff_trace_kernel(const PairDev *__restrict__ pairs, int npairs, int *scratch,
                         long long scratch_stride, int sw, int rb, int *status, TraceSel sel) {
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
    const int sbase = warp * smem_warp_ints(rb);
    int *Mg = scratch + (long long)pair * scratch_stride;
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
        walk(w, P.topM + (size_t)(sA - 1) * (P.m + 1) + (sB - 1), P.m + 1, sA - 1, sB - 1, P.res[R_MAXI],
             P.res[R_MAXJ], true, status, lam);
        P.segs[nseg++] = make_int4(-1, 0, w.ntok, 0);
    }
    if (sel.flags & TRACE_TOP_ONLY) return;
    int qtail = __shfl_sync(0xffffffffu, w.qtail, 0);
    while (qhead < qtail) {
        int4 qe = make_int4(-1, 0, 0, 0);
        if (lane == 0 && qhead < P.tq_cap) qe = P.tq[qhead];
        const int k = __shfl_sync(0xffffffffu, qe.x, 0), kaux = __shfl_sync(0xffffffffu, qe.y, 0);
        const int lefts = __shfl_sync(0xffffffffu, qe.z, 0), rights = __shfl_sync(0xffffffffu, qe.w, 0);
        ++qhead;
        if (k < 0) break;
        const int4 ends = trace_ends(lefts, rights);  // a.l, a.r, b.l, b.r
        if (lefts & TQ_CHAIN) {
            if (lane == 0) trace_chain(w, k, kaux, ends, nseg, status);
            __syncwarp();
            qtail = __shfl_sync(0xffffffffu, w.qtail, 0);
            continue;
        }
        if ((P.flags & (PF_STACK | PF_NOLP)) == PF_STACK) {
            int stacked = 0;
            if (lane == 0) stacked = trace_stack(w, k, kaux, ends, nseg);
            if (__shfl_sync(0xffffffffu, stacked, 0)) {
                qtail = __shfl_sync(0xffffffffu, w.qtail, 0);
                continue;
            }
        }
        // the arc match's rectangle: its group's kept one from the fill, else
        // recomputed into the pair's scratch slot
        const int2 kr = P.am_rect ? P.am_rect[k] : make_int2(-1, 0);
        const int *Mw = Mg;
        int pw = sw;
        if (kr.x >= 0) {
            Mw = P.rect + kr.x;
            pw = kr.y;
        } else {
            const int cpl = min(4, max(1, (min(ends.w - ends.z, P.maxband) + 31) / 32));
            run_group<false, false, false>(P, cpl, ends.x, ends.y, ends.z, ends.w, Mg, sw, sbase, rb, nullptr, 0,
                                           true, true, false, status, (volatile int *)&dummy_abort, nullptr);
        }
        __syncwarp();
        if (lane == 0) {
            const int start = w.ntok;
            walk(w, Mw, pw, ends.x, ends.z, ends.y - 1, ends.w - 1, false, status);
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

template <bool COUNT, bool FAST>
static const void *fill_fn() {
    return (const void *)sankoff_fill_kernel<COUNT, FAST>;
}

cudaError_t launch_fill(const PairDev *pairs, const int2 *queue, int nitems,
                        int *scratch, long long scratch_stride, int sw, int rb, bool fast, unsigned int *qhead,
                        int *status, int *abort_flag, int blocks, cudaStream_t st,
                        unsigned long long *counters) {
    size_t smem = (size_t)FILL_WARPS * smem_warp_ints(rb) * sizeof(int);
    if (counters && fast)
        sankoff_fill_kernel<true, true><<<blocks, FILL_WARPS * 32, smem, st>>>(
            pairs, queue, nitems, scratch, scratch_stride, sw, rb, qhead, status, abort_flag, counters);
    else if (counters)
        sankoff_fill_kernel<true, false><<<blocks, FILL_WARPS * 32, smem, st>>>(
            pairs, queue, nitems, scratch, scratch_stride, sw, rb, qhead, status, abort_flag, counters);
    else if (fast)
        sankoff_fill_kernel<false, true><<<blocks, FILL_WARPS * 32, smem, st>>>(
            pairs, queue, nitems, scratch, scratch_stride, sw, rb, qhead, status, abort_flag, counters);
    else
        sankoff_fill_kernel<false, false><<<blocks, FILL_WARPS * 32, smem, st>>>(
            pairs, queue, nitems, scratch, scratch_stride, sw, rb, qhead, status, abort_flag, counters);
    return cudaGetLastError();
}

cudaError_t launch_trace(const PairDev *pairs, int npairs, int *scratch,
                         long long scratch_stride, int sw, int rb, int *status, cudaStream_t st, TraceSel sel) {
    size_t smem = (size_t)TRACE_WARPS * smem_warp_ints(rb) * sizeof(int);
    const int nw = sel.items ? sel.nitems : npairs;
    if (nw <= 0) return cudaSuccess;
    int blocks = (nw + TRACE_WARPS - 1) / TRACE_WARPS;
    sankoff_trace_kernel<<<blocks, TRACE_WARPS * 32, smem, st>>>(pairs, npairs, scratch,
                                                                 scratch_stride, sw, rb, status, sel);
    return cudaGetLastError();
}

// The top level alone, one warp per selected pair, after the fill kernel has
// made D final: under the modified scoring view of normalized and penalized
// alignment (every position penalised by lam[pair]; align_top_level_locally /
// _free_endgaps with a ModifiedScoringView, aligner.cc:1561-1562, 1606-1610)
// and/or restricted to the interval rst[pair] of k-best alignment
// (Aligner::suboptimal, aligner.cc:1384-1512). Writes the pair's top-level
// matrix and result words like the fill kernel's top item.
__global__ void __launch_bounds__(TRACE_WARPS * 32)
    sankoff_top_kernel(const PairDev *__restrict__ pairs, const int *__restrict__ items, int nitems,
                       const int *__restrict__ lam, const int4 *__restrict__ rst, int rb, int *status) {
    const int warp = threadIdx.x >> 5;
    const int wi = blockIdx.x * TRACE_WARPS + warp;
    if (wi >= nitems) return;
    const int pair = items[wi];
    const PairDev &P = pairs[pair];
    int dummy_abort = 0;
    run_top<false, false, true>(P, 1, warp * smem_warp_ints(rb), rb, status, (volatile int *)&dummy_abort,
                                nullptr, lam ? lam[pair] : 0, rst ? rst + pair : nullptr);
}

// result words of the selected pairs, gathered for one device->host copy:
// out[5 q + k] = res[k] of items[q], k = score, max_i, max_j, min_i, min_j
__global__ void gather_res_kernel(const PairDev *__restrict__ pairs, const int *__restrict__ items, int nitems,
                                  int *__restrict__ out) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nitems) return;
    const int *r = pairs[items[q]].res;
    for (int k = 0; k < 5; ++k) out[5 * q + k] = r[k];
}

cudaError_t launch_top(const PairDev *pairs, const int *items, int nitems, const int *lam, const int4 *rst, int rb,
                       int *status, cudaStream_t st) {
    if (nitems <= 0) return cudaSuccess;
    size_t smem = (size_t)TRACE_WARPS * smem_warp_ints(rb) * sizeof(int);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(sankoff_top_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
    }
    int blocks = (nitems + TRACE_WARPS - 1) / TRACE_WARPS;
    sankoff_top_kernel<<<blocks, TRACE_WARPS * 32, smem, st>>>(pairs, items, nitems, lam, rst, rb, status);
    return cudaGetLastError();
}

cudaError_t launch_gather_res(const PairDev *pairs, const int *items, int nitems, int *out, cudaStream_t st) {
    if (nitems <= 0) return cudaSuccess;
    gather_res_kernel<<<(nitems + 127) / 128, 128, 0, st>>>(pairs, items, nitems, out);
    return cudaGetLastError();
}

int fill_warps_per_block() { return FILL_WARPS; }
int trace_warps_per_block() { return TRACE_WARPS; }

cudaError_t fill_occupancy(int rb, bool counting, bool fast, int *blocks_per_sm) {
    size_t smem = (size_t)FILL_WARPS * smem_warp_ints(rb) * sizeof(int);
    int dev = 0, optin = 0;
    cudaError_t ge = cudaGetDevice(&dev);
    if (ge == cudaSuccess) ge = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (ge != cudaSuccess) return ge;
    if (smem > (size_t)optin) {  // band rows too wide for the shared-memory rings
        *blocks_per_sm = 0;
        return cudaSuccess;
    }
    const void *k = counting ? (fast ? fill_fn<true, true>() : fill_fn<true, false>())
                             : (fast ? fill_fn<false, true>() : fill_fn<false, false>());
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k, FILL_WARPS * 32, smem);
}

cudaError_t trace_prepare(int rb) {
    size_t smem = (size_t)TRACE_WARPS * smem_warp_ints(rb) * sizeof(int);
    if (smem > 48 * 1024)
        return cudaFuncSetAttribute(sankoff_trace_kernel,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    return cudaSuccess;
}

}  // namespace lcg
