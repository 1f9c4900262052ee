// Host-side entry points of the Sankoff kernels (sankoff_kernels.cu,
// sankoff_sl_kernels.cu) used by engine.cu and noalloc.cu.
// sw: scratch row pitch (ints); rb: ring size of the shared-memory rows (a
// multiple of 32 above the column span of any two consecutive band rows).
#pragma once
#include <cuda_runtime.h>

#include "lcg_device.cuh"

namespace lcg {
// fast: every pair has a sigma class table and no anchor constraints
// queue: (pair, group) work items in dependency-respecting order
cudaError_t launch_fill(const PairDev *pairs, const int2 *queue, int nitems, int *scratch,
                        long long scratch_stride, int sw, int rb, bool fast, unsigned int *qhead, int *status,
                        int *abort_flag, int blocks, cudaStream_t st, unsigned long long *counters);
cudaError_t launch_trace(const PairDev *pairs, int npairs, int *scratch, long long scratch_stride, int sw, int rb,
                         int *status, cudaStream_t st, TraceSel sel = TraceSel());
// the top level of the selected pairs under the scoring modified by lam[pair]
// (NULL: 0) and restricted to rst[pair] (NULL: whole sequences)
cudaError_t launch_top(const PairDev *pairs, const int *items, int nitems, const int *lam, const int4 *rst, int rb,
                       int *status, cudaStream_t st);
// out[5 q + k] = result word k (score, max_i, max_j, min_i, min_j) of pair items[q]
cudaError_t launch_gather_res(const PairDev *pairs, const int *items, int nitems, int *out, cudaStream_t st);
cudaError_t fill_occupancy(int rb, bool counting, bool fast, int *blocks_per_sm);
cudaError_t trace_prepare(int rb);
int fill_warps_per_block();
int trace_warps_per_block();
// fast: every pair has a sigma class table and no anchor constraints
// (run_group_slf); keep: the instantiation for kept rectangles;
// blocks_per_sm = 0 when the shared memory does not fit
cudaError_t sl_prepare(int sw, int rb, bool fast, bool keep, int *blocks_per_sm);
int sl_fill_warps_per_block();
// keep: the pairs' group rectangles are kept (PairDev::rect, eight states)
cudaError_t launch_sl_fill(const PairDev *pairs, const int2 *queue, int nitems, int *scratch,
                           long long scratch_stride, int sw, int rb, bool fast, bool keep, unsigned int *qhead,
                           int *status, int *abort_flag, int blocks, cudaStream_t st);
cudaError_t launch_sl_trace(const PairDev *pairs, int npairs, int *scratch, long long scratch_stride, int sw,
                            int rb, bool fast, int *status, cudaStream_t st, TraceSel sel = TraceSel());
}  // namespace lcg
