// Device-side records of the LocARNA-P engine shared by the kernels
// (pf_kernels.cu) and the host side (engine_pf.cu).
#pragma once
#include <cuda_runtime.h>

namespace lcg {

// NOT_READY pattern of a D entry that a group has yet to write (a NaN that no
// arithmetic produces).
constexpr long long PF_NOT_READY_F64 = 0x7ff4c0de00000000ll;
constexpr int PF_NOT_READY_F32 = 0x7fa0c0de;

template <typename T>
struct PFPair {
    int n, m;
    int num_am;
    const int4 *rowinfo;   // n+2: (min_col, max_col, -, band offset)
    const int2 *crow;      // ((a.l-1) | (b.l-1) << 16, b.r) by row a.r, a.l descending
    const int2 *rowarc;    // n+2: [start, end) of row i's entries in crow
    const T *bm;           // (n+1)(m+1) scaled base-match weights
    const T *gA, *gB;      // scaled gap weights
    T o;                   // gap-opening weight
    T inv_s;               // 1 / pf_scale
    T arcf;                // pf_scale / c^4
    // per D position (the arc match's position in crow):
    const T *w;            // arc-match weight
    T *D;                  // NOT_READY pattern until written
    double *Dbar;          // dZ'/dD (backward), accumulated in FP64
    int *cnt;              // number of uses still to be back-propagated
    T *topM;               // (n+1)(m+1)
    double *bmacc;         // per band cell (row offset rowinfo.w): sum of X_bar M(i-1,j-1) bm, FP64
    double *res;           // [0] log Z', [1] gap-extension uses, [2] gap-opening uses
    const GroupItem *groups;  // left-end groups (work items) in dependency order, top level last
    const int4 *dw;           // D writes: (D index, ar-1, br-1, -), by group, ar ascending
    // Kept group rectangles (nullptr: the backward recomputes them): the
    // forward writes group g's M (rect_states 1) or M, E, F (3; the gap
    // gradients read E and F) to rect + rect_states g.rect_off, state k at
    // k (ar-al)(br-bl), row i-al, column j-bl, pitch br-bl; the backward
    // reads them instead of recomputing the group.
    T *rect;
    int rect_states;
};



template <typename T>
// queue: (pair, group) work items in dependency-respecting order;
// keep_states: 0, or the pairs' PFPair::rect_states (rectangles kept)
cudaError_t pf_launch_fwd(const void *pairs, const int2 *queue, int nitems, void *scratch,
                          long long stride, int pitch, int rb, unsigned int *qhead, int *status, int *abort_flag,
                          int blocks, bool count_uses, cudaStream_t st, int keep_states = 0);
// theta > 0: the truncated base-match pass (min_am_prob = theta^2) after a
// full backward pass; theta = 0: the full adjoint pass, with the gap counts
// (the indel / indel-opening gradients) when grads
template <typename T>
cudaError_t pf_launch_back(const void *pairs, const int2 *queue, int nitems, void *scratch,
                           long long stride, int pitch, int rb, unsigned int *qhead, int *status, int *abort_flag,
                           int blocks, cudaStream_t st, double theta = 0.0, bool grads = true);
// rb: ring size of the shared-memory rows (a power of two above the span of
// any two consecutive band rows)
template <typename T>
cudaError_t pf_fwd_occupancy(int rb, int *blocks_per_sm);
template <typename T>
cudaError_t pf_back_occupancy(int rb, int *blocks_per_sm);
int pf_warps_per_block();

}  // namespace lcg
