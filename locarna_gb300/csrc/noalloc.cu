// Allocation-free entry point: the score of one pair computed with every
// device byte taken from a fixed file-scope device array.
//
// Who needs it: callers that cannot allocate device memory while they run,
// for example a service whose GPU memory is reserved up front by another
// framework's allocator (a cudaMalloc of its own would fail or fragment that
// reservation), or a real-time loop in which cudaMalloc / cudaFree are not
// acceptable because they may synchronise the whole device.
// lcg_align_pairs grows its own device and pinned host buffers on demand;
// this entry point never calls cudaMalloc, cudaFree, cudaMallocHost or any
// other allocating CUDA or library routine. Host-side preparation of the
// pair's index structures uses ordinary heap memory.
//
// Limits and sharing:
//  * all device data of a call (copied inputs, the arc-match table, the
//    top-level matrix and the per-warp group matrices) must fit in
//    LCG_STATIC_SCRATCH_BYTES; larger pairs are rejected with LCG_ERR_RANGE;
//  * the array exists once per GPU that loads the library and is held until
//    the process exits;
//  * every call reuses the same array: the words that must start at zero are
//    cleared and every input is copied in at the start of each call, but two
//    calls whose GPU work overlaps (for example on two streams) race on it;
//  * the first call on a device looks up the array's device address with
//    cudaGetSymbolAddress.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/locarna_gb300.h"
#include "engine_prep.hh"
#include "lcg_device.cuh"

#include "sankoff_launch.hh"

using namespace lcg;

// The allocation-free entry point's device memory: one fixed array per GPU.
static __device__ __align__(256) unsigned char lcg_static_scratch[LCG_STATIC_SCRATCH_BYTES];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
char *g_scratch_ptr[kMaxDevices] = {};

lcg_status static_fail(lcg_status code, const std::string &msg) {
    lcg_host::set_error(msg);
    return code;
}

size_t up256(size_t x) { return (x + 255) / 256 * 256; }

// Device address of the static array on `dev` (looked up once per device,
// with that device current).
lcg_status static_base(int dev, char **out) {
    if (dev < 0 || dev >= kMaxDevices) return static_fail(LCG_ERR_ARG, "device index out of range");
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, lcg_static_scratch);
        if (e != cudaSuccess)
            return static_fail(LCG_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        g_scratch_ptr[dev] = (char *)p;
    }
    *out = g_scratch_ptr[dev];
    return LCG_OK;
}

}  // namespace

#define STATIC_TRY(call)                                                                       \
    do {                                                                                       \
        cudaError_t _e = (call);                                                               \
        if (_e != cudaSuccess)                                                                 \
            return static_fail(LCG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e)); \
    } while (0)

// After the launch: on failure, wait for the stream (ignoring its status)
// before returning, so that no work of this call still uses the shared array
// when the next call starts overwriting it.
#define STATIC_TRY_DRAIN(call, s)                                                              \
    do {                                                                                       \
        cudaError_t _e = (call);                                                               \
        if (_e != cudaSuccess) {                                                               \
            cudaStreamSynchronize(s);                                                          \
            return static_fail(LCG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e)); \
        }                                                                                      \
    } while (0)

extern "C" lcg_status lcg_align_score_static(const lcg_pair_tables *pair, const lcg_align_opts *opts,
                                             int64_t *score, int32_t *max_i, int32_t *max_j,
                                             void *stream) {
    if (!pair || !opts || !score) return static_fail(LCG_ERR_ARG, "NULL argument");
    if (opts->struct_local) return static_fail(LCG_ERR_UNSUPPORTED, "static entry point: plain (non struct-local) mode only");
    if (opts->do_trace) return static_fail(LCG_ERR_UNSUPPORTED, "static entry point computes the score only (do_trace must be 0)");
    if (opts->normalized || opts->penalized)
        return static_fail(LCG_ERR_UNSUPPORTED, "static entry point: no normalized or penalized alignment");
    int dev = 0;
    STATIC_TRY(cudaGetDevice(&dev));
    char *base = nullptr;
    lcg_status st = static_base(dev, &base);
    if (st != LCG_OK) return st;
    cudaStream_t s = (cudaStream_t)stream;

    lcg_host::Prep p;
    if (lcg_host::prep_pair(*pair, *opts, p) != LCG_OK) return static_fail(p.code, p.err);
    const int n = p.n, m = p.m;
    const int na = pair->num_arcmatches;
    const bool anch = pair->match_lo != nullptr;
    int sw = std::max(p.width_max + 1, m + 2);
    int rows_max = p.rows_max + 1;

    // layout of the static array
    size_t off = 0;
    auto take = [&](size_t bytes) {
        size_t o = off;
        off = up256(off + bytes);
        return o;
    };
    const size_t o_pair = take(sizeof(PairDev));
    const size_t o_items = take(sizeof(GroupItem) * p.groups.size());
    const size_t o_dw = take(sizeof(int4) * std::max<size_t>(p.dw.size(), 1));
    const size_t o_dwn = take(sizeof(int2) * std::max<size_t>(p.dwn.size(), 1));  // no lonely pairs
    const size_t o_queue = take(sizeof(int2) * p.groups.size());
    const size_t o_gbc = take(4ull * (m + 1));
    const size_t o_ctrl = take(64);
    const size_t o_res = take(4ull * R_NWORDS);
    const size_t o_sigma = p.use_cls ? 0 : take(4ull * (n + 1) * (m + 1));
    const size_t o_scls = p.use_cls ? take(4ull * 256) : 0;
    const size_t o_rcls = p.use_cls ? take(4ull * (n + 2)) : 0;
    const size_t o_ccls = p.use_cls ? take(4ull * (m + 1)) : 0;
    const size_t o_gapA = take(4ull * (n + 1));
    const size_t o_gapB = take(4ull * (m + 1));
    const size_t o_minc = take(4ull * (n + 2));
    const size_t o_maxc = take(4ull * (n + 2));
    const size_t o_band = take(4ull * (n + 2));
    const size_t o_row = take(16ull * (n + 2));
    const size_t o_anc = anch ? take(4ull * (4 * (n + 1) + 2 * (m + 1))) : 0;
    const size_t o_cs = take(4ull * (p.bandcells + 1));
    const size_t o_cre = take(4ull * std::max<size_t>(p.cre.size(), 4));
    const size_t o_crow = take(4ull * std::max<size_t>(p.crow.size(), 4));
    const size_t o_rowarc = take(4ull * p.rowarc.size());
    const size_t o_score = take(4ull * std::max(na, 1));
    const size_t o_D = take(4ull * std::max(p.num_pos, 1));
    const size_t o_top = take(4ull * (n + 1) * (m + 1));
    const size_t fixed = off;
    const long long stride = (long long)rows_max * sw;  // ints per warp slot
    const size_t per_block = (size_t)fill_warps_per_block() * (size_t)stride * sizeof(int);
    if (fixed + per_block > LCG_STATIC_SCRATCH_BYTES)
        return static_fail(LCG_ERR_RANGE, "pair too large for the static scratch of the allocation-free entry point: needs " +
                                              std::to_string(fixed + per_block) + " bytes, limit " +
                                              std::to_string((size_t)LCG_STATIC_SCRATCH_BYTES));
    int blocks_per_sm = 0;
    const int rb = lcg_host::ring_size(p.span);
    const bool fast = (p.flags & PF_SCLS) && !(p.flags & (PF_ANCHORS | PF_NOLP | PF_STACK));
    STATIC_TRY(fill_occupancy(rb, false, fast, &blocks_per_sm));
    int sms = 0;
    STATIC_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const size_t room = LCG_STATIC_SCRATCH_BYTES - fixed;
    long long blocks = std::min<long long>((long long)sms * std::max(blocks_per_sm, 1), (long long)(room / per_block));
    if (blocks_per_sm < 1 || blocks < 1)
        return static_fail(LCG_ERR_RANGE, "pair too large for the static scratch of the allocation-free entry point: needs " +
                                              std::to_string(fixed + per_block) + " bytes, limit " +
                                              std::to_string((size_t)LCG_STATIC_SCRATCH_BYTES));
    int *scratch = (int *)(base + fixed);

    // device view of the pair
    PairDev d;
    std::memset(&d, 0, sizeof d);
    d.n = n;
    d.m = m;
    d.go = pair->indel_opening;
    d.excl = pair->exclusion;
    d.flags = p.flags & ~PF_TRACE;
    d.free_endgaps = p.fe;
    d.la = anch ? pair->left_anchor_a : n + 1;
    d.lb = anch ? pair->left_anchor_b : m + 1;
    d.ra = anch ? pair->right_anchor_a : 0;
    d.rb = anch ? pair->right_anchor_b : 0;
    d.num_am = na;
    d.bandcells = p.bandcells;
    d.maxband = p.maxband;
    if (p.use_cls) {
        d.scls = (const int *)(base + o_scls);
        d.rcls = (const int *)(base + o_rcls);
        d.ccls = (const int *)(base + o_ccls);
    } else {
        d.sigma = (const int *)(base + o_sigma);
    }
    d.gapA = (const int *)(base + o_gapA);
    d.gapB = (const int *)(base + o_gapB);
    d.min_col = (const int *)(base + o_minc);
    d.max_col = (const int *)(base + o_maxc);
    d.bandoff = (const int *)(base + o_band);
    d.rowinfo = (const int4 *)(base + o_row);
    if (anch) {
        const int *a = (const int *)(base + o_anc);
        d.match_lo = a;
        d.match_hi = a + (n + 1);
        d.del_lo = a + 2 * (n + 1);
        d.del_hi = a + 3 * (n + 1);
        d.ins_lo = a + 4 * (n + 1);
        d.ins_hi = a + 4 * (n + 1) + (m + 1);
    }
    d.cre_start = (const int *)(base + o_cs);
    d.cre = (const int4 *)(base + o_cre);
    d.crow = (const int2 *)(base + o_crow);
    d.num_pos = p.num_pos;
    d.rowarc = (const int2 *)(base + o_rowarc);
    d.D = (int *)(base + o_D);
    d.am_score = (const int *)(base + o_score);
    d.topM = (int *)(base + o_top);
    d.res = (int *)(base + o_res);
    for (auto &g : p.groups) g.pair = 0;
    d.groups = (const GroupItem *)(base + o_items);
    d.dw = (const int4 *)(base + o_dw);
    d.dwn = (p.flags & (PF_NOLP | PF_STACK)) ? (const int2 *)(base + o_dwn) : nullptr;
    d.gbc = (const int *)(base + o_gbc);
    std::vector<int2> queue(p.groups.size());  // one pair: the groups in their own order
    for (size_t g = 0; g < queue.size(); ++g) queue[g] = make_int2(0, (int)g);

    // inputs (pageable host memory; no staging buffer), cleared control words
    auto h2d = [&](size_t o, const void *src, size_t bytes) {
        return bytes ? cudaMemcpyAsync(base + o, src, bytes, cudaMemcpyHostToDevice, s) : cudaSuccess;
    };
    STATIC_TRY(h2d(o_pair, &d, sizeof d));
    STATIC_TRY(h2d(o_items, p.groups.data(), sizeof(GroupItem) * p.groups.size()));
    STATIC_TRY(h2d(o_dw, p.dw.data(), sizeof(int4) * p.dw.size()));
    STATIC_TRY(h2d(o_dwn, p.dwn.data(), sizeof(int2) * p.dwn.size()));
    STATIC_TRY(h2d(o_queue, queue.data(), sizeof(int2) * queue.size()));
    STATIC_TRY(h2d(o_gbc, p.gbc.data(), 4ull * (m + 1)));
    STATIC_TRY(cudaMemsetAsync(base + o_ctrl, 0, 64, s));
    STATIC_TRY(cudaMemsetAsync(base + o_res, 0, 4ull * R_NWORDS, s));
    if (p.use_cls) {
        STATIC_TRY(h2d(o_scls, p.scls.data(), 4ull * 256));
        STATIC_TRY(h2d(o_rcls, p.rcls.data(), 4ull * (n + 2)));
        STATIC_TRY(h2d(o_ccls, p.ccls.data(), 4ull * (m + 1)));
    } else {
        STATIC_TRY(h2d(o_sigma, pair->sigma, 4ull * (n + 1) * (m + 1)));
    }
    STATIC_TRY(h2d(o_gapA, pair->gap_a, 4ull * (n + 1)));
    STATIC_TRY(h2d(o_gapB, pair->gap_b, 4ull * (m + 1)));
    STATIC_TRY(h2d(o_minc, p.min_col.data(), 4ull * (n + 2)));
    STATIC_TRY(h2d(o_maxc, p.max_col.data(), 4ull * (n + 2)));
    STATIC_TRY(h2d(o_band, p.bandoff.data(), 4ull * (n + 2)));
    STATIC_TRY(h2d(o_row, p.rowinfo.data(), 16ull * (n + 2)));
    if (anch) {
        const size_t A = 4ull * (n + 1), B = 4ull * (m + 1);
        STATIC_TRY(h2d(o_anc, pair->match_lo, A));
        STATIC_TRY(h2d(o_anc + A, pair->match_hi, A));
        STATIC_TRY(h2d(o_anc + 2 * A, pair->del_lo, A));
        STATIC_TRY(h2d(o_anc + 3 * A, pair->del_hi, A));
        STATIC_TRY(h2d(o_anc + 4 * A, pair->ins_lo, B));
        STATIC_TRY(h2d(o_anc + 4 * A + B, pair->ins_hi, B));
    }
    STATIC_TRY(h2d(o_cs, p.cre_start.data(), 4ull * (p.bandcells + 1)));
    STATIC_TRY(h2d(o_cre, p.cre.data(), 4ull * p.cre.size()));
    STATIC_TRY(h2d(o_crow, p.crow.data(), 4ull * p.crow.size()));
    STATIC_TRY(h2d(o_rowarc, p.rowarc.data(), 4ull * p.rowarc.size()));
    STATIC_TRY(h2d(o_score, pair->am_score, 4ull * na));
    STATIC_TRY(h2d(o_D, p.Dinit.data(), 4ull * p.num_pos));

    STATIC_TRY_DRAIN(launch_fill((const PairDev *)(base + o_pair), (const int2 *)(base + o_queue),
                                 (int)p.groups.size(), scratch, stride, sw, rb, fast,
                                 (unsigned int *)(base + o_ctrl), (int *)(base + o_ctrl + 4),
                                 (int *)(base + o_ctrl + 8), (int)blocks, s, nullptr),
                     s);
    int ctrl[4] = {0, 0, 0, 0};
    int res[R_NWORDS] = {0};
    STATIC_TRY_DRAIN(cudaMemcpyAsync(ctrl, base + o_ctrl, sizeof ctrl, cudaMemcpyDeviceToHost, s), s);
    STATIC_TRY_DRAIN(cudaMemcpyAsync(res, base + o_res, sizeof res, cudaMemcpyDeviceToHost, s), s);
    STATIC_TRY(cudaStreamSynchronize(s));
    if (ctrl[1] & ST_TIMEOUT) return static_fail(LCG_ERR_TIMEOUT, "a device wait for an arc-match entry timed out");
    if (ctrl[1]) return static_fail(LCG_ERR_DEVICE, "kernel reported an internal error");
    *score = res[R_SCORE] < MIN_FINITE ? LCG_NEG_INF : (int64_t)res[R_SCORE];
    if (max_i) *max_i = res[R_MAXI];
    if (max_j) *max_j = res[R_MAXJ];
    return LCG_OK;
}
