// State of an lcg_engine, shared by the alignment (engine.cu) and the
// partition-function (engine_pf.cu) entry points.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <vector>

#include "../../include/locarna_gb300.h"

// The CUDA graph of one buffer set's last chunk (upload, clear, fill,
// traceback, download) and the launch parameters it was captured with; a
// chunk with the same parameters replays it, a chunk with other parameters
// updates it in place (or instantiates it again when the update is
// refused). release() destroys it: before any buffer of the set that its
// nodes address is freed, so that no graph ever refers to freed memory, and
// at engine teardown.
struct lcg_graph_cache {
    cudaGraphExec_t exec = nullptr;
    std::vector<long long> key;
    void release() {
        if (exec) cudaGraphExecDestroy(exec);
        exec = nullptr;
        key.clear();
    }
};

// Device arena, pinned staging, fill scratch, stream and events of one
// in-flight chunk of an lcg_align_pairs call. The engine's own fields are
// the first set; `alt` is the second one of the double-buffered pipeline.
struct lcg_buffer_set {
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    char *d_arena = nullptr;
    size_t arena_cap = 0;
    char *h_stage = nullptr;
    size_t stage_cap = 0;
    int *d_scratch = nullptr;
    size_t scratch_cap = 0;  // ints
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev2 = nullptr;
    lcg_graph_cache graph;
};

// default budgets of kept group rectangles (bytes): plain chunks, and
// structure-local chunks, whose rectangles hold eight state matrices
constexpr long long RECT_BUDGET_PLAIN = 4ll << 30;
constexpr long long RECT_BUDGET_SL = 32ll << 30;

struct lcg_engine_s {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int sms = 0;
    char *d_arena = nullptr;
    size_t arena_cap = 0;
    char *h_stage = nullptr;
    size_t stage_cap = 0;
    int *d_scratch = nullptr;
    size_t scratch_cap = 0;  // ints
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev2 = nullptr;
    double last_ms = 0, last_fill_ms = 0, last_trace_ms = 0;
    long long last_launches = 0;
    long long last_h2d = 0, last_d2h = 0;
    long long last_groups = 0, last_cells = 0, last_terms = -1, last_visits = -1;
    bool counting = false;
    // wall-clock phases of the last lcg_align_pairs call (ms): host preparation,
    // packing, copies + kernels (until the results are on the host), result assembly
    double last_phase_ms[4] = {0, 0, 0, 0};
    void *pf = nullptr;  // partition-function state (engine_pf.cu)
    // pipeline of lcg_align_pairs: pairs per chunk (0 = automatic) and the
    // second buffer set (created on first use)
    int chunk_pairs = 0;
    lcg_buffer_set alt;
    // autotuner (lcg_engine_autotune): per length bucket the fill kernel's
    // resident blocks per SM (0 = as many as fit) and the L2 budget of a pair
    // wave in MB (0 = default); used by lcg_align_pairs when autotune is on
    bool autotune = false;
    // bytes of kept group rectangles a chunk may use (lcg_engine_set_rect_budget;
    // < 0: RECT_BUDGET_PLAIN / RECT_BUDGET_SL by the chunk's mode)
    long long rect_budget = -1;
    int tune_bps[LCG_TUNE_BUCKETS] = {0, 0, 0, 0};
    double tune_wave_mb[LCG_TUNE_BUCKETS] = {0, 0, 0, 0};
    // CUDA graphs of the chunks (lcg_engine_set_graphs): the own set's cache
    // (the second set keeps its own in `alt`) and the counts of the last call
    bool graphs = true;
    lcg_graph_cache graph;
    long long last_graph_captures = 0, last_graph_replays = 0;
    // a configuration forced for every chunk (the autotuner's trials)
    int force_bps = 0;
    double force_wave_mb = 0;
    // batched table preparation (envelope.cu): device arena and pinned staging
    char *env_dev = nullptr;
    size_t env_dev_cap = 0;
    char *env_host = nullptr;
    size_t env_host_cap = 0;
    // bytes the last lcg_prepare_pairs call copied host->device / device->host
    long long prep_h2d = 0, prep_d2h = 0;
};

namespace lcg_host {
void pf_release(lcg_engine_s *e);
}
