// Host interface of the GPU sequence envelope (envelope.cu), used by the
// batched table preparation lcg_prepare_pairs (host_prep.cpp). Plain C++
// types only: host_prep.cpp is compiled without the CUDA headers.
//
// The envelope is the reference's trace-probability band: PFGotoh forward and
// reverse partition functions of the sequence-only Gotoh alignment with
// StralScore match scores (edge_probs.icc:76-162, stral_score.cc:29-60), the
// edge probabilities of PFTraceProbs (edge_probs.icc:212-268) and the per-row
// threshold of TraceController::restrict_by_trace_probabilities
// (trace_controller.cc:565-581).
#pragma once
#include <cstdint>
#include <string>

#include "../../include/locarna_gb300.h"

namespace lcg_env {

struct Params {
    double sw;        // struct weight / 100
    double temp;      // temperature_alipf / 100
    double g_open;    // exp(gap_opening / temp)
    double g_ext;     // exp(gap_extension / temp)
    double min_prob;  // threshold (min_trace_probability)
    double score[16]; // sequence score of base codes (a, b) in 0..3 (RIBOSUM or match/mismatch)
    int local;        // sequence-local envelope
    int fe;           // LCG_FREE_* bits
    int exp_limit;    // |log2| range of the reference's float type (double / long double)
};

struct PairIn {
    int n, m;
    const int8_t *ca, *cb;                // base codes 0..3 or -1, index 1..n / 1..m
    const double *sdA, *suA, *sdB, *suB;  // sqrt of the down / up pairing probabilities, 1-based
    const int32_t *minc, *maxc;           // band before the envelope (n+1)
};

// Per pair: the row bounds the threshold keeps (new_min / new_max of
// restrict_by_trace_probabilities before clamping, n+1 each) and a flag:
// 0 = exact, 1 = a probability within the rounding margin of the threshold
// could move a bound, 2 = values outside the safe range of the reference's
// float type. Flagged pairs are recomputed on the host.
struct PairOut {
    int32_t *newmin, *newmax;
    int flag;
};

// Compute the envelopes of npairs pairs on the engine's device (one warp per
// pair). Returns LCG_OK or an error with err set.
lcg_status compute(lcg_engine eng, const Params &P, int npairs, const PairIn *in, PairOut *out, std::string &err);

// The same, enqueued on the engine's stream without waiting (the inputs are
// copied before it returns; the outputs stay valid for compute_end). Work
// enqueued on that stream later runs after it. One pending computation per
// engine; compute_end waits for it and fills out[]. The pending state is
// opaque (Pending*); compute_end frees it.
struct Pending;
lcg_status compute_begin(lcg_engine eng, const Params &P, int npairs, const PairIn *in, PairOut *out,
                         Pending **pending, std::string &err);
lcg_status compute_end(lcg_engine eng, Pending *pending, std::string &err);

// Zero the engine's count of the bytes a table preparation copied (at the
// start of each lcg_prepare_pairs call; compute() adds to it).
void reset_transfer(lcg_engine eng);

}  // namespace lcg_env
