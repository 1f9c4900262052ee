/*
 * locarna_gb300 — C ABI of the GB300-native sparsified Sankoff (LocARNA)
 * alignment engine and the LocARNA-P partition-function engine.
 *
 * Plain pointers and sizes only; no exceptions cross this boundary. Every
 * entry point returns an lcg_status (0 = ok, < 0 = error) and, on error,
 * lcg_last_error() returns a thread-local message.
 *
 * The boundary sits where the reference's LocARNA::Aligner sits
 * (src/LocARNA/aligner.hh:67-189): the caller prepares the same tables the
 * reference's Scoring / ArcMatches / BasePairs / TraceController /
 * AnchorConstraints objects hold (src/LocARNA/scoring.hh:488-607,
 * arc_matches.hh:404-413, basepairs.hh:217-222, trace_controller.hh:122-139,
 * anchor_constraints.hh:157-215) and the engine runs Aligner::align() +
 * Aligner::trace() (aligner.cc:924-957, :1345-1358) on the GPU.
 *
 * Score semantics follow the reference's InftyInt (infty_int.hh:56-480):
 * an alignment score is a finite integer or negative infinity, reported as
 * LCG_NEG_INF.
 */
#ifndef LOCARNA_GB300_H
#define LOCARNA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LCG_ABI_VERSION 4

typedef int32_t lcg_status;
#define LCG_OK 0
#define LCG_ERR_ARG (-1)       /* invalid argument (sizes, indices, NULL) */
#define LCG_ERR_CUDA (-2)      /* a CUDA runtime call failed */
#define LCG_ERR_NOMEM (-3)     /* device or host allocation failed */
#define LCG_ERR_RANGE (-4)     /* scores could overflow the int32 device range */
#define LCG_ERR_TIMEOUT (-5)   /* a bounded device wait gave up */
#define LCG_ERR_PARSE (-6)     /* malformed input file / text */
#define LCG_ERR_UNSUPPORTED (-7) /* option outside the implemented scope */
#define LCG_ERR_DEVICE (-8)    /* a kernel reported an internal error */

/* negative infinity as returned in lcg_align_result.score */
#define LCG_NEG_INF ((int64_t)(-((int64_t)1 << 40)))

/* free end gaps bits, same meaning as LocARNA::FreeEndgaps("abcd")
 * (free_endgaps.hh:27-71): character k == '+' sets bit k. */
#define LCG_FREE_LEFT_1 1   /* allow_left_1: free gaps at the start of B vs A */
#define LCG_FREE_RIGHT_1 2  /* allow_right_1 */
#define LCG_FREE_LEFT_2 4   /* allow_left_2 */
#define LCG_FREE_RIGHT_2 8  /* allow_right_2 */

/*
 * Prepared tables of one sequence pair (A of length len_a, B of length len_b).
 * Positions are 1-based as in the reference; index 0 of per-position arrays is
 * unused unless stated otherwise. All arrays are caller-owned host memory.
 */
typedef struct lcg_pair_tables {
    int32_t len_a, len_b;
    /* Scoring::basematch(i,j) = sigma[i*(len_b+1)+j]   (scoring.hh:489) */
    const int32_t *sigma;
    /* Scoring::gapA(i) / gapB(j)                        (scoring.hh:589-606) */
    const int32_t *gap_a; /* len_a+1 */
    const int32_t *gap_b; /* len_b+1 */
    int32_t indel_opening; /* Scoring::indel_opening() (scoring.hh:617) */
    int32_t exclusion;     /* Scoring::exclusion()     (scoring.hh:611) */
    /* arcs in the reference's arc index order (basepairs.cc:155-205):
     * arcs_x[2k] = left end, arcs_x[2k+1] = right end of arc k, with
     * right >= left + 3 as BasePairs makes them (others: LCG_ERR_ARG) */
    int32_t num_arcs_a, num_arcs_b;
    const int32_t *arcs_a;
    const int32_t *arcs_b;
    /* valid arc matches in the reference's index order (arc_matches.cc:159-184):
     * am_arcs[2k] = arc index in A, am_arcs[2k+1] = arc index in B,
     * am_score[k] = Scoring::arcmatch(am_k) (scoring.cc:440-554) */
    int32_t num_arcmatches;
    const int32_t *am_arcs;
    const int32_t *am_score;
    /* TraceController band: is_valid(i,j) iff min_col[i] <= j <= max_col[i],
     * i in 0..len_a (trace_controller.hh:328-336) */
    const int32_t *min_col; /* len_a+1 */
    const int32_t *max_col; /* len_a+1 */
    /* Anchor constraints as ranges (anchor_constraints.hh:157-253); all six
     * pointers NULL means "no anchors" (everything allowed).
     * allowed_match(i,j) iff match_lo[i] <= j <= match_hi[i]   (i 1..len_a)
     * allowed_del(i,j)   iff del_lo[i]   <= j <= del_hi[i]     (i 1..len_a)
     * allowed_ins(i,j)   iff ins_lo[j]   <= i <= ins_hi[j]     (j 1..len_b) */
    const int32_t *match_lo, *match_hi;
    const int32_t *del_lo, *del_hi;
    const int32_t *ins_lo, *ins_hi;
    /* rightmost_anchor() / leftmost_anchor() (anchor_constraints.hh:282-306);
     * without anchors (0,0) and (len_a+1,len_b+1) */
    int32_t right_anchor_a, right_anchor_b;
    int32_t left_anchor_a, left_anchor_b;
    /* Stacking (locarna --stacking / --new-stacking; Scoring::stacking(),
     * scoring.hh:653): both NULL = off. am_stack_score[k] =
     * Scoring::arcmatch(am_k, true) (scoring.cc:440-480), the score of am_k
     * stacked on its inner arc match; values <= LCG_STACK_NONE stand for
     * scores outside the int32 range, which the reference only produces from
     * zero stacking probabilities (undefined weights) and which never explain
     * an alignment. am_stackable[k] = Scoring::is_stackable_am(am_k)
     * (scoring.cc:567-569). Used by fill_D_entries (aligner.cc:600-608),
     * fill_D_entries_noLP (:629-650) and trace_arcmatch (:986-1006). */
    const int32_t *am_stack_score;
    const uint8_t *am_stackable;
} lcg_pair_tables;

#define LCG_STACK_NONE (-(1 << 29))

/* AlignerParams subset (aligner_params.hh:51-64) */
typedef struct lcg_align_opts {
    int32_t struct_local;  /* AlignerParams::struct_local */
    int32_t sequ_local;    /* AlignerParams::sequ_local */
    int32_t free_endgaps;  /* LCG_FREE_* bits */
    int32_t do_trace;      /* run Aligner::trace() after align() */
    /* AlignerParams::no_lonely_pairs (locarna --noLP): every arc match must
     * enclose an inner arc match (left ends +1, right ends -1); D is filled
     * by fill_D_entries_noLP (aligner.cc:612-657), groups are chosen by
     * get_max_right_ends(.., true) (arc_matches.cc:313-355) and the
     * traceback follows trace_arcmatch_noLP (aligner.cc:1030-1079). No
     * stacking terms. */
    int32_t no_lonely_pairs;
    /* locarna --normalized L (Aligner::normalized_align, aligner.cc:1521-1588):
     * sequence-local alignment maximising score / (length + L) by
     * Dinkelbach iterations over the top level with every position penalised
     * by the current ratio; the result score is that ratio (integer) and the
     * traceback the last iteration's. Needs sequ_local, not struct_local. */
    int32_t normalized;
    int32_t normalized_L;
    /* locarna --penalized PP (Aligner::penalized_align, aligner.cc:1590-1617):
     * the top level with every position penalised by PP; the result score is
     * the penalised score. Not with normalized. */
    int32_t penalized;
    int32_t position_penalty;
} lcg_align_opts;

/*
 * Result of one pair. The caller provides the edge and arc-match buffers:
 * edges needs capacity 2*(len_a+len_b) int32, traced_am needs capacity
 * min(len_a,len_b) int32 (either may be NULL when do_trace == 0).
 *
 * edges holds the raw traceback edges in the order the reference appends them
 * (Alignment::append, alignment.cc:91-95): pairs (pos_a, pos_b) with -1 for a
 * gap. traced_am lists the arc matches of the traced alignment (reference arc
 * match indices) in the order the reference's trace visits them; their arcs
 * give the structure strings (Alignment::add_basepairA/B).
 */
typedef struct lcg_align_result {
    int64_t score;               /* Aligner::align(); LCG_NEG_INF for -inf */
    int32_t max_i, max_j;        /* end of the (local) alignment */
    int32_t min_i, min_j;        /* start of a sequence-local alignment */
    int32_t num_edges;           /* number of (pos_a,pos_b) pairs in edges */
    int32_t num_traced_am;
    int32_t *edges;
    int32_t *traced_am;
} lcg_align_result;

/* Work counts of one pair, over the reference's iteration space. */
typedef struct lcg_work_counts {
    int64_t groups;          /* left-end groups (al,bl) aligned in align_D */
    int64_t cells;           /* M cells evaluated (groups + top level), state NO_NO */
    int64_t arc_terms;       /* arc-pair candidates evaluated in align_noex */
    int64_t valid_arc_terms; /* of those, valid arc matches (finite or not) */
} lcg_work_counts;

/* ---------------------------------------------------------------- engine */

typedef struct lcg_engine_s *lcg_engine;

/* Message of the last failed call on this thread ("" if none). */
const char *lcg_last_error(void);

/* ABI version (LCG_ABI_VERSION). */
int32_t lcg_abi_version(void);

/* Create an engine on CUDA device `device`, launching on `stream`
 * (a cudaStream_t, or NULL for a stream the engine creates). The engine owns
 * its device buffers; one engine per host thread. */
lcg_status lcg_engine_create(int32_t device, void *stream, lcg_engine *out);
lcg_status lcg_engine_destroy(lcg_engine eng);

/*
 * Align `npairs` independent pairs: the batched equivalent of constructing one
 * LocARNA::Aligner per pair and calling align() (+ trace()) on each
 * (reference: src/locarna.cc:727-785, aligner.cc:924-957,1345-1358).
 * Host tables in, host results out; all device traffic is inside the call.
 * Large batches run as a pipeline of chunks of pairs on two streams: the host
 * prepares chunk k+1 while the device aligns chunk k (see
 * lcg_engine_set_chunk_pairs).
 */
lcg_status lcg_align_pairs(lcg_engine eng, const lcg_pair_tables *pairs,
                           int32_t npairs, const lcg_align_opts *opts,
                           lcg_align_result *results);

/*
 * The k best alignments of each pair by interval splitting (locarna --kbest k
 * --better t; Aligner::suboptimal, aligner.cc:1384-1512): the best
 * alignment, then repeatedly the best remaining task of a queue of
 * (interval, score), whose alignment is a hit and whose interval is split in
 * the middle of that alignment along the longer sequence into two new tasks.
 * Ends after k hits, when the best task scores below threshold + 1 or is -inf,
 * or when the queue is empty (where the reference's behaviour is undefined).
 * Empty alignments are not hits. results[q*k + h] (h < num_hits[q]) is hit h
 * of pair q, its score the task's score; each needs edge and arc-match
 * buffers as in lcg_align_pairs. With opts->normalized every interval is
 * scored by normalized alignment (as suboptimal(.., normalized = true, L));
 * opts->penalized must be 0; opts->do_trace is ignored (hits are always
 * traced).
 */
lcg_status lcg_align_kbest(lcg_engine eng, const lcg_pair_tables *pairs, int32_t npairs,
                           const lcg_align_opts *opts, int32_t k, int64_t threshold,
                           lcg_align_result *results, int32_t *num_hits);

/* Pairs per chunk of lcg_align_pairs' pipeline: 0 (default) chooses by batch
 * size (one chunk below 256 pairs, else up to 8 chunks); n > 0 caps a chunk
 * at n pairs (n >= npairs: one chunk, one fill and one traceback launch). */
lcg_status lcg_engine_set_chunk_pairs(lcg_engine eng, int32_t pairs_per_chunk);

/* CUDA graphs (default on): lcg_align_pairs records each chunk's device work
 * (host->device copy, clearing, fill kernel, traceback kernel, device->host
 * copies) from its stream into a CUDA graph and launches the graph; a chunk
 * whose launch parameters (buffers, sizes, grid) equal the previous chunk's
 * on the same buffer set replays it without capturing again. Normalized,
 * penalized and k-best alignment, whose top levels iterate with the host,
 * launch directly. on = 0 launches every chunk directly. */
lcg_status lcg_engine_set_graphs(lcg_engine eng, int32_t on);
/* Kept group rectangles: when a chunk's left-end groups, stored as full
 * rectangles ((ar-al) x (br-bl) cells each; 4 bytes per cell, 32 with
 * --struct-local, whose traceback switches between the eight state
 * matrices), fit in `bytes`, the fill writes every group's matrices to a
 * rectangle of its own and the traceback walks each traced arc match on its
 * group's rectangle instead of recomputing it (the reference recomputes too,
 * trace_arcmatch, aligner.cc:967-1028); the results are the same. Single
 * pairs and small batches; not with --noLP. bytes = 0 always recomputes;
 * bytes < 0 restores the default budgets, 4 GiB for plain chunks and 32 GiB
 * for structure-local chunks (a 400 x 400 nt pair takes ~25 GB).
 * LocARNA-P (lcg_pf_forward / lcg_pf_backward) keeps the groups' M (and E, F
 * for the gap gradients) from the forward for the backward pass under the
 * same budget, by default in FP64 only (4 GiB; in FP32 the backward's
 * recomputation is faster than reading the kept values back). */
lcg_status lcg_engine_set_rect_budget(lcg_engine eng, int64_t bytes);
/* Graph captures and replays of the last lcg_align_pairs call. */
lcg_status lcg_engine_last_graphs(lcg_engine eng, int64_t *captures, int64_t *replays);

/* ------------------------------------------------------------- autotuner
 *
 * The fill kernel's launch configuration chosen per length bucket by
 * measurement: for the pairs of each bucket (by max(len_a, len_b): <= 128,
 * <= 224, <= 320, longer) a sample is aligned under every configuration of a
 * grid (resident blocks per SM of the persistent fill kernel, i.e. warps
 * per SM; L2 budget of a pair wave of its work queue, i.e. how many pairs'
 * tables are interleaved at a time) and the fastest fill is kept. With
 * autotune on, lcg_align_pairs orders a batch by bucket, forms its chunks
 * within buckets and launches each chunk with its bucket's configuration;
 * results come back in input order and are the same as without. The
 * reference has no counterpart (its all-pairs driver mlocarna runs one
 * locarna process per pair, lib/perl/MLocarna/threaded.pm:28-65). */
#define LCG_TUNE_BUCKETS 4
typedef struct lcg_tune_entry {
    int32_t max_len;        /* bucket: pairs with max(len_a, len_b) <= max_len (last: any) */
    int32_t pairs_sampled;  /* 0: no pair of the batch in this bucket (defaults kept) */
    int32_t blocks_per_sm;  /* chosen (0 = as many as fit) */
    double wave_mb;         /* chosen (0 = default 8 MB) */
    double best_ms;         /* fill time of the sample under the chosen configuration */
    double default_ms;      /* fill time of the sample under the default configuration */
    int32_t trials;         /* configurations measured */
} lcg_tune_entry;
/* Measure and store the configuration of every bucket present in the batch
 * (sample_pairs: pairs per bucket, 0 = 64); report[LCG_TUNE_BUCKETS] may be
 * NULL. Uses opts' mode; opts->do_trace is ignored (fill only). */
lcg_status lcg_engine_autotune(lcg_engine eng, const lcg_pair_tables *pairs, int32_t npairs,
                               const lcg_align_opts *opts, int32_t sample_pairs, lcg_tune_entry *report);
/* Use the stored configurations in lcg_align_pairs (on = 1) or not (0). */
lcg_status lcg_engine_set_autotune(lcg_engine eng, int32_t on);

/* Device time (ms) of the last lcg_align_pairs call's kernels (summed over its
 * chunks, whose kernels may overlap on the two streams), and the number of
 * kernel launches it made. */
lcg_status lcg_engine_last_stats(lcg_engine eng, double *kernel_ms,
                                 int64_t *launches);

/* Device time (ms) of the last call's D-fill kernels and traceback kernels
 * (summed over chunks). */
lcg_status lcg_engine_last_timing(lcg_engine eng, double *fill_ms, double *trace_ms);

/* Wall-clock phases (ms) of the last lcg_align_pairs call: host preparation of
 * the pairs' index structures, packing of the upload, time the host waited for
 * copies + kernels, and assembly of the alignments (summed over chunks; with
 * several chunks the device works during the host phases). For
 * lcg_align_pp_pairs the host preparation also counts the staging of the
 * inputs (parsing, bands, the first chunk's envelopes) and every chunk's
 * tables. */
lcg_status lcg_engine_last_phases(lcg_engine eng, double *prep_ms, double *pack_ms,
                                  double *device_ms, double *results_ms);

/* Bytes the last lcg_align_pairs call copied host->device and device->host. */
lcg_status lcg_engine_last_transfer(lcg_engine eng, int64_t *h2d_bytes,
                                    int64_t *d2h_bytes);

/* Work counts of the last call (all pairs): groups and cells always; with
 * counting on, arc_terms = candidate list entries visited and
 * valid_arc_terms = arc-match terms evaluated (else -1). Counting makes the
 * fill kernel slower: use it for measurement runs only. */
lcg_status lcg_engine_set_counting(lcg_engine eng, int32_t on);
lcg_status lcg_engine_last_work(lcg_engine eng, lcg_work_counts *out);

/* Work of one pair before it is aligned, on the host (no GPU): the left-end
 * groups of align_D (aligner.cc:660-732) and the M cells of their rectangles
 * plus the top level, as lcg_engine_last_work counts them; arc_terms = the
 * arc matches whose right ends are band cells (the D entries);
 * valid_arc_terms = -1. Validates the tables like lcg_align_pairs. The
 * estimate by which a batch is split across GPUs (the reference's mlocarna
 * splits its pair list over processes, src/Utils/mlocarna:3547-3625). */
lcg_status lcg_pair_work(const lcg_pair_tables *pair, const lcg_align_opts *opts,
                         lcg_work_counts *out);


/* --------------------------------------------- LocARNA-P forward/backward
 *
 * The partition-function aligner LocARNA::AlignerP<T> (aligner_p.hh:53-622,
 * driven by src/locarna_p.cc:466-531) as a forward/backward pair:
 *   forward  = AlignerP::align_inside() (aligner_p.icc:413-438): log Z;
 *   backward = the adjoint of the inside recursion, which yields what
 *              align_outside() + compute_arcmatch_probabilities() +
 *              compute_basematch_probabilities() (aligner_p.icc:1113-1399)
 *              yield, and the derivatives of log Z with respect to the
 *              scoring parameters, in one pass.
 * Global mode without anchors (the reference's AlignerP supports no other).
 * The Boltzmann weights are exp(score / temperature) (scoring.hh:857-860)
 * from the same integer tables lcg_align_pairs takes. precision 64 runs
 * the recursions in double; precision 32 runs them in float with a
 * per-position scale factor chosen on the host, accumulating log Z, the
 * expected counts and the normalisation in double.
 */
typedef struct lcg_pf_opts {
    double temperature; /* --temperature-alipf (300) */
    double pf_scale;    /* AlignerPParams::pf_scale (1): arc terms times pf_scale, D divided */
    int32_t precision;  /* 64 or 32 */
    /* Continuous offsets of the scoring parameters the gradients are taken
     * with respect to (all 0 = the integer tables as given): [0] indel (added
     * to gap_a, gap_b), [1] indel_opening, [2] struct_weight (arc-match score
     * plus delta * am_dscore_dsw), [3 + 4x + y] base-match score S[x][y]
     * (sigma(i,j) plus delta where code_a[i] = x, code_b[j] = y). Offsets
     * [2..18] need the grad specs of lcg_pf_forward. */
    double param_delta[19];
    /* AlignerPParams::min_am_prob / min_bm_prob (aligner_params.hh:122-156;
     * locarna_p --min-am-prob / --min-bm-prob, default 0.001 each). With
     * min_am_prob > 0, bm_prob is what compute_basematch_probabilities
     * (aligner_p.icc:1201-1327) reports: the contributions of base matches
     * inside arc matches of probability <= sqrt(min_am_prob) are left out.
     * min_am_prob = 0 gives the exact base-match marginals. am_prob, log Z
     * and the gradients do not depend on either; min_bm_prob / min_am_prob
     * are also the thresholds of the probability writers (aligner_p.icc:
     * 1404-1435), which the caller applies. */
    double min_am_prob;
    double min_bm_prob;
    /* 1 (default): lcg_pf_backward also returns the gap counts and
     * d log Z / d indel, indel_opening; 0: probabilities (and the struct-weight
     * and base-match gradients) only, and those four results are NaN. The
     * gap counts need the E and F matrices, which the backward pass then
     * keeps and reads besides M; locarna_p prints probabilities only. */
    int32_t gap_gradients;
} lcg_pf_opts;

/* Per pair input of the parameter gradients (all optional, see below). */
typedef struct lcg_pf_grad_spec {
    const int8_t *code_a; /* [len_a+1]; code_a[i] in 0..3 for A,C,G,U of position i, -1 otherwise */
    const int8_t *code_b; /* [len_b+1] */
    const double *am_dscore_dsw; /* [num_arcmatches]: d arc-match score / d struct_weight */
} lcg_pf_grad_spec;

typedef struct lcg_pf_result {
    /* caller-owned outputs, NULL = not wanted */
    double *am_prob; /* [num_arcmatches] arc-match probabilities (compute_arcmatch_probabilities) */
    double *bm_prob; /* [(len_a+1)*(len_b+1)] base-match probabilities, arc-match ends not included */
    /* filled by lcg_pf_backward */
    double log_z;
    double gap_ext_uses;  /* expected number of gapped positions (uses of gap_a / gap_b) */
    double gap_open_uses; /* expected number of gap openings (uses of indel_opening) */
    /* d log Z / d parameter: indel (gap_a[i] = gap_b[j] = indel), indel_opening
     * unless lcg_pf_opts.gap_gradients = 0 (then NaN, as the two gap counts);
     * struct_weight and the 16 base-match scores (sigma(i,j) =
     * S[code_a[i]][code_b[j]], index 4*x+y) when a grad spec is given */
    double dlogz_dindel;
    double dlogz_dindel_opening;
    double dlogz_dstruct_weight;
    double dlogz_dbasematch[16];
} lcg_pf_result;

void lcg_pf_opts_default(lcg_pf_opts *opts);

/* log Z of `npairs` pairs in one batched launch. specs: NULL or [npairs]
 * (needed for nonzero param_delta[2..18]). The engine keeps the state the
 * backward pass needs until the next lcg_pf_forward or lcg_pf_backward. */
lcg_status lcg_pf_forward(lcg_engine eng, const lcg_pair_tables *pairs, int32_t npairs,
                          const lcg_pf_opts *opts, const lcg_pf_grad_spec *specs,
                          double *log_z);

/* Backward pass of the last lcg_pf_forward: results[npairs]; specs NULL or
 * [npairs] (entries with NULL members skip those gradients). */
lcg_status lcg_pf_backward(lcg_engine eng, const lcg_pf_grad_spec *specs,
                           lcg_pf_result *results);

/* Device time (ms) of the last forward and backward kernels. */
lcg_status lcg_pf_last_timing(lcg_engine eng, double *forward_ms, double *backward_ms);

/* -------------------------------------------- allocation-free entry point
 *
 * No counterpart in the reference: an addition of this library for callers
 * that cannot allocate device memory while they run (a service whose GPU
 * memory is reserved up front by another framework's allocator, a real-time
 * loop where cudaMalloc / cudaFree would synchronise the device). It computes
 * what lcg_align_pairs computes without traceback (the score and the end cell
 * of one pair: global, sequence-local, free end gaps, --noLP, stacking,
 * anchor constraints) and takes every device byte from one fixed file-scope
 * device array of LCG_STATIC_SCRATCH_BYTES held per GPU for the life of the
 * process; it calls no cudaMalloc, cudaFree, cudaMallocHost or other
 * allocating CUDA routine. Pairs whose data do not fit are rejected with
 * LCG_ERR_RANGE (about 400 x 400 nt with the default envelope is beyond the
 * limit). All calls share the array: calls whose GPU work overlaps race on it.
 * The first call on a device looks the array's address up
 * (cudaGetSymbolAddress).
 * opts->struct_local and opts->do_trace must be 0. stream is a cudaStream_t
 * (NULL = default stream); the call returns when its results are on the host.
 */
#define LCG_STATIC_SCRATCH_BYTES (64u << 20)
lcg_status lcg_align_score_static(const lcg_pair_tables *pair, const lcg_align_opts *opts,
                                  int64_t *score, int32_t *max_i, int32_t *max_j,
                                  void *stream);

/* ------------------------------------------------------ host preparation
 *
 * Builds lcg_pair_tables from two PP 2.0 inputs the way the reference's
 * locarna driver builds its Scoring / ArcMatches / TraceController objects
 * (src/locarna.cc:398-703): PP reading (rna_data.cc:979-1104), arcs
 * (basepairs.cc:155-205), sigma / gap / arc weights / arc-match scores
 * (scoring.cc:28-554, RIBOSUM85_60 built in), the max-diff band
 * (trace_controller.cc:360-390) and the sequence envelope
 * (edge_probs.icc:7-268, trace_controller.cc:565-597). Sequences or
 * profiles (alignment rows); #A anchor lines as strict anchor constraints
 * (anchor_constraints.cc:10-395, trace_controller.cc:542-563).
 */
typedef struct lcg_prep_opts {
    double min_prob;              /* --min-prob (0.001) */
    int32_t indel;                /* --indel (-150) */
    int32_t indel_opening;        /* --indel-opening (-750) */
    int32_t struct_weight;        /* --struct-weight (200) */
    int32_t tau;                  /* --tau (50) */
    int32_t exclusion;            /* --exclusion (0) */
    int32_t match, mismatch;      /* --match (50) / --mismatch (0) */
    int32_t use_ribosum;          /* --use-ribosum (1) */
    double min_trace_probability; /* --min-trace-probability (1e-4) */
    int32_t max_diff;             /* --max-diff (-1) */
    int32_t max_diff_am;          /* --max-diff-am (-1) */
    int32_t max_diff_at_am;       /* --max-diff-at-am (-1) */
    int32_t temperature_alipf;    /* --temperature-alipf (300) */
    int32_t sequ_local;           /* --sequ-local: local envelope */
    int32_t free_endgaps;         /* LCG_FREE_* bits for the envelope */
    int32_t pf_precision;         /* envelope float type: 0 double, 1 long double (locarna's default) */
    double exp_prob;              /* --exp-prob; <= 0 means 1/(2 len) per sequence */
    /* --stacking (needs --exp-prob, else off as in src/locarna.cc:407-414)
     * and --new-stacking: read the joint probabilities of the PP input's
     * #STACK section and fill lcg_pair_tables.am_stack_score/am_stackable */
    int32_t stacking;
    int32_t new_stacking;
    /* --relaxed-anchors: anchor names need not be ordered (relaxed
     * AnchorConstraints, anchor_constraints.cc:322-357) */
    int32_t relaxed_anchors;
    /* --unpaired-penalty (0): subtracted from every gap cost and twice from
     * every base-match score, before the arc-match scores read them
     * (Scoring::apply_unpaired_penalty, scoring.cc:65-74) */
    int32_t unpaired_penalty;
} lcg_prep_opts;

typedef struct lcg_prepared_s *lcg_prepared;

/* Defaults of the locarna command line (src/locarna.cc:83-272). */
void lcg_prep_opts_default(lcg_prep_opts *opts);

/* Parse two PP 2.0 texts and build the pair's tables (opts NULL = defaults). */
lcg_status lcg_prepare_pair(const char *pp_a, const char *pp_b, const lcg_prep_opts *opts,
                            lcg_prepared *out);

/* Batched lcg_prepare_pair: the tables of npairs pairs (pp_a[q], pp_b[q]),
 * identical to lcg_prepare_pair's, with the sequence envelope of all pairs
 * computed on the engine's GPU (PFGotoh / PFTraceProbs, edge_probs.icc:76-268,
 * in FP64 with per-row power-of-two scaling). A pair whose edge probability
 * lies within 1e-7 relative of min_trace_probability where it could move a
 * band row, or whose values would leave the range of the reference's float
 * type (or whose lengths sum above 1000 for double, 16000 for long double),
 * gets its envelope from the host path in the reference's precision; their
 * number goes to *host_envelopes (may be NULL). Parsing and table building
 * run on the host threads. out[q] are freed with lcg_prepared_free. */
lcg_status lcg_prepare_pairs(lcg_engine eng, const char *const *pp_a, const char *const *pp_b,
                             int32_t npairs, const lcg_prep_opts *opts, lcg_prepared *out,
                             int32_t *host_envelopes);
/* PP texts in, alignments out: lcg_prepare_pairs + lcg_align_pairs as one
 * pipeline. The inputs, bands and sequence envelopes of all pairs are
 * computed first (the envelopes in one GPU launch); then, chunk by chunk of
 * lcg_align_pairs' pipeline, the host builds a chunk's tables while the
 * device aligns the previous chunk. results[q] as for lcg_align_pairs, with
 * edge buffers for the PP sequences' lengths (2 (len_a + len_b) int32) and
 * traced_am buffers of min(len_a, len_b) int32. This is what the locarna
 * command line does per pair (src/locarna.cc:398-785), for a batch. */
lcg_status lcg_align_pp_pairs(lcg_engine eng, const char *const *pp_a, const char *const *pp_b, int32_t npairs,
                              const lcg_prep_opts *prep_opts, const lcg_align_opts *opts,
                              lcg_align_result *results, int32_t *host_envelopes);
/* Views into the prepared tables; valid until lcg_prepared_free. */
lcg_status lcg_prepared_tables(lcg_prepared p, lcg_pair_tables *out);
/* which: 0 sequence A, 1 sequence B, 2 name A, 3 name B */
const char *lcg_prepared_sequence(lcg_prepared p, int32_t which);
/* Rows of the inputs (a profile input is an alignment of several rows; a
 * single sequence has one), as the reference's MultipleAlignment of the PP
 * sequence section holds them (multiple_alignment.cc:577-584: upper case,
 * T as U): which = 0 row k of A, 1 row k of B, 2 name of row k of A, 3 name of
 * row k of B, 4 anchor line k+1 of A (its #A<k+1> lines concatenated,
 * multiple_alignment.cc:324-346), 5 anchor line k+1 of B; NULL past the last
 * row. Valid until lcg_prepared_free. */
const char *lcg_prepared_row(lcg_prepared p, int32_t which, int32_t k);
/* 0 if the envelope partition function failed (PFGotoh::fail, edge_probs.hh:202) */
int32_t lcg_prepared_envelope_ok(lcg_prepared p);
/* Gradient inputs of the prepared pair for lcg_pf_backward: base codes and
 * d am_score / d struct_weight of the unrounded arc weights,
 * (1 - ln p_a / ln pe_A) + (1 - ln p_b / ln pe_B) (scoring.cc:250-265);
 * views valid until lcg_prepared_free. */
lcg_status lcg_prepared_grad_spec(lcg_prepared p, lcg_pf_grad_spec *out);
lcg_status lcg_prepared_free(lcg_prepared p);

#ifdef __cplusplus
}
#endif
#endif /* LOCARNA_GB300_H */
