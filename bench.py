#!/usr/bin/env python3
"""Benchmark of the GB300 sparsified Sankoff engine.

Workload (one "step"): all-pairs structural alignment of 64 synthetic RNAs with
lengths uniform in [60, 400] nt = 2,016 pairs, locarna default scoring and
flags (global, RIBOSUM85_60, envelope 1e-4), bit-exact scores + traceback.
Inputs are seeded synthetic PP data (locarna_gb300/synth.py) with the shapes of
the all-pairs workload; there is no public dataset involved.

Metric: aligns/s (pairs aligned per second, whole job).
  value : pairs / device time of the kernels (inputs resident in HBM)
  e2e   : pairs / wall time of the public C-ABI pipeline from PP texts to
          alignments, as the locarna command line runs it: lcg_prepare_pairs
          (parsing, scoring, arc matches, envelopes on the GPU) and
          lcg_align_pairs (all copies inside)

With N > 1 ranks (torchrun) the 2,016 pairs are split by estimated work
(LPT over the host's cell counts, locarna_gb300/shard.py), every rank aligns
its shard on its own GPU with no exchange, and value = 2,016 / the slowest
rank's time.

--impl reference times the CPU port of the reference's locarna pipeline
(oracle/port_locarna: the host table preparation and the plain-C restatement
of the reference's Aligner; the reference's own sources are not available
where the bench runs, oracle/calibrate_port.py relates the two rates) from
PP files, one process per pair over a pool of one worker per host core, as
mlocarna runs locarna, on a bounded sample of the workload per step.
"""
import argparse
import json
import multiprocessing as mp
import os
import random
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = dict(count=64, len_lo=60, len_hi=400, seed=2024, q=0.05)
WORKLOAD_NAME = "sankoff_allpairs_64rnas_60-400nt_global"
PER_PAIR = dict(len_a=400, seed_a=3, len_b=400, seed_b=4)
CPU_SAMPLE_SECONDS = 20.0
# LocARNA-P: all pairs of 128 RNAs of 80-500 nt, inside + adjoint outside, in
# launches grouped by pair size (buckets of PF_BUCKET pairs)
PF_WORKLOAD = dict(count=128, len_lo=80, len_hi=500, seed=2025, q=0.05)
PF_WORKLOAD_NAME = "locarna_p_allpairs_128rnas_80-500nt"
PF_BUCKET = 1024
PF_FP64_STRIDE = 8  # FP64 (and the FP32 error) on every 8th pair of each launch
PF_CPU_SECONDS = 20.0
REF_PAIRS_PER_CORE = 4  # pairs per host core in one step of the reference arm
# DRAM traffic of the fill kernel per M cell, from the ncu capture of the
# 496-pair case (profiles/sankoff_fill_small_496pairs.md: dram read + write
# bytes of one launch / the launch's cells); the traffic of a launch of the
# workload is this times its cells
FILL_DRAM_BYTES_PER_CELL = (1.598e9 + 3.921e9) / 1.2018e9


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def int_peak_gops(dpx, device=0):
    """The measured int32 add+max rate (G ops/s) from the probe library."""
    import ctypes as C

    from locarna_gb300.build import build_probe
    lib = C.CDLL(build_probe())
    lib.lcg_probe_int_peak.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_double)]
    lib.lcg_probe_int_peak.restype = C.c_int
    g = C.c_double()
    rc = lib.lcg_probe_int_peak(device, int(bool(dpx)), C.byref(g))
    if rc != 0:
        raise RuntimeError(f"int32 rate probe failed (cuda error {rc})")
    return g.value


def workload_pp(families=1):
    """PP texts of the all-pairs workload and its pairs (index pairs). With
    families = N (N GPUs), N families of 64 RNAs (seeds 2024, 2025, ...),
    all pairs within each family: N x 2,016 pairs."""
    from locarna_gb300.synth import make_family
    pp, pairs = [], []
    for f in range(families):
        fam = make_family(WORKLOAD["count"], WORKLOAD["len_lo"], WORKLOAD["len_hi"], WORKLOAD["seed"] + f,
                          q=WORKLOAD["q"])
        base = len(pp)
        pp += [r.to_pp() for r in fam]
        pairs += [(base + a, base + b) for a in range(len(fam)) for b in range(a + 1, len(fam))]
    return pp, pairs


def build_tables(threads=None, families=1):
    """Tables of the workload from the host path (lcg_prepare_pair on every
    host thread; the envelope in long double as locarna computes it)."""
    from concurrent.futures import ThreadPoolExecutor

    from locarna_gb300.prep import prepare_pair
    pp, pairs = workload_pp(families)
    threads = threads or os.cpu_count() or 4
    with ThreadPoolExecutor(threads) as ex:
        tables = list(ex.map(lambda ab: prepare_pair(pp[ab[0]], pp[ab[1]]), pairs))
    return tables, pairs


def table_prep_gpu(eng, host_tables, host_s):
    """The same tables through lcg_prepare_pairs (envelopes on the GPU),
    timed once and checked against the host path's tables."""
    import numpy as np

    from locarna_gb300.prep import prepare_pairs
    pp, pairs = workload_pp()
    pp_pairs = [(pp[a], pp[b]) for a, b in pairs]
    prepare_pairs(eng, pp_pairs[:64])  # first-call set-up outside the timing
    t0 = time.perf_counter()
    tables, nhost = prepare_pairs(eng, pp_pairs)
    gpu_s = time.perf_counter() - t0
    for k, (t, r) in enumerate(zip(tables, host_tables)):
        for f in ("min_col", "max_col", "am_arcs", "am_score", "sigma"):
            if not np.array_equal(getattr(t, f), getattr(r, f)):
                raise RuntimeError(f"pair {k}: lcg_prepare_pairs {f} differs from lcg_prepare_pair")
    return {"pairs": len(pairs), "host_s": host_s, "host_threads": os.cpu_count() or 1,
            "gpu_envelope_s": gpu_s, "host_envelopes": nhost, "speedup": host_s / gpu_s,
            "what": "PP texts -> lcg_pair_tables (parsing, arcs, scoring, envelope 1e-4, arc matches): "
                    "lcg_prepare_pair on every host thread vs lcg_prepare_pairs (envelopes on the GPU)"}


def build_pf_tables(threads=None):
    """Tables of the LocARNA-P workload, prepared as locarna_p prepares them
    (envelope 1e-5 in double precision, src/locarna_p.cc defaults)."""
    from concurrent.futures import ThreadPoolExecutor

    from locarna_gb300.prep import prepare_pair
    from locarna_gb300.synth import make_family
    W = PF_WORKLOAD
    fam = make_family(W["count"], W["len_lo"], W["len_hi"], W["seed"], q=W["q"])
    pp = [r.to_pp() for r in fam]
    pairs = [(a, b) for a in range(len(fam)) for b in range(a + 1, len(fam))]
    threads = threads or os.cpu_count() or 4
    with ThreadPoolExecutor(threads) as ex:
        tables = list(ex.map(lambda ab: prepare_pair(pp[ab[0]], pp[ab[1]], min_trace_probability=1e-5,
                                                     pf_precision=0), pairs))
    return tables


def per_pair_tables():
    from locarna_gb300.prep import prepare_pair
    from locarna_gb300.synth import make_rna
    a = make_rna(PER_PAIR["len_a"], PER_PAIR["seed_a"])
    b = make_rna(PER_PAIR["len_b"], PER_PAIR["seed_b"])
    return prepare_pair(a.to_pp(), b.to_pp())


# ---------------------------------------------------------------- CPU side

_CPU_TABLES = None  # inherited by forked workers (the pool starts before any GPU call)


def _cpu_worker(args):
    idx, budget = args
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle_ffi import oracle_align
    t0 = time.perf_counter()
    done = 0
    for k in idx:
        if time.perf_counter() - t0 >= budget:
            break
        oracle_align(_CPU_TABLES[k])
        done += 1
    return done, time.perf_counter() - t0


def _cpu_pf_worker(args):
    idx, budget = args
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle_ffi import oracle_pf
    t0 = time.perf_counter()
    done = 0
    for k in idx:
        if time.perf_counter() - t0 >= budget:
            break
        oracle_pf(_CPU_TABLES[k])
        done += 1
    return done, time.perf_counter() - t0


def cpu_sample(tables, budget_s, cores, seed=7, worker=None):
    """Time-bounded CPU sample of the workload: a seeded permutation of the
    pairs dealt round-robin to one forked process per core; each process
    aligns its pairs until budget_s is spent. Returns (pairs, aligns/s)."""
    import random
    global _CPU_TABLES
    _CPU_TABLES = tables
    order = list(range(len(tables)))
    random.Random(seed).shuffle(order)
    lists = [order[c::cores] for c in range(cores)]
    ctx = mp.get_context("fork")
    with ctx.Pool(cores) as pool:
        res = pool.map(worker or _cpu_worker, [(lst, budget_s) for lst in lists])
    done = sum(d for d, _ in res)
    rate = sum(d / t for d, t in res if t > 0)
    return done, rate


def write_pp_files(pp, d):
    paths = []
    for k, text in enumerate(pp):
        path = os.path.join(d, f"r{k}.pp")
        with open(path, "w") as f:
            f.write(text)
        paths.append(path)
    return paths


def port_run(paths, pairs, sample, cores):
    """The CPU port of `locarna A.pp B.pp` (oracle/_build/port_locarna) on
    pairs[sample], one process per pair, `cores` processes at a time (as
    mlocarna runs locarna). Returns (pairs done, wall seconds, scores)."""
    from concurrent.futures import ThreadPoolExecutor
    port = os.path.join(ROOT, "oracle", "_build", "port_locarna")

    def one(k):
        a, b = pairs[k]
        r = subprocess.run([port], input=f"{paths[a]} {paths[b]}\n", capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"port_locarna failed on pair {k}: {r.stderr.strip()}")
        return int(r.stdout.split()[0])

    t0 = time.perf_counter()
    with ThreadPoolExecutor(cores) as ex:
        scores = list(ex.map(one, sample))
    return len(sample), time.perf_counter() - t0, scores


def port_baseline(pp, pairs, cores, budget_s, seed=7):
    """Time-bounded CPU baseline: the port on seeded random pairs of the
    workload, batches of REF_PAIRS_PER_CORE x cores pairs (the reference
    arm's step, so that a long pair does not idle the other cores at every
    few pairs) until budget_s is spent."""
    rng = random.Random(seed)
    order = list(range(len(pairs)))
    rng.shuffle(order)
    done, wall = 0, 0.0
    step = REF_PAIRS_PER_CORE * cores
    with tempfile.TemporaryDirectory(prefix="lcg_pp_") as d:
        paths = write_pp_files(pp, d)
        for i in range(0, len(order), step):
            n, w, _ = port_run(paths, pairs, order[i:i + step], cores)
            done += n
            wall += w
            if wall >= budget_s:
                break
    return done, wall


# ---------------------------------------------------------------- clocks

class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region, written to
    LCG_CLOCK_LOG (default: a file in the temporary directory)."""

    def __init__(self):
        import tempfile
        self.proc = None
        self.path = os.environ.get("LCG_CLOCK_LOG") or os.path.join(tempfile.gettempdir(), "lcg_bench_clocks.csv")

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,"
                 "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sms, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sms.append(float(p[1]))
                mx = float(p[2])
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        sms.sort()
        return {"sm_mhz": sms[len(sms) // 2] if sms else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sms)}


# ---------------------------------------------------------------- LocARNA-P

MODES_SAMPLE = 256  # pairs of the workload (every 8th) for the alignment-mode lines


def run_modes(eng, tables, flush_l2):
    """Sequence-local alignment modes on a sample of the workload's pairs
    (every 8th of the 2,016): plain local, --normalized 100 (Dinkelbach
    iterations), --penalized 50 and --kbest 5; pairs per second of the public
    calls (wall, host tables in and results out) and their device time, each
    checked against the oracle on a few pairs."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from checks import assert_same_result
    from oracle_ffi import oracle_align, oracle_kbest
    sample = tables[::max(1, len(tables) // MODES_SAMPLE)][:MODES_SAMPLE]
    out = {"sample": f"{len(sample)} pairs (every {max(1, len(tables) // MODES_SAMPLE)}th of the workload)"}
    specs = [("local", dict(sequ_local=True)), ("normalized_100", dict(sequ_local=True, normalized=100)),
             ("penalized_50", dict(sequ_local=True, penalized=50))]
    # each line's call runs once untimed first (buffers sized for the sample:
    # a growing pinned staging buffer costs as much as the call itself)
    for name, kw in specs:
        eng.align_pairs(sample, **kw)
        flush_l2()
        t0 = time.perf_counter()
        res = eng.align_pairs(sample, **kw)
        wall = time.perf_counter() - t0
        dev_ms = eng.last_stats()[0]
        for k in range(0, len(sample), 64):
            assert_same_result(res[k], oracle_align(sample[k], **kw), f"{name} pair {k}")
        out[name] = {"pairs_per_s": len(sample) / wall, "device_ms": dev_ms, "launches": eng.last_stats()[1]}
    eng.align_kbest(sample, 5, sequ_local=True)
    flush_l2()
    t0 = time.perf_counter()
    hits = eng.align_kbest(sample, 5, sequ_local=True)
    wall = time.perf_counter() - t0
    for k in range(0, len(sample), 64):
        ref = oracle_kbest(sample[k], 5, sequ_local=True)
        assert len(ref) == len(hits[k])
        for a, b in zip(hits[k], ref):
            assert_same_result(a, b, f"kbest pair {k}")
    out["kbest_5"] = {"pairs_per_s": len(sample) / wall, "hits": sum(len(h) for h in hits),
                      "launches": eng.last_stats()[1]}
    return out


def run_pf(eng, tables, flush_l2, cpu):
    """LocARNA-P over the whole workload: all pairs in size order, in
    launches of PF_BUCKET pairs (length-grouped persistent launches), inside
    + adjoint outside in FP32 with per-position scaling, for what locarna_p
    reports (log Z, arc-match and base-match probabilities; no gap
    gradients); FP64 on every PF_FP64_STRIDE-th pair of each launch
    (size-stratified), and per pair of that subset the largest FP32 error of
    any arc-match or base-match probability against the FP64 run of the same
    kernels (exact marginals, min_am_prob 0); one 200-nt pair with every
    gradient."""
    import numpy as np
    order = sorted(range(len(tables)), key=lambda k: (tables[k].len_a * tables[k].len_b, k))
    buckets = [order[i:i + PF_BUCKET] for i in range(0, len(order), PF_BUCKET)]
    # both precisions on the same path: the backward recomputes the groups'
    # rectangles (the workload's launches exceed the kept-rectangle budget;
    # a smaller FP64 subset could otherwise keep them)
    eng.set_rect_budget(0)
    for prec in (64, 32):  # warm-up
        eng.pf_forward([tables[k] for k in buckets[0][:64]], precision=prec, min_am_prob=0.0, gap_gradients=False)
        eng.pf_backward(probs=False)
    dev = {64: 0.0, 32: 0.0}
    wall = {64: 0.0, 32: 0.0}
    n64 = 0
    err_am, err_bm, pair_err = 0.0, 0.0, []
    launches = 0
    for b in buckets:
        tb = [tables[k] for k in b]
        sub = list(range(0, len(b), PF_FP64_STRIDE))
        flush_l2()
        t0 = time.perf_counter()
        eng.pf_forward(tb, precision=32, min_am_prob=0.0, gap_gradients=False)
        r32 = eng.pf_backward(probs=True)
        wall[32] += time.perf_counter() - t0
        f, bw = eng.pf_last_timing()
        dev[32] += f + bw
        keep = {k: (r32[k]["am_prob"], r32[k]["bm_prob"]) for k in sub}
        del r32
        flush_l2()
        t0 = time.perf_counter()
        eng.pf_forward([tb[k] for k in sub], precision=64, min_am_prob=0.0, gap_gradients=False)
        r64 = eng.pf_backward(probs=True)
        wall[64] += time.perf_counter() - t0
        f, bw = eng.pf_last_timing()
        dev[64] += f + bw
        n64 += len(sub)
        launches += 4
        for k, r in zip(sub, r64):
            am32, bm32 = keep[k]
            ea = float(np.max(np.abs(r["am_prob"] - am32))) if r["am_prob"].size else 0.0
            eb = float(np.max(np.abs(r["bm_prob"] - bm32)))
            err_am, err_bm = max(err_am, ea), max(err_bm, eb)
            pair_err.append(max(ea, eb))
        del r64, keep
    n = len(tables)
    pair_err.sort()
    out = {
        "workload": PF_WORKLOAD_NAME, "workload_pairs": n,
        "fp32": {"pairs": n, "pairs_per_s": n / (dev[32] / 1e3), "device_ms": dev[32], "e2e_pairs_per_s": n / wall[32],
                 "what": "every pair of the workload, inside + adjoint outside (log Z, arc-match and base-match "
                         "probabilities, as locarna_p; no gap gradients), FP32 with per-position scaling"},
        "fp64": {"pairs": n64, "pairs_per_s": n64 / (dev[64] / 1e3), "device_ms": dev[64],
                 "e2e_pairs_per_s": n64 / wall[64],
                 "what": f"every {PF_FP64_STRIDE}th pair of each launch in size order (size-stratified)"},
        "buckets": len(buckets), "bucket_pairs": PF_BUCKET,
        "fp32_over_fp64_device": (n / dev[32]) / (n64 / dev[64]),
        "fp32_over_fp64_e2e": (n / wall[32]) / (n64 / wall[64]),
        "fp32_max_abs_err": {"am_prob": err_am, "bm_prob": err_bm, "pairs_checked": len(pair_err),
                             "pair_max_median": pair_err[len(pair_err) // 2], "pair_max_max": pair_err[-1],
                             "tolerance": 1e-5, "against": "FP64 run of the same kernels"},
        "gpu_launches": launches,
        "cpu_baseline": cpu,
    }
    # one pair of 200 nt: log Z and gradients, FP64 and FP32 with the
    # engine's defaults (in FP64 the forward keeps the groups' rectangles for
    # the backward)
    eng.set_rect_budget(-1)
    from locarna_gb300.prep import prepare_pair
    from locarna_gb300.synth import make_rna
    t = prepare_pair(make_rna(200, 11).to_pp(), make_rna(200, 12).to_pp(), min_trace_probability=1e-5,
                     pf_precision=0)
    one = {}
    for prec in (64, 32):
        for _ in range(3):
            eng.pf_forward([t], precision=prec)
            eng.pf_backward(probs=False)
        ms = []
        for _ in range(5):
            flush_l2()
            lz = eng.pf_forward([t], precision=prec)[0]
            r = eng.pf_backward(probs=False)[0]
            f, bw = eng.pf_last_timing()
            ms.append(f + bw)
        ms.sort()
        one[prec] = (lz, r, ms[len(ms) // 2])
    g64 = np.array([one[64][1][k] for k in ("dlogz_dindel", "dlogz_dindel_opening", "dlogz_dstruct_weight")]
                   + list(one[64][1]["dlogz_dbasematch"]))
    g32 = np.array([one[32][1][k] for k in ("dlogz_dindel", "dlogz_dindel_opening", "dlogz_dstruct_weight")]
                   + list(one[32][1]["dlogz_dbasematch"]))
    nz = np.abs(g64) > 0
    out["pair_200nt"] = {"fp64_ms": one[64][2], "fp32_ms": one[32][2], "log_z_fp64": one[64][0],
                         "log_z_fp32": one[32][0],
                         "grad_fp32_max_rel_err": float(np.max(np.abs(g32[nz] - g64[nz]) / np.abs(g64[nz])))}
    return out


# ---------------------------------------------------------------- arms

def dist_setup():
    """(rank, world, local_rank); initialises torch.distributed for N > 1."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    return rank, world, local


def barrier_sync(world):
    import torch
    torch.cuda.synchronize()
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        torch.cuda.synchronize()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch.distributed as dist
    vals = [None] * world
    dist.all_gather_object(vals, x)
    return max(vals)


def run_ours(args):
    import numpy as np
    from locarna_gb300.engine import Engine
    from locarna_gb300.shard import lpt_partition, pair_weights, shard_loads
    rank, world, local = dist_setup()
    lead = rank == 0
    extras = world == 1  # the secondary lines are measured at N = 1 only
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    # weak scaling: N families of the workload for N GPUs, LPT-sharded
    pp, pairs = workload_pp(world)
    t0 = time.time()
    all_tables, _ = build_tables(families=world)
    host_prep_s = time.time() - t0
    if lead:
        log(f"host preparation of {len(all_tables)} pairs: {host_prep_s:.1f} s")
    # the pairs of this rank: LPT shards by the host's cell counts
    weights = pair_weights(all_tables)
    shards = lpt_partition(weights, world)
    mine = shards[rank]
    tables = [all_tables[k] for k in mine]
    pp_pairs = [(pp[pairs[k][0]], pp[pairs[k][1]]) for k in mine]
    npairs_total = len(all_tables)
    npairs = len(tables)
    cores = os.cpu_count() or 1
    cpu_rate, cpu_done = None, 0
    pf_tables, pf_cpu = None, None
    if extras:
        # CPU baselines before the first GPU call (forked pools): the CPU
        # port of the locarna pipeline on a bounded sample
        cpu_done, cpu_wall = port_baseline(pp, pairs, cores, CPU_SAMPLE_SECONDS)
        cpu_rate = cpu_done / cpu_wall
        log(f"cpu baseline: {cpu_done} pairs, {cpu_rate:.2f} aligns/s on {cores} cores")
        if not args.no_pf:
            t0 = time.time()
            pf_tables = build_pf_tables()
            log(f"host preparation of {len(pf_tables)} LocARNA-P pairs: {time.time() - t0:.1f} s")
            pf_done, pf_rate = cpu_sample(pf_tables, PF_CPU_SECONDS, cores, seed=9, worker=_cpu_pf_worker)
            log(f"cpu baseline LocARNA-P: {pf_done} pairs, {pf_rate:.3f} pairs/s on {cores} cores")
            pf_cpu = {"value": pf_rate, "unit": "pairs/s", "cores": cores, "kind": "port",
                      "sample": f"{pf_done} of the {len(pf_tables)} pairs (seeded permutation), one process "
                                f"per core, {PF_CPU_SECONDS:.0f} s per process; the oracle restatement of "
                                f"AlignerP (inside, outside, arc-match and base-match probabilities)"}
    eng = Engine(local)
    table_prep = None
    if extras:
        table_prep = table_prep_gpu(eng, all_tables, host_prep_s)
        log(f"table preparation with GPU envelopes: {table_prep['gpu_envelope_s']:.2f} s "
            f"({table_prep['host_envelopes']} host envelopes)")
    call = eng.prepare_call(tables)

    # the autotuner on this workload (per length bucket, outside the timed
    # region), reported; the timed runs use the library's default launch (one
    # persistent fill over the whole batch), which the tuner finds as fast
    tune = eng.autotune(tables, sample_pairs=64) if extras else None
    # measurement-only runs (outside the timed region): work counts
    eng.set_counting(True)
    eng.run_call(call)
    work = eng.last_work()
    eng.set_counting(False)
    int_peak = max(int_peak_gops(False, local), int_peak_gops(True, local))

    # L2 flush buffer (larger than the 129 MB L2)
    import torch
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.int32, device=f"cuda:{local}")

    def flush_l2():
        flush.fill_(1)
        torch.cuda.synchronize()

    sampler = ClockSampler() if lead else None
    if sampler:
        sampler.start()
    # device time: the shard as one chunk (one fill + one traceback launch over
    # inputs already resident in HBM); the slowest rank sets the step time
    eng.set_chunk_pairs(npairs)
    for _ in range(args.warmup):
        eng.run_call(call)
    kern_ms, fill_ms, launches = 0.0, 0.0, 0
    barrier_sync(world)
    for _ in range(args.steps):
        flush_l2()
        eng.run_call(call)
        ms, nl = eng.last_stats()
        f, _ = eng.last_timing()
        kern_ms += ms
        fill_ms += f
        launches += nl
    barrier_sync(world)
    res_one = Engine.decode_call(call)
    # end to end: PP texts in, alignments out through the public pipeline,
    # lcg_prepare_pairs (envelopes on the GPU) + lcg_align_pairs with its
    # default chunk pipeline
    # PP texts in, alignments out: lcg_align_pp_pairs (inputs, bands and GPU
    # envelopes of all pairs first; then each chunk's tables built on the host
    # while the device aligns the previous chunk), caller-owned result buffers
    # allocated once
    eng.set_chunk_pairs(0)
    pcall = eng.prepare_pp_call(pp_pairs, [(t.len_a, t.len_b) for t in tables])
    for _ in range(max(1, args.warmup // 2)):
        eng.run_pp_call(pcall)
    wall_s = 0.0
    phases = [0.0, 0.0, 0.0, 0.0]
    e2e_launches = 0
    barrier_sync(world)
    for _ in range(args.steps):
        flush_l2()
        s0 = time.perf_counter()
        eng.run_pp_call(pcall)  # results are on the host when it returns
        wall_s += time.perf_counter() - s0
        phases = [a + b for a, b in zip(phases, eng.last_phases())]
        e2e_launches += eng.last_stats()[1] + 1  # + the envelope launch
    barrier_sync(world)
    res = Engine.decode_pp_call(pcall)
    graph_captures, graph_replays = eng.last_graphs()
    clocks = sampler.stop() if sampler else None
    h2d, d2h = eng.last_transfer()
    ph2d, pd2h = eng.last_prep_transfer()
    for k in range(npairs):
        if (res[k].score, res[k].edges) != (res_one[k].score, res_one[k].edges):
            raise RuntimeError(f"pair {mine[k]}: the end-to-end pipeline differs from the one-chunk call")
    # spot check against the oracle
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from checks import assert_same_result
    from oracle_ffi import oracle_align
    for k in range(0, npairs, max(1, npairs // 6)):
        assert_same_result(res[k], oracle_align(tables[k]), f"pair {mine[k]}")

    T = max_over_ranks(kern_ms / 1e3 / args.steps, world)
    Tf_mine = fill_ms / 1e3 / args.steps
    We = max_over_ranks(wall_s / args.steps, world)
    if not lead:
        eng.close()
        return
    value = npairs_total / T
    Tf = Tf_mine
    ops = 10 * work["cells"] + 2 * max(work["arc_terms"], 0)
    alg_bytes = h2d + d2h  # every input table read once, every result written once
    out = {
        "metric": "aligns/s (Sankoff all-pairs, bit-exact score+traceback)",
        "value": value,
        "unit": "aligns/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": T * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "int32",
        "data": "synthetic (seeded PP inputs, locarna_gb300/synth.py)",
        "config": {"workload": WORKLOAD_NAME, "pairs": npairs_total, "rnas": WORKLOAD["count"],
                   "len_range": [WORKLOAD["len_lo"], WORKLOAD["len_hi"]], "seed": WORKLOAD["seed"],
                   "mode": "global, default locarna scoring, envelope 1e-4",
                   "families": world,
                   "parallelism": f"{world} x 2016 pairs sharded over {world} GPU(s) by LPT of the host cell counts",
                   "shard_cells": shard_loads(weights, shards),
                   "l2": "flushed between steps (256 MB write)"},
        "gcups": sum(weights) / T / 1e9,
        "e2e": {"value": npairs_total / We, "unit": "aligns/s", "h2d_bytes_per_step": h2d + ph2d,
                "d2h_bytes_per_step": d2h + pd2h, "ms_per_step": We * 1e3,
                "what": "PP texts -> alignments: lcg_align_pp_pairs (parsing, scoring, arc matches, GPU "
                        "envelopes; each chunk's tables built while the device aligns the previous chunk; "
                        "default chunk pipeline), all copies inside",
                "cuda_graphs_last_step": {"captures": graph_captures, "replays": graph_replays},
                "gpu_launches": e2e_launches,
                "pipeline_phases_ms_per_step": dict(zip(("host_tables_and_prep", "pack", "host_waits_for_device",
                                                         "results"),
                                                     (x / args.steps for x in phases)))},
        "gpu_launches": launches,
        "roofline": {"bound": "int32", "kernel": "sankoff_fill_kernel",
                     "achieved": ops / Tf / 1e9, "peak": int_peak, "unit": "Gops/s",
                     "frac": ops / Tf / 1e9 / int_peak,
                     "traffic": FILL_DRAM_BYTES_PER_CELL * work["cells"],
                     "traffic_note": "DRAM read + write bytes per launch: bytes per cell of the ncu capture of "
                                     "the 496-pair case times this launch's cells",
                     "ops_per_launch": ops, "fill_ms": Tf * 1e3,
                     "peak_source": "measured int32 add+max rate (locarna_gb300/_build/liblcg_probe.so)",
                     "hbm_frac_of_measured": alg_bytes / Tf / 1e9 / peaks.get("hbm_gbs", 6800.0)},
        "int_ops": {"ops_per_step": ops, "cells": work["cells"], "arc_terms": work["arc_terms"],
                    "arc_candidates_visited": work["visits"], "groups": work["groups"]},
        "clocks": clocks,
    }
    if tune is not None:
        out["autotune"] = {"buckets": tune, "note": "per length bucket the measured fastest (resident fill blocks per "
                           "SM, pair-wave L2 MB) of 12 on a 64-pair sample; 0 = the default (as many blocks as fit, "
                           "8 MB); value and e2e use the default launch"}
    if extras:
        out["cpu_baseline"] = {"value": cpu_rate, "unit": "aligns/s", "cores": cores, "kind": "port",
                               "sample": f"{cpu_done} random workload pairs, PP files to alignments by "
                                         f"oracle/_build/port_locarna, one process per pair, {cores} at a time, "
                                         f"in batches of {REF_PAIRS_PER_CORE * cores} pairs, "
                                         f"~{CPU_SAMPLE_SECONDS:.0f} s"}
        out.update(run_extras(args, eng, tables, flush_l2, value, table_prep))
        if pf_tables is not None:
            out["locarna_p"] = run_pf(eng, pf_tables, flush_l2, pf_cpu)
    print(json.dumps(out), flush=True)
    eng.close()


def run_extras(args, eng, tables, flush_l2, value, table_prep):
    """Secondary lines at N = 1: one pair alone (global and structure-local),
    the workload one pair per call, --noLP, the local alignment modes."""
    from locarna_gb300.engine import Engine
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from checks import assert_same_result
    from oracle_ffi import oracle_align
    npairs = len(tables)
    # per-pair: the 400 x 400 pair alone, and the workload one pair per call
    pt = per_pair_tables()
    pcall = eng.prepare_call([pt])
    for _ in range(3):
        eng.run_call(pcall)
    single_ms = []
    for _ in range(5):
        flush_l2()
        eng.run_call(pcall)
        single_ms.append(eng.last_stats()[0])
    single_ms.sort()
    # the same pair in structure-local mode
    scall = eng.prepare_call([pt], struct_local=True)
    for _ in range(2):
        eng.run_call(scall)
    sl_ms = []
    for _ in range(3):
        flush_l2()
        eng.run_call(scall)
        sl_ms.append(eng.last_stats()[0])
    sl_ms.sort()
    assert_same_result(Engine.decode_call(scall)[0], oracle_align(pt, struct_local=True), "400x400 struct-local")
    sample = list(range(0, npairs, 16))
    per_calls = [eng.prepare_call([tables[k]]) for k in sample]
    for c in per_calls[:4]:
        eng.run_call(c)
    t1 = time.perf_counter()
    dev_ms_single = 0.0
    for c in per_calls:
        eng.run_call(c)
        dev_ms_single += eng.last_stats()[0]
    wall_single = time.perf_counter() - t1

    # the same workload with locarna --noLP (no lonely pairs): device time of
    # the one-chunk call and wall time of the default call
    ncall = eng.prepare_call(tables, no_lonely_pairs=True)
    eng.set_chunk_pairs(npairs)
    eng.run_call(ncall)
    nolp_ms = []
    for _ in range(max(1, args.steps // 2)):
        flush_l2()
        eng.run_call(ncall)
        nolp_ms.append(eng.last_stats()[0])
    eng.set_chunk_pairs(0)
    eng.run_call(ncall)
    nolp_wall = []
    for _ in range(max(1, args.steps // 2)):
        flush_l2()
        s0 = time.perf_counter()
        eng.run_call(ncall)
        nolp_wall.append(time.perf_counter() - s0)
    nres = Engine.decode_call(ncall)
    for k in range(0, npairs, max(1, npairs // 6)):
        assert_same_result(nres[k], oracle_align(tables[k], no_lonely_pairs=True), f"pair {k} (noLP)")
    return {
        "per_pair": {"workload": "one 400x400 nt pair, global", "device_ms": single_ms[len(single_ms) // 2],
                     "aligns_per_s": 1e3 / single_ms[len(single_ms) // 2],
                     "struct_local_device_ms": sl_ms[len(sl_ms) // 2],
                     "per_pair_launch_aligns_per_s_device": len(sample) / (dev_ms_single / 1e3),
                     "per_pair_launch_aligns_per_s_wall": len(sample) / wall_single,
                     "batched_over_per_pair_launch": value / (len(sample) / (dev_ms_single / 1e3))},
        "table_prep": table_prep,
        "nolp": {"mode": "global, --noLP (no lonely pairs)", "pairs": npairs,
                 "aligns_per_s": npairs / (sum(nolp_ms) / len(nolp_ms) / 1e3),
                 "e2e_aligns_per_s": npairs / (sum(nolp_wall) / len(nolp_wall)),
                 "stacked_arc_matches_traced": sum(len(r.traced_am) for r in nres)},
        "modes": run_modes(eng, tables, flush_l2),
    }


def run_reference(args):
    """The reference arm: the CPU port of the locarna pipeline (PP files in,
    alignments out; oracle/port_locarna) on the machine's host cores, one process
    per pair over a pool of one worker per core. Each step aligns a seeded
    random sample of REF_PAIRS_PER_CORE x cores workload pairs; value = the
    pairs of the timed steps / their measured wall time. Rank 0 only."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from locarna_gb300.build import build_oracle
    build_oracle()
    pp, pairs = workload_pp()
    cores = os.cpu_count() or 1
    per_step = REF_PAIRS_PER_CORE * cores
    rng = random.Random(11)
    walls, dones = [], []
    with tempfile.TemporaryDirectory(prefix="lcg_pp_") as d:
        paths = write_pp_files(pp, d)
        for s in range(args.warmup + args.steps):
            sample = rng.sample(range(len(pairs)), min(per_step, len(pairs)))
            n, wall, _ = port_run(paths, pairs, sample, cores)
            if s >= args.warmup:
                walls.append(wall)
                dones.append(n)
    v = sum(dones) / sum(walls)
    out = {
        "metric": "aligns/s (Sankoff all-pairs, bit-exact score+traceback)",
        "value": v, "unit": "aligns/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * sum(walls) / len(walls), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int64", "data": "synthetic (seeded PP inputs, locarna_gb300/synth.py)",
        "impl": "reference",
        "config": {"workload": WORKLOAD_NAME, "pairs": len(pairs), "rnas": WORKLOAD["count"],
                   "len_range": [WORKLOAD["len_lo"], WORKLOAD["len_hi"]], "seed": WORKLOAD["seed"],
                   "mode": "global, default locarna scoring, envelope 1e-4"},
        "cpu_baseline": {"value": v, "unit": "aligns/s", "cores": cores, "kind": "port",
                         "sample": f"{per_step} random workload pairs per step ({REF_PAIRS_PER_CORE} per core), "
                                   f"PP files to alignments by oracle/_build/port_locarna (host table "
                                   f"preparation + the C restatement of the reference's Aligner), one process "
                                   f"per pair, {cores} at a time; oracle/calibrate_port.py relates its rate "
                                   f"to the reference's locarna"},
        "e2e": {"value": v, "unit": "aligns/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def run_small_case(args):
    """A smaller batch of the same kind of work, one plain run, for profiling:
    `--case small` aligns all pairs of 32 RNAs of 100-150 nt (496 pairs),
    `--case large` all pairs of 16 RNAs of 300-400 nt (120 pairs, the long
    end of the workload's length range)."""
    from concurrent.futures import ThreadPoolExecutor

    from locarna_gb300.engine import Engine
    from locarna_gb300.prep import prepare_pair
    from locarna_gb300.synth import make_family
    if args.case == "large":
        fam = make_family(16, 300, 400, 78)
    else:
        fam = make_family(32, 100, 150, 77)
    pp = [r.to_pp() for r in fam]
    pairs = [(a, b) for a in range(len(fam)) for b in range(a + 1, len(fam))]
    with ThreadPoolExecutor(os.cpu_count() or 4) as ex:
        tables = list(ex.map(lambda ab: prepare_pair(pp[ab[0]], pp[ab[1]]), pairs))
    eng = Engine(0)
    eng.set_chunk_pairs(len(tables))  # one fill launch over the whole case
    for mode in ({}, {"struct_local": True}) if args.struct_local else ({},):
        call = eng.prepare_call(tables, **mode)
        for _ in range(max(1, args.warmup)):
            eng.run_call(call)
        ms, nl = eng.last_stats()
        f, t = eng.last_timing()
        work = None
        if not mode:  # the work counts of the plain mode (a counting launch)
            eng.set_counting(True)
            eng.run_call(call)
            eng.set_counting(False)
            work = eng.last_work()
        print(json.dumps({"case": args.case, "mode": mode, "pairs": len(tables), "kernel_ms": ms,
                          "fill_ms": f, "trace_ms": t, "launches": nl, "work": work}), flush=True)
    eng.close()


def run_pf_small_case(args):
    """A small LocARNA-P batch for profiling: `--case pf-small` runs the
    forward and the backward pass (FP32, then FP64; probabilities only, then
    with the gap gradients) on every 256th pair of the LocARNA-P workload in
    size order (32 pairs of 80-500 nt)."""
    from locarna_gb300.engine import Engine
    tables = build_pf_tables()
    order = sorted(range(len(tables)), key=lambda k: tables[k].len_a * tables[k].len_b)
    tb = [tables[k] for k in order[::256]]
    eng = Engine(0)
    for prec in (32, 64):
        for grads in (False, True):
            for _ in range(max(1, args.warmup)):
                eng.pf_forward(tb, precision=prec, min_am_prob=0.0, gap_gradients=grads)
                eng.pf_backward(probs=True)
            f, b = eng.pf_last_timing()
            print(json.dumps({"case": "pf-small", "precision": prec, "gap_gradients": grads, "pairs": len(tb),
                              "forward_ms": f, "backward_ms": b}), flush=True)
    eng.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--case", default="full", choices=["full", "small", "large", "pf-small"])
    ap.add_argument("--struct-local", action="store_true", help="small case: also struct-local")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-pf", action="store_true", help="skip the LocARNA-P part")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
        return
    from locarna_gb300.build import build_engine, build_oracle, build_probe
    build_engine()
    build_oracle()
    build_probe()
    if args.case in ("small", "large"):
        run_small_case(args)
        return
    if args.case == "pf-small":
        run_pf_small_case(args)
        return
    run_ours(args)


if __name__ == "__main__":
    main()
