"""Batched pairs across GPUs: one shard of the pair list per rank.

Pairs are independent, so a batch shards with no exchange during the
alignment: the pair list is split by estimated work with longest-processing-
time-first (LPT) bin packing, every rank aligns its shard on its own GPU, and
the results are gathered on the host in the input order. This is what the
reference's mlocarna does with processes (src/Utils/mlocarna:3547-3625 spreads
the pairwise alignments over worker processes; :389-400 splits a pair list
k of N ways), here with one process per GPU.

The work estimate of a pair is its M cells (the left-end groups' rectangles
plus the top level) from lcg_pair_work, computed on the host before any
alignment.
"""
import heapq


def lpt_partition(weights, nshards):
    """Split item indices into nshards lists by LPT: items in order of
    decreasing weight (ties: lower index first), each to the shard with the
    least total weight so far (ties: lower shard). Each shard's indices come
    back ascending, so a shard keeps the input order."""
    if nshards < 1:
        raise ValueError("nshards must be >= 1")
    order = sorted(range(len(weights)), key=lambda k: (-weights[k], k))
    heap = [(0, s) for s in range(nshards)]
    shards = [[] for _ in range(nshards)]
    for k in order:
        load, s = heapq.heappop(heap)
        shards[s].append(k)
        heapq.heappush(heap, (load + weights[k], s))
    return [sorted(sh) for sh in shards]


def shard_loads(weights, shards):
    return [sum(weights[k] for k in sh) for sh in shards]


def pair_weights(tables, **align_kw):
    """Work estimate per pair: M cells from lcg_pair_work (host only)."""
    from .engine import pair_work
    return [pair_work(t, **align_kw)[1] for t in tables]


def merge_shards(shards, shard_results, n):
    """Results of all shards back in input order."""
    out = [None] * n
    for sh, res in zip(shards, shard_results):
        if len(sh) != len(res):
            raise ValueError("shard result count differs from its pair count")
        for k, r in zip(sh, res):
            out[k] = r
    if any(r is None for r in out):
        raise ValueError("a pair has no result")
    return out


def align_sharded(tables, align_fn, rank, world, group=None, weights=None, **align_kw):
    """Align `tables` across `world` ranks of torch.distributed: this rank
    aligns its LPT shard with align_fn(shard_tables, **align_kw) and every
    rank receives all results in input order (a host gather of Python
    objects; no device collective). Every rank must pass the same tables.
    Returns (results, shards)."""
    import torch.distributed as dist
    if weights is None:
        weights = pair_weights(tables, **align_kw)
    shards = lpt_partition(weights, world)
    mine = align_fn([tables[k] for k in shards[rank]], **align_kw) if shards[rank] else []
    gathered = [None] * world
    dist.all_gather_object(gathered, list(mine), group=group)
    return merge_shards(shards, gathered, len(tables)), shards
