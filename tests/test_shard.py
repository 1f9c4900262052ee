"""Sharding a batch of pairs across ranks (CPU, gloo, world_size 2).

The multi-GPU path of lcg_align_pairs batches is a host-side split: an LPT
partition of the pairs by their estimated work, one shard per rank, and a
host gather in input order. Here two gloo ranks each align their shard with
the oracle (standing in for one GPU per rank) and the gathered results must
equal a single-rank run pair for pair.
"""
import multiprocessing as mp
import os
import socket

import pytest

from locarna_gb300.shard import lpt_partition, merge_shards, shard_loads


def test_lpt_partition_covers_every_pair_once_and_balances():
    w = [5, 1, 9, 3, 3, 7, 2, 8, 4, 6, 1, 1]
    sh = lpt_partition(w, 3)
    flat = sorted(k for s in sh for k in s)
    assert flat == list(range(len(w)))
    assert all(s == sorted(s) for s in sh)
    loads = shard_loads(w, sh)
    assert max(loads) - min(loads) <= max(w)
    # deterministic: the same split on every rank
    assert lpt_partition(w, 3) == sh
    assert lpt_partition([], 2) == [[], []]
    assert lpt_partition([3], 4) == [[0], [], [], []]


def test_merge_restores_input_order():
    sh = [[0, 3], [1, 2, 4]]
    assert merge_shards(sh, [["a", "d"], ["b", "c", "e"]], 5) == list("abcde")
    with pytest.raises(ValueError):
        merge_shards(sh, [["a"], ["b", "c", "e"]], 5)


def _family_tables():
    from locarna_gb300.prep import prepare_pair
    from locarna_gb300.synth import make_family
    fam = make_family(8, 40, 120, 5, q=0.05)
    pp = [r.to_pp() for r in fam]
    return [prepare_pair(pp[a], pp[b]) for a in range(len(fam)) for b in range(a + 1, len(fam))]


def _oracle_batch(tables, **kw):
    from oracle_ffi import oracle_align
    return [oracle_align(t, **kw) for t in tables]


def _rank_main(rank, world, port, out_q):
    import torch.distributed as dist

    from locarna_gb300.shard import align_sharded
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        tables = _family_tables()
        res, shards = align_sharded(tables, _oracle_batch, rank, world)
        out_q.put((rank, [(r.score, r.max_ij, r.edges, r.traced_am) for r in res], shards))
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_rank_shards_gather_equal_the_single_rank_result():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = [q.get(timeout=240) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    tables = _family_tables()
    single = [(r.score, r.max_ij, r.edges, r.traced_am) for r in _oracle_batch(tables)]
    shards = None
    for rank, res, sh in got:
        assert res == single, f"rank {rank}"
        shards = sh if shards is None else shards
        assert sh == shards  # every rank made the same split
    assert len(shards) == 2 and all(shards) and sorted(shards[0] + shards[1]) == list(range(len(tables)))
