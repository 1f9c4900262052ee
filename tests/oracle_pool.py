"""The oracle over many pairs in parallel (test infrastructure).

Worker processes are started with spawn: a process forked after the first GPU
call of its parent can hang, and the GPU tests call this after the engine
fixture has initialised CUDA.
"""
import multiprocessing as mp
import os


def _align(args):
    from oracle_ffi import oracle_align
    tables, kw = args
    return oracle_align(tables, **kw)


def oracle_align_many(tables, procs=None, **kw):
    """oracle_align on every pair of `tables`, in input order."""
    procs = procs or min(len(tables), os.cpu_count() or 1)
    with mp.get_context("spawn").Pool(procs) as pool:
        return pool.map(_align, [(t, kw) for t in tables], chunksize=1)
