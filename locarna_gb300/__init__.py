"""locarna_gb300 — GB300-native sparsified Sankoff (LocARNA) alignment engine.

Host tables in the layout of include/locarna_gb300.h go through the C ABI into
hand-written sm_103a kernels; see ``engine.Engine``.
"""
from .abi import PairTables, make_opts  # noqa: F401

__all__ = ["PairTables", "make_opts"]
