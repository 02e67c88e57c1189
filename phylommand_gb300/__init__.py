"""GB300 phylogenetic likelihood engine: a drop-in for the likelihood path of
phylommand's treeator (simpleML / sub_model / rate_model).

The engine is ``lib/libplk.so`` behind the C ABI in ``include/plk.h``;
``plk`` binds it with ctypes, ``synth`` makes seeded workloads.
"""
from . import plk  # noqa: F401

__all__ = ["plk"]
