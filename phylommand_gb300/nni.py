"""Explicit NNI neighbour trees (the rearrangements `treebender --nni` writes
out, src/tree.cpp:2482-2548).  The batch engine scores every neighbour from
the vectors around its edge without building the trees; this module builds
them, for callers that want the topologies and for the one-launch-per-tree
comparison.

A move is (v, which) as plk_batch_nni_moves reports it:
  0  swap right(v) with v's sibling       (v's parent is not the root)
  1  swap left(v)  with v's sibling
  2  swap right(v) with left(c)           (v, c the root's children)
  3  swap right(v) with right(c)
Branch lengths stay with their nodes (the arrays are indexed by node id).
"""
from __future__ import annotations

import numpy as np


def neighbour_tree(left, right, v: int, which: int):
    L = np.array(left, dtype=np.int32).copy()
    R = np.array(right, dtype=np.int32).copy()
    parent = np.full(L.shape[0], -1, dtype=np.int64)
    for p in range(L.shape[0]):
        for c in (L[p], R[p]):
            if c >= 0:
                parent[c] = p
    u = int(parent[v])
    if which in (0, 1):
        c = R[u] if L[u] == v else L[u]
        if which == 0:
            moved, R[v] = R[v], c
        else:
            moved, L[v] = L[v], c
        if L[u] == c:
            L[u] = moved
        else:
            R[u] = moved
    elif which in (2, 3):
        c = R[u]
        if which == 2:
            R[v], L[c] = L[c], R[v]
        else:
            R[v], R[c] = R[c], R[v]
    else:
        raise ValueError(f"unknown NNI move kind {which}")
    return L, R
