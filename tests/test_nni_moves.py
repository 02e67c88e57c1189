"""NNI neighbour generation on the host: 2(n - 3) moves per binary tree, each
an unrooted topology one interchange (one split) away from the original, all
distinct.  The reference's treebender --nni skips one edge and writes
2(n - 4) trees (src/treebender.cpp:897-915); the engine covers every internal
edge of the unrooted tree."""
import numpy as np
import pytest

from phylommand_gb300 import plk, synth
from phylommand_gb300.nni import neighbour_tree


def splits(left, right):
    """Non-trivial bipartitions of the unrooted tree, as frozensets of tips on
    the side without tip 0."""
    n_nodes = len(left)
    tips = [v for v in range(n_nodes) if left[v] < 0 and right[v] < 0]
    n_tips = len(tips)
    below = {}

    def rec(u):
        if left[u] < 0 and right[u] < 0:
            below[u] = frozenset([u])
            return below[u]
        s = frozenset()
        for c in (left[u], right[u]):
            if c >= 0:
                s |= rec(c)
        below[u] = s
        return s

    root = (set(range(n_nodes)) - {c for v in range(n_nodes) for c in (left[v], right[v]) if c >= 0}).pop()
    rec(root)
    out = set()
    for u, s in below.items():
        if 1 < len(s) < n_tips - 1:
            side = s if 0 not in s else frozenset(tips) - s
            out.add(side)
    return out


@pytest.mark.parametrize("n_tips,seed", [(4, 0), (5, 1), (8, 2), (16, 3), (41, 4)])
def test_nni_moves_cover_every_internal_edge(n_tips, seed):
    rng = np.random.default_rng(seed)
    left, right, bl = synth.yule_tree(n_tips, 0.1, rng)
    moves = plk.nni_moves(left, right)
    assert len(moves) == 2 * (n_tips - 3)
    base = splits(left, right)
    seen = set()
    for v, which in moves:
        L, R = neighbour_tree(left, right, int(v), int(which))
        s = splits(L, R)
        assert len(s) == len(base) == n_tips - 3
        assert len(s - base) == 1 and len(base - s) == 1  # one interchange
        key = frozenset(s)
        assert key not in seen
        seen.add(key)


def test_nni_moves_with_a_tip_at_the_root():
    # root = (t0, ((t1,t2),(t3,t4)))
    left = np.array([-1, -1, -1, -1, -1, 1, 3, 5, 0])
    right = np.array([-1, -1, -1, -1, -1, 2, 4, 6, 7])
    moves = plk.nni_moves(left, right)
    assert len(moves) == 2 * (5 - 3)
    assert set(int(w) for _, w in moves) <= {0, 1}


def _newick(left, right, v=None):
    root = len(left) - 1 if v is None else v

    def rec(u):
        if left[u] < 0 and right[u] < 0:
            return f"t{u}:1"
        return "(" + ",".join(rec(c) for c in (left[u], right[u]) if c >= 0) + "):1"

    return rec(root)[:-2] + ";"


@pytest.mark.parametrize("n_tips,seed", [(5, 11), (7, 12), (12, 13), (20, 14), (33, 15)])
def test_engine_neighbours_include_reference_nni_trees(tmp_path, n_tips, seed):
    """Every tree the reference's own treebender writes with --nni all
    (src/treebender.cpp:897-915 over tree::nni, src/tree.cpp:2482-2548),
    compiled from the reference sources by the oracle's recipe, is one of the
    engine's NNI neighbours (as an unrooted topology)."""
    import os
    import subprocess
    from oracle import oracle as O
    from oracle import refpath
    if not refpath.have_sources():
        pytest.skip("reference sources absent")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    res = subprocess.run(["make", "-s", "-C", os.path.join(root, "oracle"), "bender", f"REFSRC={refpath.REF_SRC}"],
                         capture_output=True, text=True)
    assert res.returncode == 0, res.stdout + res.stderr
    rng = np.random.default_rng(seed)
    left, right, bl = synth.yule_tree(n_tips, 0.1, rng)
    out = subprocess.run([os.path.join(root, "oracle", "_ref", "treebender"), "--nni", "all"],
                         input=_newick(left, right) + "\n", capture_output=True, text=True, check=True).stdout
    trees = [t for t in out.split("\n") if t.strip()]
    assert len(trees) == 1 + 2 * (n_tips - 4)  # the input tree, then two per swapped branch

    def ours(text):
        ft = O.parse_newick(text)
        names = [f"t{i}" for i in range(n_tips)]
        L, R, _, _ = O.reorder_tips_first(ft, names)
        return splits(L, R)

    assert ours(trees[0]) == splits(left, right)
    engine = {frozenset(splits(*neighbour_tree(left, right, int(v), int(w)))) for v, w in plk.nni_moves(left, right)}
    for t in trees[1:]:
        s = frozenset(ours(t))
        assert s != frozenset(splits(left, right))
        assert s in engine
