"""The batch engine (many alignments/trees/models in one persistent launch,
replayed from a CUDA graph) against per-tree evaluations and the oracle."""
import numpy as np
import pytest

from oracle import oracle as O
from phylommand_gb300 import plk, synth
from phylommand_gb300.nni import neighbour_tree

pytestmark = pytest.mark.gpu

SHAPES = [(4, 1), (7, 50), (16, 129), (40, 1000), (130, 3000), (200, 257), (5, 2000), (64, 128), (9, 1300),
          (33, 700)]


def _items(seed=1, C=4, shapes=SHAPES):
    rng = np.random.default_rng(seed)
    out = []
    for n_tips, n_sites in shapes:
        left, right, bl = synth.yule_tree(n_tips, 0.1, rng)
        freqs = rng.dirichlet(np.full(4, 10.0))
        Q = synth.reversible_q(4, rng.uniform(0.5, 5.0, 6), freqs)
        cr = plk.discrete_gamma(rng.uniform(0.3, 2.0), C) if C > 1 else np.ones(1)
        cw = np.full(C, 1.0 / C)
        masks = (np.uint32(1) << rng.integers(0, 4, size=(n_tips, n_sites)).astype(np.uint32)).astype(np.uint32)
        masks[rng.random(masks.shape) < 0.02] = 15
        out.append((masks, left, right, bl, Q, freqs, cr, cw))
    return out


def _single(masks, left, right, bl, Q, freqs, cr, cw, precision=plk.PLK_FP32S):
    with plk.Handle() as h:
        h.set_alignment(masks, 4)
        h.set_tree(left, right, bl)
        h.set_rate_model(False)
        h.set_model(Q, freqs, True, cr, cw, plk.PLK_P_EXACT)
        return h.loglik(precision)


def _batch(items, C=4):
    b = plk.Batch(C)
    for masks, left, right, bl, Q, freqs, cr, cw in items:
        i = b.add(masks, left, right, bl)
        b.set_model(i, Q, freqs, cr, cw)
    return b


def test_batch_matches_single_tree_evaluations():
    items = _items()
    with _batch(items) as b:
        got = b.loglik()
        tune = b.tuning()
    assert tune["grid"] > 0 and tune["sites_per_thread"] in (1, 2)
    for (masks, left, right, bl, Q, freqs, cr, cw), g in zip(items, got):
        assert g == pytest.approx(_single(masks, left, right, bl, Q, freqs, cr, cw), rel=1e-12)
        teff = O.effective_lengths(left, right, bl, root_dist0=1e-30)
        orc = O.loglik(left, right, masks, teff, Q, freqs, cr, cw, p_mode=O.P_EXACT)
        assert g == pytest.approx(orc.lnl, rel=1e-6)


def test_model_updates_reach_graph_replays():
    items = _items(seed=2, shapes=SHAPES[:6])
    with _batch(items) as b:
        first = b.loglik()
        masks, left, right, bl, Q, freqs, cr, cw = items[3]
        b.set_model(3, Q, freqs, cr * 1.7, cw)
        second = b.loglik()
        assert second[3] == pytest.approx(_single(masks, left, right, bl, Q, freqs, cr * 1.7, cw), rel=1e-12)
        assert np.array_equal(np.delete(second, 3), np.delete(first, 3))
        assert second[3] != first[3]


@pytest.mark.parametrize("env", [{"PLK_BATCH_NOGRAPH": "1"}, {"PLK_BATCH_SPT": "1"}, {"PLK_BATCH_SPT": "2"}])
def test_batch_paths_agree(monkeypatch, env):
    items = _items(seed=3, shapes=SHAPES[2:8])
    with _batch(items) as b:
        ref = b.loglik()
    for k, v in env.items():
        monkeypatch.setenv(k, v)
    with _batch(items) as b:
        got = b.loglik()
        if "PLK_BATCH_NOGRAPH" in env:
            assert not b.tuning()["graph"]
    np.testing.assert_allclose(got, ref, rtol=1e-12)


@pytest.mark.parametrize("C", [2, 4, 8])
@pytest.mark.parametrize("spt", ["1", "2"])
def test_paired_form_same_bits(monkeypatch, C, spt):
    """Categories in pairs on the FP32x2 pipe round lane by lane like the
    one-at-a-time body: with the same tile size the lnL bits agree."""
    items = _items(seed=30 + C, C=C, shapes=SHAPES[:7])
    monkeypatch.setenv("PLK_BATCH_SPT", spt)
    got = {}
    for paired in ("0", "1"):
        monkeypatch.setenv("PLK_BATCH_PAIRED", paired)
        with _batch(items, C) as b:
            got[paired] = b.loglik()
            tune = b.tuning()
            assert tune["paired"] == (paired == "1") and tune["sites_per_thread"] == int(spt)
            # a model update after tuning reaches the paired layouts too
            masks, left, right, bl, Q, freqs, cr, cw = items[2]
            b.set_model(2, Q, freqs, cr * 1.3, cw)
            again = b.loglik()
            assert again[2] == pytest.approx(_single(masks, left, right, bl, Q, freqs, cr * 1.3, cw), rel=1e-12)
    assert np.array_equal(got["0"], got["1"])
    for (masks, left, right, bl, Q, freqs, cr, cw), g in zip(items, got["1"]):
        assert g == pytest.approx(_single(masks, left, right, bl, Q, freqs, cr, cw), rel=1e-12)


@pytest.mark.parametrize("C", [4, 1])
def test_nni_neighbours_match_explicit_trees(C):
    shapes = [(4, 60), (6, 129), (13, 300), (25, 77), (40, 1000)]
    items = _items(seed=10 + C, C=C, shapes=shapes)
    # one tree with a tip as a root child
    masks, left, right, bl, Q, freqs, cr, cw = items[2]
    with _batch(items, C=C) as b:
        base = b.loglik()
        nni = b.nni_loglik()
        moves = [b.nni_moves(i) for i in range(len(items))]
    for (masks, left, right, bl, Q, freqs, cr, cw), got, mv, lb in zip(items, nni, moves, base):
        n_tips = masks.shape[0]
        assert len(got) == len(mv) == 2 * (n_tips - 3)
        for (v, which), g in zip(mv, got):
            L, R = neighbour_tree(left, right, int(v), int(which))
            ref64 = _single(masks, L, R, bl, Q, freqs, cr, cw, precision=plk.PLK_FP64)
            assert g == pytest.approx(ref64, rel=1e-6)
        assert np.isfinite(lb)


def test_batch_single_category_and_errors():
    items = _items(seed=4, C=1, shapes=SHAPES[:4])
    with _batch(items, C=1) as b:
        got = b.loglik()
    for (masks, left, right, bl, Q, freqs, cr, cw), g in zip(items, got):
        assert g == pytest.approx(_single(masks, left, right, bl, Q, freqs, cr, cw), rel=1e-12)
    with plk.Batch(4) as b:
        with pytest.raises(plk.PlkError):
            b.loglik()  # empty batch
        masks, left, right, bl, Q, freqs, cr, cw = _items(seed=5, shapes=[(6, 10)])[0]
        bad = masks.copy()
        bad[1, 2] = 0
        with pytest.raises(plk.PlkError) as e:
            b.add(bad, left, right, bl)
        assert e.value.status == plk.PLK_ERR_TIP
        b.add(masks, left, right, bl)
        with pytest.raises(plk.PlkError) as e:
            b.loglik()  # no model yet
        assert e.value.status == plk.PLK_ERR_STATE
