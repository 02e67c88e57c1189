"""The warm-start network's kernels (BF16 tensor-core GEMMs, loss, bias
gradients, Adam) against the FP64 network oracle, and the feature kernel
against a numpy restatement."""
import numpy as np
import pytest

from oracle import mlp as M
from phylommand_gb300 import plk, synth, warmstart

pytestmark = pytest.mark.gpu

DIMS = [43, 256, 256, 256, 7]


def _data(seed, batch, dims=DIMS):
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(batch, dims[0])).astype(np.float32)
    t = rng.normal(size=(batch, dims[-1])).astype(np.float32)
    return x, t


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.parametrize("batch", [1, 37, 64, 100, 300])
def test_forward_matches_oracle(batch):
    with plk.MLP(43, 7, 256, 3, seed=5) as net:
        p = net.get_params()
        x, _ = _data(batch, batch)
        y = net.forward(x)
        ref_bf16, _, _ = M.forward(p, DIMS, x, bf16_mirror=True)
        ref64, _, _ = M.forward(p, DIMS, x)
        # same roundings as the kernels: FP32 accumulation order only
        assert _rel(y, ref_bf16) < 2e-3
        # against exact FP64 arithmetic: the BF16 storage error
        assert _rel(y, ref64) < 5e-2


def test_gradients_match_oracle_per_layer():
    dims = DIMS
    with plk.MLP(43, 7, 256, 3, seed=11) as net:
        p = net.get_params()
        x, t = _data(3, 200)
        g, loss = net.gradients(x, t)
        ref_loss, ref_g = M.loss_and_grad(p, dims, x, t, bf16_mirror=True)
        _, g64 = M.loss_and_grad(p, dims, x, t)
        assert abs(loss - ref_loss) / ref_loss < 1e-3
        off = 0
        for i in range(len(dims) - 1):
            n_w, n_b = dims[i] * dims[i + 1], dims[i + 1]
            for lo, hi in ((off, off + n_w), (off + n_w, off + n_w + n_b)):
                assert _rel(g[lo:hi], ref_g[lo:hi]) < 5e-3, (i, lo, hi)
                assert _rel(g[lo:hi], g64[lo:hi]) < 6e-2, (i, lo, hi)
            off += n_w + n_b
        assert off == g.size


def test_gradient_of_a_small_network_against_finite_differences():
    dims = [5, 16, 16, 3]
    with plk.MLP(5, 3, 16, 2, seed=2) as net:
        p = net.get_params()
        x, t = _data(4, 50, dims)
        g, _ = net.gradients(x, t)
        idx = np.random.default_rng(0).choice(p.size, 60, replace=False)
        fd = M.finite_difference(p.astype(np.float64), dims, x.astype(np.float64), t.astype(np.float64), idx)
        # BF16 storage: about 1% of the gradient's scale
        assert np.max(np.abs(g[idx] - fd)) < 2e-2 * np.max(np.abs(fd))


def test_adam_step_matches_oracle():
    with plk.MLP(43, 7, 64, 2, seed=4) as net:
        x, t = _data(5, 128, [43, 7])
        p0 = net.get_params().astype(np.float64)
        g, _ = net.gradients(x, t)
        net.train_step(x, t, 1e-3)
        p1 = net.get_params()
        ref, m, v = M.adam(p0, g.astype(np.float64), np.zeros_like(p0), np.zeros_like(p0), 1, 1e-3)
        np.testing.assert_allclose(p1, ref, rtol=1e-5, atol=1e-6)
        # a second step from the same data continues the moments
        g2, _ = net.gradients(x, t)
        net.train_step(x, t, 1e-3)
        ref2, _, _ = M.adam(ref, g2.astype(np.float64), m, v, 2, 1e-3)
        np.testing.assert_allclose(net.get_params(), ref2, rtol=1e-5, atol=1e-6)


def test_training_fits_a_smooth_map():
    rng = np.random.default_rng(6)
    x = rng.normal(size=(2048, 8)).astype(np.float32)
    A = rng.normal(size=(8, 3))
    t = np.tanh(x @ A).astype(np.float32)
    with plk.MLP(8, 3, 64, 2, seed=1) as net:
        first = net.train_step(x[:256], t[:256], 3e-3)
        for step in range(400):
            k = (step % 8) * 256
            last = net.train_step(x[k:k + 256], t[k:k + 256], 3e-3)
        assert last < 0.1 * first


def test_params_round_trip_and_determinism():
    with plk.MLP(43, 7, 256, 3, seed=9) as a, plk.MLP(43, 7, 256, 3, seed=10) as b:
        x, _ = _data(7, 33)
        assert not np.array_equal(a.forward(x), b.forward(x))
        b.set_params(a.get_params())
        np.testing.assert_array_equal(a.forward(x), b.forward(x))
        np.testing.assert_array_equal(a.forward(x), a.forward(x))
        with pytest.raises(ValueError):
            b.set_params(np.zeros(3))


def test_bad_sizes_are_rejected():
    with pytest.raises(plk.PlkError):
        plk.MLP(0, 7)
    with plk.MLP(4, 2, 8, 1) as net:
        with pytest.raises(plk.PlkError):
            net.forward(np.zeros((0, 4), dtype=np.float32))


def _features_ref(masks):
    """numpy restatement of plk_batch_features for one alignment."""
    n = masks.shape[0]
    m_taxa = min(n, 32)
    masks = masks[[(q * n) // m_taxa for q in range(m_taxa)]]
    c = np.stack([(masks == (1 << s)).sum(axis=0) for s in range(4)]).astype(np.float64)  # [4, sites]
    m = c.sum(axis=0)
    out = np.zeros(43)
    out[:4] = c.sum(axis=1) / c.sum()
    pairs = (0.5 * m * (m - 1)).sum()
    types = [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]
    for q, (a, b) in enumerate(types):
        out[4 + q] = (c[a] * c[b]).sum() / pairs
    same = (0.5 * c * (c - 1)).sum(axis=0)
    ok = (m >= 2) & (same > 0)
    h = -np.log(np.where(ok, same, 1.0) / np.where(ok, 0.5 * m * (m - 1), 1.0))
    bins = np.where(ok, np.clip((h / np.log(4.0) * 32.0 + 1e-9).astype(int), 0, 31), 31)
    out[10:42] = np.bincount(bins, minlength=32) / masks.shape[1]
    out[42] = 1.0 - (0.5 * c * (c - 1)).sum() / pairs
    return out


def test_features_match_numpy():
    rng = np.random.default_rng(12)
    with plk.Batch(4) as b:
        al = []
        for n, N in ((4, 1), (16, 700), (33, 1500), (64, 5000), (9, 130)):
            left, right, bl = synth.yule_tree(n, 0.1, rng)
            f = rng.dirichlet(np.full(4, 10.0))
            Q = synth.reversible_q(4, rng.uniform(0.5, 5, 6), f)
            masks = plk.simulate(left, right, bl, Q, f, plk.discrete_gamma(0.7, 4), N, seed=int(rng.integers(1 << 40)))
            masks[rng.random(masks.shape) < 0.05] = 15
            masks[rng.random(masks.shape) < 0.02] = 5       # ambiguous A/C
            b.add(masks, left, right, bl)
            al.append(masks)
        got = b.features()
    for i, masks in enumerate(al):
        np.testing.assert_allclose(got[i], _features_ref(masks), rtol=2e-6, atol=1e-7)


def test_eval_gtr_matches_single_tree_fp64():
    rng = np.random.default_rng(13)
    items = []
    with plk.Batch(4) as b, plk.Handle() as h:
        for n, N in ((8, 400), (32, 2000), (20, 900)):
            left, right, bl = synth.yule_tree(n, 0.08, rng)
            f = rng.dirichlet(np.full(4, 10.0))
            masks = plk.simulate(left, right, bl, synth.reversible_q(4, rng.uniform(0.5, 5, 6), f), f,
                                 plk.discrete_gamma(0.5, 4), N, seed=int(rng.integers(1 << 40)))
            b.add(masks, left, right, bl)
            items.append((masks, left, right, bl))
        freqs = warmstart.empirical_freqs(b.features())
        x = rng.normal(0.0, 0.4, size=(3, 7))
        got = b.eval_gtr(freqs, x)
        for i, (masks, left, right, bl) in enumerate(items):
            exch = np.append(np.exp(x[i, :5]), 1.0)
            Q = synth.reversible_q(4, exch, freqs[i])
            cr = plk.discrete_gamma(np.exp(x[i, 5]), 4) * np.exp(x[i, 6])
            h.set_alignment(masks, 4)
            h.set_tree(left, right, bl)
            h.set_rate_model(False)
            h.set_model(Q, freqs[i], True, cr, np.full(4, 0.25), plk.PLK_P_EXACT)
            ref = h.loglik(plk.PLK_FP64)
            assert abs(got[i] - ref) / abs(ref) < 1e-6


def test_warm_start_end_to_end_small():
    """Labels from the plain GPU fit, a network trained on them, and the
    warm fit of held-out alignments: fewer evaluations, same optimum."""
    data = warmstart.make_labelled(3000, 32, 2000, seed=21)
    assert np.all(np.isfinite(data.lnl)) and np.all(np.isfinite(data.labels))
    ws, hist = warmstart.train(data, epochs=60, seed=3)
    assert hist["train_loss"][-1] < 0.5 * hist["train_loss"][0]
    # the network beats predicting the label mean on held-out labels
    assert np.mean(hist["val_rmse"]) < 0.5 * np.mean(hist["val_rmse_mean_predictor"])
    # held out, and with twice the taxa of the training alignments
    res = warmstart.evaluate(ws, n_items=200, n_taxa=64, n_sites=2000, seed=99)
    # the plain fit judges every warm fit: none ends more than 1e-3 below it
    assert res["frac_final_within_tol_of_plain"] == 1.0, res
    assert res["max_lnl_deficit"] <= 1e-3, res
    assert res["judge"]["fallback_max_abs_lnl_diff_vs_plain"] <= 1e-3, res
    assert res["evals_to_optimum_ratio_warm_over_plain"] < 0.75, res
