"""Branch-length derivatives and the ML branch-length optimiser of the batch
engine against FP64 finite differences of the single-tree engine."""
import numpy as np
import pytest

from phylommand_gb300 import plk, synth

pytestmark = pytest.mark.gpu


def _items(seed, shapes, C=4):
    rng = np.random.default_rng(seed)
    out = []
    for n_tips, n_sites in shapes:
        left, right, bl = synth.yule_tree(n_tips, 0.1, rng)
        f = rng.dirichlet(np.full(4, 10.0))
        Q = synth.reversible_q(4, rng.uniform(0.5, 5.0, 6), f)
        cr = plk.discrete_gamma(0.7, C) if C > 1 else np.ones(1)
        cw = np.full(C, 1.0 / C)
        masks = plk.simulate(left, right, bl, Q, f, cr, n_sites, seed=int(rng.integers(1 << 40)))
        masks[rng.random(masks.shape) < 0.02] = 15
        out.append((masks, left, right, bl, Q, f, cr, cw))
    return out


def _fp64(h, item, bl):
    masks, left, right, _, Q, f, cr, cw = item
    h.set_alignment(masks, 4)
    h.set_tree(left, right, bl)
    h.set_rate_model(False)
    h.set_model(Q, f, True, cr, cw, plk.PLK_P_EXACT)
    return h.loglik(plk.PLK_FP64)


@pytest.mark.parametrize("C", [4, 1])
def test_edge_derivatives_match_finite_differences(C):
    items = _items(3 + C, [(8, 500), (21, 1200), (5, 300)], C=C)
    rng = np.random.default_rng(C)
    with plk.Batch(C) as b, plk.Handle() as h:
        for i, (masks, left, right, bl, Q, f, cr, cw) in enumerate(items):
            b.add(masks, left, right, bl)
            b.set_model(i, Q, f, cr, cw)
        der = b.edge_derivatives()
        for i, item in enumerate(items):
            bl = item[3]
            n_nodes = len(bl)
            root = n_nodes - 1
            assert np.all(der[i][root] == 0.0)
            for v in rng.choice(root, size=min(6, root), replace=False):
                eps = 1e-4 * max(bl[v], 1e-2)
                lp = _fp64(h, item, np.where(np.arange(n_nodes) == v, bl + eps, bl))
                lm = _fp64(h, item, np.where(np.arange(n_nodes) == v, bl - eps, bl))
                l0 = _fp64(h, item, bl)
                d1 = (lp - lm) / (2 * eps)
                d2 = (lp - 2 * l0 + lm) / eps ** 2
                scale = item[0].shape[1]
                assert abs(der[i][v, 0] - d1) <= 2e-4 * (abs(d1) + scale), (i, v, der[i][v], d1)
                assert abs(der[i][v, 1] - d2) <= 2e-2 * abs(d2) + 1e-3 * scale / max(bl[v], 1e-2), (i, v, der[i][v], d2)


def test_optimize_branches_reaches_a_stationary_point():
    items = _items(11, [(12, 2000), (30, 3000), (6, 800)])
    rng = np.random.default_rng(5)
    start = [it[3] * np.exp(rng.normal(0.0, 0.7, len(it[3]))) for it in items]
    with plk.Batch(4) as b, plk.Handle() as h:
        for i, (masks, left, right, bl, Q, f, cr, cw) in enumerate(items):
            b.add(masks, left, right, start[i])
            b.set_model(i, Q, f, cr, cw)
        before = b.loglik()
        lnl, iters = b.optimize_branches(max_iter=60, tol=1e-5)
        assert iters >= 1
        assert np.all(lnl >= before)
        der = b.edge_derivatives()
        for i, item in enumerate(items):
            fitted = b.branch_lengths(i)
            # the batch's FP32 lnL at the fitted lengths equals the FP64 engine's
            l64 = _fp64(h, item, fitted)
            assert lnl[i] == pytest.approx(l64, rel=1e-6)
            # at least as good as the generating lengths (the ML point beats them)
            assert l64 >= _fp64(h, item, item[3]) - 1e-3
            # stationary: on every non-root edge off the length floor another
            # Newton step would gain next to nothing, g^2 / (2 |c|), with the
            # curvature negative (the two root edges act through their sum,
            # so both carry the same slope)
            root = len(fitted) - 1
            g, c = der[i][:root, 0], der[i][:root, 1]
            free = fitted[:root] > 1e-6
            assert np.all(c[free] < 0.0), (i, c[free].max())
            gain = g[free] ** 2 / (2.0 * np.abs(c[free]))
            assert gain.max() < 1e-3, (i, gain.max(), g[free][np.argmax(gain)], c[free][np.argmax(gain)])
