"""The oracle against the reference: golden fixtures made by the reference's own
code, plus live runs of the reference harness when its sources are present."""
import os

import numpy as np
import pytest

from oracle import oracle as O
import helpers as H

from oracle import refpath

REF = refpath.REF_EXAMPLES


@pytest.mark.parametrize("name", H.fixture_names())
def test_oracle_reproduces_reference_lnl(name):
    fx = H.load_fixture(name)
    r = H.oracle_for_fixture(fx, want_cond=True)
    assert r.lnl == pytest.approx(float(fx["lnl"]), rel=1e-13, abs=0)
    np.testing.assert_allclose(r.site_lnl, fx["site_lnl"], rtol=1e-13, atol=0)
    k = fx["node_cond"].shape[1]
    np.testing.assert_allclose(r.cond[:, :k], fx["node_cond"], rtol=1e-13, atol=1e-300)


@pytest.mark.parametrize("name", ["ex_jc100", "cfg1_jc16x1000", "syn_gtr_gamma_ambig", "syn_protein20",
                                  "syn_nontr", "syn_multifurc", "syn_ratemodel", "quirk_a"])
def test_oracle_bitwise_where_order_is_the_reference(name):
    """Same operation order and no contraction: equal bits, not just close."""
    fx = H.load_fixture(name)
    r = H.oracle_for_fixture(fx, want_cond=True)
    if len(fx["cat_rates"]) == 1:
        assert r.lnl == float(fx["lnl"])
        assert np.array_equal(r.site_lnl, fx["site_lnl"])
    k = fx["node_cond"].shape[1]
    assert np.array_equal(r.cond[:, :k], fx["node_cond"])


@pytest.mark.parametrize("name", ["ex_gtr100", "syn_protein20", "syn_nontr"])
def test_taylor20_pmat_bitwise(name):
    fx = H.load_fixture(name)
    for t, P in zip(fx["pmat_t"], fx["pmat"]):
        assert np.array_equal(O.pmat_taylor20(fx["Q"], float(t)), P)


def test_q_matrix_matches_reference():
    fx = H.load_fixture("ex_gtr100")
    Q = O.q_matrix(4, True, range(6), [1, 2, 3, 4, 5, 6], [0.1, 0.2, 0.3])
    assert np.array_equal(Q, fx["Q"])
    fx = H.load_fixture("syn_nontr")
    assert np.allclose(fx["Q"].sum(axis=1), 0.0, atol=1e-15)


def test_root_quirk_known_answer():
    """Root-edge lengths do not change the reference's lnL (-22.7094062648644)."""
    a, b = H.load_fixture("quirk_a"), H.load_fixture("quirk_b")
    assert float(a["lnl"]) == pytest.approx(-22.7094062648644, abs=1e-12)
    assert float(a["lnl"]) == float(b["lnl"])
    assert H.oracle_for_fixture(a).lnl == H.oracle_for_fixture(b).lnl


def test_example_known_answers():
    """Known answers of the example files (JC, -m 0,0,0,0,0,0 -P 1 -F .25x4)."""
    fx = H.load_fixture("ex_jc100")
    site = fx["site_lnl"]
    assert site[0] == pytest.approx(-3.73099358652151, abs=1e-13)
    assert site[:10].sum() == pytest.approx(-89.970132644772, abs=1e-11)
    assert float(fx["lnl"]) == pytest.approx(-1205.45062332, abs=1e-8)


def test_exact_pmat_matches_scipy():
    from scipy.linalg import expm
    rng = np.random.default_rng(2)
    for S in (2, 4, 20):
        f = rng.dirichlet(np.ones(S))
        Q = O.q_matrix(S, True, np.arange(S * (S - 1) // 2), rng.uniform(0.2, 3, S * (S - 1) // 2), f[:-1])
        for t in (1e-4, 0.05, 0.7, 4.0):
            np.testing.assert_allclose(O.pmat_exact(Q, t), expm(Q * t), atol=5e-14, rtol=0)


def test_discrete_gamma_matches_quadrature():
    from scipy import integrate, stats
    for alpha in (0.3, 0.5, 1.0, 2.5):
        K = 4
        r = O.discrete_gamma(alpha, K)
        g = stats.gamma(a=alpha, scale=1.0 / alpha)
        edges = [0.0] + [g.ppf((k + 1) / K) for k in range(K - 1)] + [np.inf]
        for k in range(K):
            m, _ = integrate.quad(lambda x: x * g.pdf(x), edges[k], edges[k + 1], limit=200)
            assert r[k] == pytest.approx(m * K, rel=1e-8)
        assert r.mean() == pytest.approx(1.0, abs=1e-12)


def test_marginal_matches_enumeration():
    """Pre-order marginals against brute-force enumeration of internal states."""
    import itertools
    rng = np.random.default_rng(4)
    # ((t0,t1)n4,(t2,t3)n5)n6
    left = np.array([-1, -1, -1, -1, 0, 2, 4])
    right = np.array([-1, -1, -1, -1, 1, 3, 5])
    bl = rng.uniform(0.05, 0.5, 7)
    bl[6] = 0
    f = rng.dirichlet(np.ones(4) * 3)
    Q = O.q_matrix(4, True, range(6), rng.uniform(0.5, 3, 6), f[:-1])
    cr = O.discrete_gamma(0.8, 3)
    cw = np.full(3, 1 / 3)
    tips = (1 << rng.integers(0, 4, size=(4, 6))).astype(np.uint32)
    tips[1, 2] = 15
    r = O.loglik(left, right, tips, bl, Q, f, cr, cw, p_mode=O.P_EXACT, want_marginal=True, want_cond_norm=True)
    ranks = O.internal_postorder(left, right)
    for site in range(6):
        post = {u: np.zeros(4) for u in (4, 5, 6)}
        total = 0.0
        for k in range(3):
            P = {v: O.pmat_exact(Q, bl[v] * cr[k]) for v in range(6)}
            for a6, a4, a5 in itertools.product(range(4), repeat=3):
                p = cw[k] * f[a6] * P[4][a6, a4] * P[5][a6, a5]
                for tip, par, st in ((0, 4, a4), (1, 4, a4), (2, 5, a5), (3, 5, a5)):
                    m = tips[tip, site]
                    p *= sum(P[tip][st, j] for j in range(4) if (m >> j) & 1)
                total += p
                post[4][a4] += p
                post[5][a5] += p
                post[6][a6] += p
        assert np.log(total) == pytest.approx(r.site_lnl[site], rel=1e-12)
        for rank, u in enumerate(ranks):
            np.testing.assert_allclose(r.marginal[rank, site], post[u] / total, atol=1e-13)


def test_newick_parser_resolves_multifurcations_like_the_reference():
    t = O.parse_newick("((a:1,b:2,c:3):4,d:5);")
    # (a,b,c) -> ((a,b):0,c): post-order a b extra c abc d root
    assert t.labels[:2] == ["a", "b"]
    assert t.bl[2] == 0.0 and not t.is_tip(2)
    assert t.labels[3] == "c"
    assert t.n_nodes == 7


@pytest.mark.skipif(not (O.harness_available() and os.path.isdir(REF)), reason="reference sources absent")
def test_parsers_match_reference_on_example_files():
    h = O.run_harness(os.path.join(REF, "alignment_file.fst"), os.path.join(REF, "tree_file.tree"),
                      [0] * 6, [1.0], freqs=[0.25] * 4, nsites=3, dump_tips=True)
    t = O.parse_newick(open(os.path.join(REF, "tree_file.tree")).read())
    assert np.array_equal(t.left, h.tree.left) and np.array_equal(t.right, h.tree.right)
    assert np.array_equal(t.bl, h.tree.bl)
    names, masks = O.parse_fasta(open(os.path.join(REF, "alignment_file.fst")).read())
    assert names == h.names
    full = O.run_harness(os.path.join(REF, "alignment_file.fst"), None, [0] * 6, [1.0], dump_tips=True)
    assert np.array_equal(masks, full.masks)


@pytest.mark.skipif(not O.harness_available(), reason="reference harness not built")
def test_oracle_against_live_reference_random_cases(tmp_path):
    import sys
    sys.path.insert(0, os.path.dirname(__file__))
    from golden import make_golden as G
    rng = np.random.default_rng(123)
    for case in range(4):
        n = int(rng.integers(3, 30))
        fp, tp = G.synthetic(str(tmp_path), f"c{case}", n, int(rng.integers(1, 90)), 4, seed=case, ambig=0.05)
        rates = list(rng.uniform(0.2, 4, 6))
        freqs = list(rng.dirichlet(np.ones(4) * 4))
        h = O.run_harness(fp, tp, range(6), rates, freqs=freqs, dump_tips=True, sites=True)
        left, right, bl, _ = O.reorder_tips_first(h.tree, h.names)
        Q = O.q_matrix(4, True, range(6), rates, freqs[:3])
        last = 1.0
        for f in freqs[:3]:
            last -= f  # sub_model::get_freq order (src/sub_model.cpp:47-50)
        r = O.loglik(left, right, h.masks, O.effective_lengths(left, right, bl), Q, freqs[:3] + [last])
        assert r.lnl == h.lnl
