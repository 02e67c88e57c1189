"""GPU parity: the engine (through the C ABI) against the reference's golden
fixtures and against the FP64 oracle.

Tolerances: FP64 plain form 1e-12 relative on lnL (the reference order is kept,
so it is equal up to the order of the final site sum); FP32 scaled form 1e-6
relative on lnL and 1e-5 absolute on normalised node probabilities."""
import numpy as np
import pytest

from oracle import oracle as O
from phylommand_gb300 import plk, synth
import helpers as H

pytestmark = pytest.mark.gpu

FP64_REL = 1e-12
FP32_REL = 1e-6
FP32_PROB = 1e-5
BF16_SITE_REL = 5e-5


@pytest.mark.parametrize("name", H.fixture_names())
def test_fp64_matches_reference_fixture(name):
    fx = H.load_fixture(name)
    with H.engine_for_fixture(fx) as h:
        lnl = h.loglik(plk.PLK_FP64)
        assert lnl == pytest.approx(float(fx["lnl"]), rel=FP64_REL)
        site = h.site_loglik()
        # per site, the same operations in the same order as the reference
        np.testing.assert_allclose(site, fx["site_lnl"], rtol=1e-14, atol=1e-14)
        nodes = h.node_states(plk.PLK_NODES_COND, plk.PLK_FP64)
        k = fx["node_cond"].shape[1]
        ref = H.normalise_cond(fx["node_cond"], fx["cat_weights"])
        np.testing.assert_allclose(nodes[:, :k], ref, rtol=0, atol=1e-14)


@pytest.mark.parametrize("name", H.fixture_names())
def test_fp32_scaled_matches_reference_fixture(name):
    fx = H.load_fixture(name)
    with H.engine_for_fixture(fx) as h:
        lnl = h.loglik(plk.PLK_FP32S)
        assert lnl == pytest.approx(float(fx["lnl"]), rel=FP32_REL)
        nodes = h.node_states(plk.PLK_NODES_COND, plk.PLK_FP32S)
        k = fx["node_cond"].shape[1]
        ref = H.normalise_cond(fx["node_cond"], fx["cat_weights"])
        np.testing.assert_allclose(nodes[:, :k], ref, rtol=0, atol=FP32_PROB)


@pytest.mark.parametrize("name", H.fixture_names())
def test_marginals_match_oracle(name):
    fx = H.load_fixture(name)
    orc = H.oracle_for_fixture(fx, want_marginal=True)
    with H.engine_for_fixture(fx) as h:
        m64 = h.node_states(plk.PLK_NODES_MARGINAL, plk.PLK_FP64)
        np.testing.assert_allclose(m64, orc.marginal, rtol=0, atol=1e-12)
        m32 = h.node_states(plk.PLK_NODES_MARGINAL, plk.PLK_FP32S)
        np.testing.assert_allclose(m32, orc.marginal, rtol=0, atol=FP32_PROB)


@pytest.mark.parametrize("name", ["ex_gtr_gamma_noquirk", "syn_gtr_gamma_ambig", "syn_protein20", "syn_nontr"])
def test_exact_pmat_mode_matches_oracle(name):
    fx = H.load_fixture(name)
    orc = H.oracle_for_fixture(fx, p_mode=O.P_EXACT)
    with H.engine_for_fixture(fx, p_mode=plk.PLK_P_EXACT) as h:
        assert h.loglik(plk.PLK_FP64) == pytest.approx(orc.lnl, rel=1e-11)
        assert h.loglik(plk.PLK_FP32S) == pytest.approx(orc.lnl, rel=FP32_REL)


def _random_case(rng, n_tips, n_sites, S=4, C=1, missing=0.02, shape="yule"):
    if shape == "yule":
        left, right, bl = synth.yule_tree(n_tips, 0.1, rng)
    elif shape == "balanced":  # tips paired level by level: the deepest spill stack
        n_nodes = 2 * n_tips - 1
        left = np.full(n_nodes, -1, dtype=np.int32)
        right = np.full(n_nodes, -1, dtype=np.int32)
        level, u = list(range(n_tips)), n_tips
        while len(level) > 1:
            nxt = []
            for i in range(0, len(level) - 1, 2):
                left[u], right[u] = level[i], level[i + 1]
                nxt.append(u)
                u += 1
            if len(level) % 2:
                nxt.append(level[-1])
            level = nxt
        bl = rng.exponential(0.1, n_nodes)
    else:  # caterpillar: ((((t0,t1),t2),t3)...)
        n_nodes = 2 * n_tips - 1
        left = np.full(n_nodes, -1, dtype=np.int32)
        right = np.full(n_nodes, -1, dtype=np.int32)
        prev = 0
        for i in range(1, n_tips):
            u = n_tips + i - 1
            left[u], right[u] = prev, i
            prev = u
        bl = rng.exponential(0.1, n_nodes)
    f = rng.dirichlet(np.ones(S) * 5)
    npos = S * (S - 1) // 2
    Q = synth.reversible_q(S, rng.uniform(0.5, 3, npos), f)
    masks = (np.uint32(1) << rng.integers(0, S, size=(n_tips, n_sites)).astype(np.uint32)).astype(np.uint32)
    masks[rng.random(masks.shape) < missing] = np.uint32((1 << S) - 1)
    cr = plk.discrete_gamma(0.6, C) if C > 1 else np.ones(1)
    cw = np.full(C, 1.0 / C)
    return left, right, bl, masks, Q, f, cr, cw


def _engine(left, right, bl, masks, S, Q, f, cr, cw, p_mode=plk.PLK_P_EXACT, quirk=False):
    h = plk.Handle()
    h.set_alignment(masks, S)
    h.set_tree(left, right, bl)
    h.set_rate_model(quirk)
    h.set_model(Q, f, True, cr, cw, p_mode)
    return h


@pytest.mark.parametrize("n_sites", [1, 31, 127, 128, 129, 1000, 4099])
def test_ragged_site_counts(n_sites):
    rng = np.random.default_rng(n_sites)
    left, right, bl, masks, Q, f, cr, cw = _random_case(rng, 13, n_sites, C=4)
    teff = plk.effective_lengths(left, right, bl, False)
    orc = O.loglik(left, right, masks, teff, Q, f, cr, cw, p_mode=O.P_EXACT)
    with _engine(left, right, bl, masks, 4, Q, f, cr, cw) as h:
        assert h.loglik(plk.PLK_FP64) == pytest.approx(orc.lnl, rel=1e-11)
        np.testing.assert_allclose(h.site_loglik(), orc.site_lnl, rtol=1e-11)
        assert h.loglik(plk.PLK_FP32S) == pytest.approx(orc.lnl, rel=FP32_REL)


@pytest.mark.parametrize("S,C", [(2, 1), (3, 2), (4, 8), (4, 12), (5, 4), (20, 4), (24, 2)])
def test_state_and_category_counts(S, C):
    """Fused 4-state kernel for C <= 8, generic kernel otherwise."""
    rng = np.random.default_rng(S * 100 + C)
    left, right, bl, masks, Q, f, cr, cw = _random_case(rng, 17, 300, S=S, C=C)
    teff = plk.effective_lengths(left, right, bl, False)
    orc = O.loglik(left, right, masks, teff, Q, f, cr, cw, p_mode=O.P_EXACT, want_marginal=True)
    with _engine(left, right, bl, masks, S, Q, f, cr, cw) as h:
        assert h.loglik(plk.PLK_FP64) == pytest.approx(orc.lnl, rel=1e-11)
        assert h.loglik(plk.PLK_FP32S) == pytest.approx(orc.lnl, rel=FP32_REL)
        np.testing.assert_allclose(h.node_states(plk.PLK_NODES_MARGINAL, plk.PLK_FP64), orc.marginal, atol=1e-11)


@pytest.mark.parametrize("shape,n_tips", [("yule", 600), ("caterpillar", 400)])
def test_deep_and_wide_trees(shape, n_tips):
    rng = np.random.default_rng(n_tips)
    left, right, bl, masks, Q, f, cr, cw = _random_case(rng, n_tips, 333, C=4, shape=shape)
    teff = plk.effective_lengths(left, right, bl, False)
    orc = O.loglik(left, right, masks, teff, Q, f, cr, cw, p_mode=O.P_EXACT)
    with _engine(left, right, bl, masks, 4, Q, f, cr, cw) as h:
        assert h.loglik(plk.PLK_FP64) == pytest.approx(orc.lnl, rel=1e-11)
        # a caterpillar of 400 tips underflows FP32 without the per-site scaling
        assert h.loglik(plk.PLK_FP32S) == pytest.approx(orc.lnl, rel=FP32_REL)


def test_unary_nodes():
    """A node with one child passes its child's transported vector up."""
    # root(6) has one child 5; 5 = (4, t2); 4 = (t0, t1); node 3 = unary above t3? keep tips 0..3
    left = np.array([-1, -1, -1, -1, 0, 4, 5, 3], dtype=np.int32)
    right = np.array([-1, -1, -1, -1, 1, 2, -1, 6], dtype=np.int32)
    bl = np.array([0.1, 0.2, 0.3, 0.15, 0.05, 0.07, 0.2, 0.0])
    rng = np.random.default_rng(3)
    masks = (1 << rng.integers(0, 4, size=(4, 50))).astype(np.uint32)
    f = np.full(4, 0.25)
    Q = synth.reversible_q(4, np.ones(6), f)
    teff = plk.effective_lengths(left, right, bl, False)
    orc = O.loglik(left, right, masks, teff, Q, f, p_mode=O.P_EXACT, want_marginal=True)
    with _engine(left, right, bl, masks, 4, Q, f, np.ones(1), np.ones(1)) as h:
        assert h.loglik(plk.PLK_FP64) == pytest.approx(orc.lnl, rel=1e-12)
        assert h.loglik(plk.PLK_FP32S) == pytest.approx(orc.lnl, rel=FP32_REL)
        np.testing.assert_allclose(h.node_states(plk.PLK_NODES_MARGINAL, plk.PLK_FP64), orc.marginal, atol=1e-12)


def test_tip_without_state_returns_zero_like_the_reference():
    """simpleML::check_nodes fails -> calculate_log_likelihood returns 0.0."""
    fx = H.load_fixture("quirk_a")
    masks = fx["masks"].copy()
    masks[2, 3] = 0
    with plk.Handle() as h:
        h.set_alignment(masks, 4)
        h.set_tree(fx["left"], fx["right"], fx["bl"])
        h.set_model(fx["Q"], fx["root_w"], True)
        st, v = h.loglik_status(plk.PLK_FP64)
        assert st == plk.PLK_ERR_TIP and v == 0.0


def test_call_order_and_argument_errors():
    with plk.Handle() as h:
        st, _ = h.loglik_status()
        assert st == plk.PLK_ERR_STATE
        with pytest.raises(plk.PlkError) as e:
            h.set_alignment(np.zeros((3, 0), dtype=np.uint32), 4)
        assert e.value.status == plk.PLK_ERR_ARG
        with pytest.raises(plk.PlkError):
            h.set_tree([-1, -1, 0], [-1, -1, 1], [0.1, np.nan, 0.0])
        h.set_alignment(np.full((2, 5), 15, dtype=np.uint32), 4)
        h.set_tree([-1, -1, -1, 0, 3], [-1, -1, -1, 1, 2], [0.1, 0.1, 0.1, 0.1, 0.0])  # 3 leaves vs 2 rows
        h.set_model(np.full((4, 4), 1 / 3) - np.eye(4) * (4 / 3), np.full(4, 0.25), True)
        st, _ = h.loglik_status()
        assert st == plk.PLK_ERR_ARG


@pytest.mark.parametrize("S,patterns,n_sites", [(4, False, 777), (4, True, 777), (3, False, 777), (6, False, 777),
                                                (4, False, 784), (3, False, 1600)])
def test_byte_masks_match_32bit_masks(S, patterns, n_sites):
    """plk_set_alignment8 (device encoding for <= 4 states -- 16 cells per
    thread when rows are a multiple of 16 sites --, host widening otherwise
    or with patterns) gives the same bits as plk_set_alignment, ignores the
    bits above the alphabet, and reports an empty cell (no state bit left)
    the same way."""
    rng = np.random.default_rng(S + 10 * patterns + n_sites)
    left, right, bl, masks, Q, f, cr, cw = _random_case(rng, 19, n_sites, S=S, C=4)
    masks[rng.random(masks.shape) < 0.05] |= np.uint32(0x40)  # bits above the alphabet
    out = []
    for m in (masks.astype(np.uint32), masks.astype(np.uint8)):
        h = plk.Handle()
        h.set_patterns(patterns)
        h.set_alignment(m, S)
        h.set_tree(left, right, bl)
        h.set_rate_model(False)
        h.set_model(Q, f, True, cr, cw, plk.PLK_P_EXACT)
        out.append((h.loglik(plk.PLK_FP64), h.site_loglik(), h.loglik(plk.PLK_FP32S)))
        for cell in (0, 0x40):  # no bit at all / only bits above the alphabet
            bad = m.copy()
            bad[3, 5] = cell
            h.set_alignment(bad, S)
            st, _ = h.loglik_status()
            assert st == plk.PLK_ERR_TIP
        h.close()
    assert out[0][0] == out[1][0] and out[0][2] == out[1][2]
    np.testing.assert_array_equal(out[0][1], out[1][1])


def test_repeat_calls_are_deterministic():
    fx = H.load_fixture("syn_gtr_gamma_ambig")
    with H.engine_for_fixture(fx, p_mode=plk.PLK_P_EXACT) as h:
        a = [h.loglik(plk.PLK_FP32S) for _ in range(3)]
        b = [h.loglik(plk.PLK_FP64) for _ in range(3)]
        assert a[0] == a[1] == a[2] and b[0] == b[1] == b[2]


@pytest.mark.parametrize("n_tips,n_sites,C", [(128, 1000, 4), (40, 257, 1), (1300, 300, 4), (60, 129, 8),
                                             (20, 33, 4), (5, 1, 2)])
def test_fp32_kernel_variants_agree(monkeypatch, n_tips, n_sites, C):
    """Every candidate of the autotuner (prune4_kernel, prune4s_kernel with 1
    and 2 sites per thread, prune4p_kernel with category pairs on FP32x2 where
    C is 2, 4 or 8 -- one or two sites per thread, or two threads per site
    for 4 and 8 categories; tip codes in shared memory or read from global
    for the 1300-tip tree, or staged with each op's tables; the
    warp-independent prune4w_kernel) gives the same per-site values."""
    rng = np.random.default_rng(n_tips + n_sites)
    left, right, bl, masks, Q, f, cr, cw = _random_case(rng, n_tips, n_sites, C=C)
    teff = plk.effective_lengths(left, right, bl, False)
    orc = O.loglik(left, right, masks, teff, Q, f, cr, cw, p_mode=O.P_EXACT)
    sites = []
    variants = {1: ("0", "1", "2"), 2: ("0", "1", "2", "3", "4", "5", "6", "9", "10", "11", "12", "13", "14"),
                8: ("0", "1", "2", "3", "4", "5", "6", "7", "8", "9", "10", "11", "12", "13")}.get(
        C, ("0", "1", "2", "3", "4", "5", "6", "7", "8", "9", "10", "11", "12", "13", "14"))
    n_nodes = 2 * n_tips - 1
    if C > 1 and n_nodes * (C // 2) * 128 + n_tips * (C // 2) * 512 + (n_tips - 1) * 32 <= 219 * 1024:
        variants = variants + ("15", "16") + (("17",) if C < 8 else ()) + (("18",) if C > 2 else ())  # tables fit
    for v in variants:
        monkeypatch.setenv("PLK_PRUNE_VARIANT", v)
        with _engine(left, right, bl, masks, 4, Q, f, cr, cw) as h:
            assert h.loglik(plk.PLK_FP32S) == pytest.approx(orc.lnl, rel=FP32_REL)
            assert h.prune_kernel() == plk.Handle.PRUNE_KERNELS[4][int(v)]
            sites.append(h.site_loglik())
    np.testing.assert_allclose(sites[1], sites[0], rtol=1e-12)
    for s in sites[2:]:
        # the staged kernels do the same operations in the same order: the same bits
        np.testing.assert_array_equal(s, sites[1])


def test_full_size_dna_gtr_gamma_fp32_against_fp64():
    """128 taxa x 100,000 sites, GTR+Gamma4, 2% missing: FP32-scaled vs FP64
    engine vs FP64 oracle (a size-independent relative bound)."""
    w = synth.make("cfg2", seed=2)
    teff = plk.effective_lengths(w.left, w.right, w.bl, False)
    orc = O.loglik(w.left, w.right, w.masks, teff, w.Q, w.freqs, w.cat_rates, w.cat_weights,
                   p_mode=O.P_EXACT, threads=8)
    with _engine(w.left, w.right, w.bl, w.masks, 4, w.Q, w.freqs, w.cat_rates, w.cat_weights) as h:
        l64 = h.loglik(plk.PLK_FP64)
        l32 = h.loglik(plk.PLK_FP32S)
    assert l64 == pytest.approx(orc.lnl, rel=1e-11)
    assert l32 == pytest.approx(orc.lnl, rel=FP32_REL)


@pytest.mark.parametrize("n_tips,n_sites,C,shape", [(64, 2000, 4, "yule"), (7, 1, 1, "yule"), (33, 129, 8, "yule"),
                                                    (200, 300, 4, "caterpillar"), (16, 4099, 2, "yule"),
                                                    (128, 700, 4, "balanced"), (45, 257, 3, "balanced")])
def test_protein_kernel_variants(monkeypatch, n_tips, n_sites, C, shape):
    """20 states: prune20_kernel on CUDA cores (1, 3) and on mma.sync tensor
    cores with the split-TF32 products (2, 4), and on tcgen05 tensor cores
    with TMEM accumulators prune20u_kernel (5, spill stack in TMEM) and its
    compact form prune20v_kernel (6, spills in global memory; 7, with the
    split-BF16 products of kind::f16), against the
    FP64 oracle, per site; the caterpillar tree forces repeated rescaling,
    the balanced trees the deepest spill stacks, ambiguity codes the table
    look-ups."""
    rng = np.random.default_rng(n_tips * 7 + n_sites)
    left, right, bl, masks, Q, f, cr, cw = _random_case(rng, n_tips, n_sites, S=20, C=C, missing=0.03, shape=shape)
    amb = rng.random(masks.shape) < 0.02
    masks[amb] |= np.uint32(1 << 3)                          # two-state ambiguity
    teff = plk.effective_lengths(left, right, bl, False)
    orc = O.loglik(left, right, masks, teff, Q, f, cr, cw, p_mode=O.P_EXACT)
    for v in ("5", "6", "7", "1", "2", "3", "4"):
        monkeypatch.setenv("PLK_PRUNE_VARIANT", v)
        with _engine(left, right, bl, masks, 20, Q, f, cr, cw) as h:
            got = h.loglik(plk.PLK_FP32S)
            assert h.prune_kernel() == plk.Handle.PRUNE_KERNELS[20][int(v)]
            assert got == pytest.approx(orc.lnl, rel=FP32_REL), v
            # the split-BF16 products keep about 16 bits per product (the
            # split-TF32 and FP32 forms about 21 and 24): a looser per-site bound
            site_rtol = BF16_SITE_REL if v == "7" else 2e-6
            np.testing.assert_allclose(h.site_loglik(), orc.site_lnl, rtol=site_rtol, atol=1e-9)
            # the plain FP64 form stays bit-compatible with the oracle
            assert h.loglik(plk.PLK_FP64) == pytest.approx(orc.lnl, rel=1e-11)


def test_protein_autotuned_full_size():
    """64 taxa x 20,000 sites, 20 states, Gamma4: the autotuned 20-state
    kernel within 1e-6 relative of the FP64 oracle."""
    w = synth.make("cfg3", seed=3)
    teff = plk.effective_lengths(w.left, w.right, w.bl, False)
    orc = O.loglik(w.left, w.right, w.masks, teff, w.Q, w.freqs, w.cat_rates, w.cat_weights,
                   p_mode=O.P_EXACT, threads=8)
    with _engine(w.left, w.right, w.bl, w.masks, 20, w.Q, w.freqs, w.cat_rates, w.cat_weights) as h:
        assert h.loglik(plk.PLK_FP32S) == pytest.approx(orc.lnl, rel=FP32_REL)


@pytest.mark.parametrize("S,n_tips,n_sites,C", [(4, 24, 3000, 4), (20, 12, 700, 2), (4, 5, 1, 1)])
def test_site_patterns(S, n_tips, n_sites, C):
    """Pattern mode against plain mode on an alignment with many repeated
    columns: the same total (compensated weighted sum), the same per-site
    values and node states for every input site, fewer evaluated columns."""
    rng = np.random.default_rng(S * 100 + n_tips)
    left, right, bl, masks, Q, f, cr, cw = _random_case(rng, n_tips, n_sites, S=S, C=C)
    # few distinct columns: draw every column from a small pool
    pool = masks[:, : max(1, n_sites // 30)]
    masks = np.ascontiguousarray(pool[:, rng.integers(0, pool.shape[1], n_sites)])
    teff = plk.effective_lengths(left, right, bl, False)
    orc = O.loglik(left, right, masks, teff, Q, f, cr, cw, p_mode=O.P_EXACT)
    res = {}
    for on in (False, True):
        h = plk.Handle()
        h.set_patterns(on)
        h.set_alignment(masks, S)
        h.set_tree(left, right, bl)
        h.set_rate_model(False)
        h.set_model(Q, f, True, cr, cw, plk.PLK_P_EXACT)
        res[on] = (h.loglik(plk.PLK_FP64), h.site_loglik(), h.loglik(plk.PLK_FP32S), h.site_loglik(),
                   h.node_states(plk.PLK_NODES_MARGINAL, plk.PLK_FP64), h.n_patterns)
        h.close()
    assert res[False][5] == n_sites
    assert res[True][5] == len({tuple(c) for c in masks.T})
    assert res[True][0] == pytest.approx(orc.lnl, rel=1e-12)
    assert res[True][0] == pytest.approx(res[False][0], rel=1e-13)
    assert res[True][2] == pytest.approx(orc.lnl, rel=FP32_REL)
    # FP64: the same operations per column, so the same bits
    np.testing.assert_array_equal(res[True][1], res[False][1])
    np.testing.assert_array_equal(res[True][4], res[False][4])
    # FP32: the autotuner may pick another 20-state form for the other column count
    np.testing.assert_allclose(res[True][3], res[False][3], rtol=1e-6)


@pytest.mark.parametrize("variant", [9, 16])
def test_withheld_stage_times_out_and_the_handle_recovers(monkeypatch, variant):
    """Failure path of the TMA-fed post-order forms (the staged ring of
    variant 9, the bulk table copy of the shared-table variant 16): with the
    copies withheld every bounded mbarrier wait runs out, the evaluation
    reports PLK_ERR_NUMERIC, and the next evaluation on the same handle is
    exact."""
    import time
    rng = np.random.default_rng(77)
    left, right, bl, masks, Q, f, cr, cw = _random_case(rng, 24, 700, C=4)
    monkeypatch.setenv("PLK_PRUNE_VARIANT", str(variant))
    with _engine(left, right, bl, masks, 4, Q, f, cr, cw) as h:
        good = h.loglik(plk.PLK_FP32S)
        assert h.prune_kernel() == plk.Handle.PRUNE_KERNELS[4][variant]
        h.test_withhold_stage()
        t0 = time.perf_counter()
        with pytest.raises(plk.PlkError) as err:
            h.loglik(plk.PLK_FP32S)
        waited = time.perf_counter() - t0
        assert err.value.status == plk.PLK_ERR_NUMERIC
        assert waited < 120.0
        assert h.loglik(plk.PLK_FP32S) == good


@pytest.mark.parametrize("variant", [5, 6])
def test_withheld_mma_commit_times_out_and_the_handle_recovers(monkeypatch, variant):
    """Failure path of the tcgen05 20-state forms: with the first MMA commit
    withheld every bounded mbarrier wait runs out, the evaluation reports
    PLK_ERR_NUMERIC (TMEM still freed), and the next evaluation is exact."""
    import time
    rng = np.random.default_rng(78)
    left, right, bl, masks, Q, f, cr, cw = _random_case(rng, 16, 300, S=20, C=4)
    monkeypatch.setenv("PLK_PRUNE_VARIANT", str(variant))
    with _engine(left, right, bl, masks, 20, Q, f, cr, cw) as h:
        good = h.loglik(plk.PLK_FP32S)
        assert h.prune_kernel() == plk.Handle.PRUNE_KERNELS[20][variant]
        h.test_withhold_stage()
        t0 = time.perf_counter()
        with pytest.raises(plk.PlkError) as err:
            h.loglik(plk.PLK_FP32S)
        assert err.value.status == plk.PLK_ERR_NUMERIC
        assert time.perf_counter() - t0 < 120.0
        assert h.loglik(plk.PLK_FP32S) == good


def test_back_to_back_alignments_on_one_handle():
    """The byte masks travel and are encoded on the handle's copy stream:
    replacing the alignment before evaluating, or with a host-encoded
    20-state one, must leave no stale or half-written tip codes."""
    rng = np.random.default_rng(91)
    left, right, bl, m1, Q, f, cr, cw = _random_case(rng, 30, 2000, C=4)
    m2 = m1[:, ::-1].copy()
    teff = plk.effective_lengths(left, right, bl, False)
    want1 = O.loglik(left, right, m1, teff, Q, f, cr, cw, p_mode=O.P_EXACT).lnl
    want2 = O.loglik(left, right, m2, teff, Q, f, cr, cw, p_mode=O.P_EXACT).lnl
    l20, r20, b20, m20, Q20, f20, cr20, cw20 = _random_case(rng, 30, 500, S=20, C=4)
    with plk.Handle() as h:
        h.set_tree(left, right, bl)
        for _ in range(3):
            h.set_alignment(m1.astype(np.uint8), 4)
            h.set_alignment(m2.astype(np.uint8), 4)   # replaced before any evaluation
            h.set_tree(left, right, bl)
            h.set_rate_model(False)
            h.set_model(Q, f, True, cr, cw, plk.PLK_P_EXACT)
            assert h.loglik(plk.PLK_FP32S) == pytest.approx(want2, rel=FP32_REL)
            h.set_alignment(m1.astype(np.uint8), 4)
            assert h.loglik(plk.PLK_FP32S) == pytest.approx(want1, rel=FP32_REL)
        # a host-encoded 20-state alignment right after a byte-mask one
        h.set_alignment(m1.astype(np.uint8), 4)
        h.set_alignment(m20, 20)
        h.set_tree(l20, r20, b20)
        h.set_rate_model(False)
        h.set_model(Q20, f20, True, cr20, cw20, plk.PLK_P_EXACT)
        t20 = plk.effective_lengths(l20, r20, b20, False)
        want20 = O.loglik(l20, r20, m20, t20, Q20, f20, cr20, cw20, p_mode=O.P_EXACT).lnl
        assert h.loglik(plk.PLK_FP32S) == pytest.approx(want20, rel=FP32_REL)



@pytest.mark.parametrize("name", ["syn_gtr_gamma_ambig", "syn_protein20"])
def test_error_reporting_entry_points(name):
    """plk_loglik_err and plk_node_states_err: the fast form's results with
    their error against the FP64 plain form, equal to separate evaluations of
    both forms, and the FP64 form held to the oracle."""
    fx = H.load_fixture(name)
    orc = H.oracle_for_fixture(fx, p_mode=O.P_EXACT, want_marginal=True)
    with H.engine_for_fixture(fx, p_mode=plk.PLK_P_EXACT) as h:
        fast, f64, abs_err, rel_err = h.loglik_err()
        assert f64 == pytest.approx(orc.lnl, rel=1e-11)
        assert fast == h.loglik(plk.PLK_FP32S)
        assert f64 == h.loglik(plk.PLK_FP64)
        assert abs_err == abs(fast - f64) and rel_err == pytest.approx(abs_err / abs(f64), rel=1e-15)
        assert rel_err < FP32_REL
        for mode in (plk.PLK_NODES_COND, plk.PLK_NODES_MARGINAL):
            out, err = h.node_states_err(mode)
            n64 = h.node_states(mode, plk.PLK_FP64)
            n32 = h.node_states(mode, plk.PLK_FP32S)
            np.testing.assert_array_equal(out, n32)
            assert err == float(np.abs(n32 - n64).max())
            assert err < FP32_PROB
        np.testing.assert_allclose(h.node_states(plk.PLK_NODES_MARGINAL, plk.PLK_FP64), orc.marginal, atol=1e-11)


@pytest.mark.parametrize("variant", [None, "13", "16"])
def test_streamed_byte_alignment_matches_the_32bit_path(monkeypatch, variant):
    """plk_set_alignment8 with 4 states and at least 16,384 sites copies the
    masks in place as codes, in chunks each followed by an arrival flag; a
    warp-independent pass starts while they land and waits per tile.  Every
    evaluation after a fresh alignment gives the bits of the 32-bit path,
    whose codes are encoded before the pass."""
    rng = np.random.default_rng(31)
    left, right, bl, masks, Q, f, cr, cw = _random_case(rng, 40, 20000, C=4)
    if variant:
        monkeypatch.setenv("PLK_PRUNE_VARIANT", variant)
    res = []
    for m in (masks.astype(np.uint32), masks.astype(np.uint8)):
        with _engine(left, right, bl, m, 4, Q, f, cr, cw) as h:
            vals = []
            for _ in range(3):  # a fresh alignment each time (the first one tunes the form)
                h.set_alignment(m, 4)
                vals.append(h.loglik(plk.PLK_FP32S))
            res.append((vals, h.site_loglik(), h.prune_kernel()))
    np.testing.assert_array_equal(res[0][1], res[1][1])  # every FP32 form: the same per-site bits
    if res[0][2] == res[1][2]:  # the same form (the tuner may pick another on timing noise)
        assert res[0][0] == res[1][0]
    else:
        assert res[0][0] == pytest.approx(res[1][0], rel=1e-12)


def test_streamed_alignment_reports_an_empty_cell(monkeypatch):
    """The empty-cell check of a streamed alignment runs on the copy stream
    beside the pass and still turns a cell that allows no state (here the
    last site of a row) into PLK_ERR_TIP, as the encoded path does."""
    rng = np.random.default_rng(32)
    left, right, bl, masks, Q, f, cr, cw = _random_case(rng, 24, 17000, C=4)
    m8 = masks.astype(np.uint8)
    m8[5, 16999] = 0
    monkeypatch.setenv("PLK_PRUNE_VARIANT", "16")
    with _engine(left, right, bl, m8, 4, Q, f, cr, cw) as h:
        with pytest.raises(plk.PlkError) as err:
            h.loglik(plk.PLK_FP32S)
        assert err.value.status == plk.PLK_ERR_TIP


def test_streamed_arrival_wait_times_out_and_the_handle_recovers(monkeypatch):
    """Failure path of the per-tile arrival wait: with the arrival withheld
    (the test hook waits for a generation no copy writes) every tile's
    bounded wait runs out, the evaluation reports PLK_ERR_NUMERIC, and the
    next evaluation on the same handle is exact."""
    import time
    rng = np.random.default_rng(33)
    left, right, bl, masks, Q, f, cr, cw = _random_case(rng, 24, 17000, C=4)
    monkeypatch.setenv("PLK_PRUNE_VARIANT", "13")  # tables through L1: no table copy to withhold first
    m8 = masks.astype(np.uint8)
    with _engine(left, right, bl, m8, 4, Q, f, cr, cw) as h:
        good = h.loglik(plk.PLK_FP32S)
        h.set_alignment(m8, 4)
        h.test_withhold_stage()
        t0 = time.perf_counter()
        with pytest.raises(plk.PlkError) as err:
            h.loglik(plk.PLK_FP32S)
        assert err.value.status == plk.PLK_ERR_NUMERIC
        assert time.perf_counter() - t0 < 120.0
        assert h.loglik(plk.PLK_FP32S) == good


def test_streamed_masks_with_bits_past_the_alphabet():
    """Bits past the 4 states in a byte mask mean nothing (the encoded path
    drops them), but a streamed alignment's codes are the caller's bytes, so
    every reader masks them: the FP32 and FP64 lnL, the per-site values and
    the node states (post-order FP64 and the pre-order marginals) carry the
    bits of the 32-bit path."""
    rng = np.random.default_rng(34)
    left, right, bl, masks, Q, f, cr, cw = _random_case(rng, 30, 17000, C=4)
    out = []
    for m in (masks.astype(np.uint32), (masks.astype(np.uint8) | np.uint8(0xF0))):
        with _engine(left, right, bl, m, 4, Q, f, cr, cw) as h:
            r = [h.loglik(plk.PLK_FP32S)]
            h.set_alignment(m, 4)  # streamed again (the first evaluation tuned the form)
            r.append(h.loglik(plk.PLK_FP32S))
            r.append(h.site_loglik())
            r.append(h.loglik(plk.PLK_FP64))
            r.append(h.node_states(plk.PLK_NODES_COND, plk.PLK_FP64))
            r.append(h.node_states(plk.PLK_NODES_MARGINAL, plk.PLK_FP64))
            out.append(r)
    a, b = out
    assert a[0] == b[0] and a[1] == b[1] and a[3] == b[3]
    for x, y in zip(a[2:], b[2:]):
        np.testing.assert_array_equal(x, y)
