"""The engine's Nelder-Mead ML fit (the likelihood calls of treeator's NLopt
optimisation).  NLopt itself is absent, so the optimiser is judged on its
final lnL: it must match an independent optimiser (scipy's Nelder-Mead)
driving the FP64 oracle to within 1e-3, and beat the generating parameters."""
import numpy as np
import pytest

from oracle import oracle as O
from phylommand_gb300 import plk, synth

pytestmark = pytest.mark.gpu


def _simulated(seed=5, n_tips=20, n_sites=3000):
    rng = np.random.default_rng(seed)
    left, right, bl = synth.yule_tree(n_tips, 0.08, rng)
    exch = rng.uniform(0.5, 5.0, 6)
    freqs = rng.dirichlet(np.full(4, 10.0))
    Q = synth.reversible_q(4, exch, freqs)
    cr = plk.discrete_gamma(0.5, 4)
    states = synth.simulate(left, right, bl, Q, freqs, cr, n_sites, rng)
    return left, right, bl, synth.to_masks(states), freqs, exch


def _oracle_negll(x, left, right, bl, masks, freqs):
    exch = np.append(np.exp(x[:5]), 1.0)
    Q = O.q_matrix(4, True, range(6), exch, freqs[:3])
    mu = -float(np.dot(freqs, np.diag(Q)))
    Q = Q / mu
    alpha, scale = np.exp(x[5]), np.exp(x[6])
    if not (1e-4 < alpha < 1e4):
        return np.inf
    cr = O.discrete_gamma(alpha, 4) * scale
    teff = O.effective_lengths(left, right, bl, root_dist0=1e-30)
    return -O.loglik(left, right, masks, teff, Q, freqs, cr, np.full(4, 0.25), p_mode=O.P_EXACT, threads=8).lnl


@pytest.mark.parametrize("precision", [plk.PLK_FP64, plk.PLK_FP32S])
def test_fit_matches_independent_optimiser(precision):
    from scipy.optimize import minimize
    left, right, bl, masks, freqs, exch = _simulated()
    with plk.Handle() as h:
        h.set_alignment(masks, 4)
        h.set_tree(left, right, bl)
        h.set_rate_model(False)
        x, lnl, n_evals = h.fit_gtr(freqs, 4, precision=precision, ftol=1e-6, xtol=1e-4, max_evals=4000)
    assert 20 < n_evals < 4000
    # the engine's optimum, re-scored by the oracle
    assert -_oracle_negll(x, left, right, bl, masks, freqs) == pytest.approx(lnl, abs=1e-6 if precision == plk.PLK_FP64 else 2e-3)
    ref = minimize(_oracle_negll, np.zeros(7), args=(left, right, bl, masks, freqs), method="Nelder-Mead",
                   options={"xatol": 1e-5, "fatol": 1e-7, "maxfev": 6000, "maxiter": 6000,
                            "initial_simplex": np.vstack([np.zeros(7), 0.5 * np.eye(7)])})
    assert lnl == pytest.approx(-ref.fun, abs=1e-3)
    # the ML estimate is at least as likely as the generating parameters
    x_true = np.r_[np.log(exch[:5] / exch[5]), np.log(0.5), 0.0]
    assert lnl >= -_oracle_negll(x_true, left, right, bl, masks, freqs) - 1e-6


def test_fit_from_a_warm_start_takes_fewer_evaluations():
    left, right, bl, masks, freqs, exch = _simulated(seed=8)
    with plk.Handle() as h:
        h.set_alignment(masks, 4)
        h.set_tree(left, right, bl)
        h.set_rate_model(False)
        x_cold, l_cold, n_cold = h.fit_gtr(freqs, 4, ftol=1e-6, xtol=1e-4)
        x_warm, l_warm, n_warm = h.fit_gtr(freqs, 4, x0=x_cold + 0.01, step=0.05, ftol=1e-6, xtol=1e-4)
    assert l_warm == pytest.approx(l_cold, abs=1e-3)
    assert n_warm < n_cold


@pytest.mark.parametrize("method", [plk.PLK_FIT_QUASI_NEWTON, plk.PLK_FIT_NEWTON_START])
def test_quasi_newton_fit_reaches_the_nelder_mead_optimum(method):
    """The quasi-Newton optimisers end at (or above) the Nelder-Mead optimum
    in far fewer evaluations, on one handle and in a batch."""
    left, right, bl, masks, freqs, exch = _simulated(seed=9)
    with plk.Handle() as h:
        h.set_alignment(masks, 4)
        h.set_tree(left, right, bl)
        h.set_rate_model(False)
        _, l_nm, n_nm = h.fit_gtr(freqs, 4, ftol=1e-6, xtol=1e-4)
        h.set_fit_method(method)
        x_qn, l_qn, n_qn = h.fit_gtr(freqs, 4, ftol=1e-6, xtol=1e-4)
        with pytest.raises(plk.PlkError):
            h.set_fit_method(7)
    assert l_qn >= l_nm - 1e-3
    assert n_qn < n_nm
    # the same fit in a batch of three copies: each item as on its own
    with plk.Batch(4) as b:
        for _ in range(3):
            b.add(masks, left, right, bl)
        b.set_fit_method(method)
        fit = b.fit_gtr(np.tile(freqs, (3, 1)), None, 0.5, 1e-6, 1e-4, 4000)
    assert np.all(fit.lnl >= l_nm - 1e-3)
    assert np.all(fit.evals == fit.evals[0]) and fit.evals[0] < n_nm
