"""CPU-only checks of libplk: the library loads, exports every symbol that
include/plk.h declares, and its host-side FP64 model code agrees with the
oracle (no kernel is launched here)."""
import os
import re

import numpy as np
import pytest

from oracle import oracle as O
from phylommand_gb300 import plk
import helpers as H

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            text = open(os.path.join(ROOT, "include", fn)).read()
            names |= set(re.findall(r"^\s*(?:[\w\*]+\s+)+\**(plk_\w+)\s*\(", text, flags=re.M))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    lib = plk.lib()
    names = declared_symbols()
    assert len(names) >= 17
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(plk.EXPORTS) <= set(names)
    assert lib.plk_api_version() == 1


def test_status_strings():
    lib = plk.lib()
    for s in range(0, -10, -1):
        assert lib.plk_status_string(s)


def test_create_reports_missing_device():
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(plk.PlkError) as e:
        plk.Handle()
    assert e.value.status == plk.PLK_ERR_NODEV


@pytest.mark.parametrize("S,tr", [(2, True), (4, True), (4, False), (5, True), (20, True), (3, False)])
def test_q_matrix_bitwise_against_oracle(S, tr):
    rng = np.random.default_rng(S * 10 + tr)
    npos = S * (S - 1) // (2 if tr else 1)
    spec = np.minimum(np.arange(npos), rng.integers(0, npos, npos))
    spec = np.unique(spec, return_inverse=True)[1]  # parameters named in order
    rates = rng.uniform(0.1, 5, spec.max() + 1)
    freqs = rng.dirichlet(np.ones(S))[:-1]
    for i in range(S):
        for j in range(S):
            assert plk.lib().plk_q_matrix is not None
            if i != j:
                assert O.rate_pos(S, tr, i, j) < npos
    Qa = plk.q_matrix(S, tr, spec, rates, freqs)
    Qb = O.q_matrix(S, tr, spec, rates, freqs)
    assert np.array_equal(Qa, Qb)


def test_q_matrix_matches_reference_fixture():
    fx = H.load_fixture("ex_gtr100")
    assert np.array_equal(plk.q_matrix(4, True, range(6), [1, 2, 3, 4, 5, 6], [0.1, 0.2, 0.3]), fx["Q"])


@pytest.mark.parametrize("name", ["ex_gtr100", "syn_protein20", "syn_nontr"])
def test_host_taylor20_bitwise_against_reference(name):
    fx = H.load_fixture(name)
    for t, P in zip(fx["pmat_t"], fx["pmat"]):
        assert np.array_equal(plk.pmat_host(fx["Q"], float(t), plk.PLK_P_TAYLOR20), P)


def test_host_exact_pmat_against_scipy():
    from scipy.linalg import expm
    rng = np.random.default_rng(9)
    for S in (2, 4, 7, 20, 24):
        f = rng.dirichlet(np.ones(S) * 2)
        npos = S * (S - 1) // 2
        Q = plk.q_matrix(S, True, np.arange(npos), rng.lognormal(0, 1, npos), f[:-1])
        Qn = plk.q_matrix(S, False, np.arange(S * S - S), rng.uniform(0.05, 2, S * S - S))
        for t in (1e-5, 0.03, 0.4, 3.0):
            np.testing.assert_allclose(plk.pmat_host(Q, t, plk.PLK_P_EXACT, f, True), expm(Q * t), atol=2e-13, rtol=0)
            np.testing.assert_allclose(plk.pmat_host(Qn, t, plk.PLK_P_EXACT, None, False), expm(Qn * t), atol=2e-13, rtol=0)


@pytest.mark.parametrize("alpha", [0.05, 0.3, 0.5, 1.0, 4.0, 50.0])
@pytest.mark.parametrize("K", [1, 2, 4, 8])
def test_discrete_gamma_against_oracle(alpha, K):
    a = plk.discrete_gamma(alpha, K)
    b = O.discrete_gamma(alpha, K)
    np.testing.assert_allclose(a, b, rtol=1e-9, atol=1e-14)
    assert a.mean() == pytest.approx(1.0, abs=1e-12)


def test_effective_lengths_against_oracle_and_reference():
    fx = H.load_fixture("syn_ratemodel")
    con = fx["clade_of_node"]
    a = plk.effective_lengths(fx["left"], fx["right"], fx["bl"], True, fx["cut_off"], fx["cut_rate"], con, fx["clade_rate"])
    assert np.array_equal(a, H.fixture_teff(fx))
    fx = H.load_fixture("syn_multifurc")
    a = plk.effective_lengths(fx["left"], fx["right"], fx["bl"], True)
    b = O.effective_lengths(fx["left"], fx["right"], fx["bl"])
    assert np.array_equal(a, b)
    assert (a == 0).sum() > 2  # root children and the edges under a zero-length root child
    c = plk.effective_lengths(fx["left"], fx["right"], fx["bl"], False)
    internal_root = int(np.where(~np.isin(np.arange(len(a)), np.r_[fx["left"], fx["right"]]))[0][0])
    mask = np.arange(len(c)) != internal_root
    assert np.array_equal(c[mask], fx["bl"][mask])


def test_effective_lengths_rejects_bad_trees():
    with pytest.raises(plk.PlkError):
        plk.effective_lengths([-1, -1, 0], [-1, -1, 0], [0.1, 0.1, 0.0])  # a node with one child twice
    with pytest.raises(plk.PlkError):
        plk.effective_lengths([1, -1, 1], [-1, -1, 0], [0.1, 0.1, 0.0])  # tip id with children


def test_discrete_gamma_rejects_bad_alpha():
    with pytest.raises(plk.PlkError):
        plk.discrete_gamma(0.0, 4)
    with pytest.raises(plk.PlkError):
        plk.discrete_gamma(1.0, 0)


def test_simulator_is_seeded_and_follows_the_model():
    from phylommand_gb300 import synth
    rng = np.random.default_rng(3)
    left, right, bl = synth.yule_tree(20, 0.1, rng)
    f = rng.dirichlet(np.full(4, 5.0))
    Q = synth.reversible_q(4, rng.uniform(0.5, 4, 6), f)
    cr = plk.discrete_gamma(0.7, 4)
    a = plk.simulate(left, right, bl, Q, f, cr, 20000, seed=11, threads=1)
    b = plk.simulate(left, right, bl, Q, f, cr, 20000, seed=11, threads=7)
    c = plk.simulate(left, right, bl, Q, f, cr, 20000, seed=12, threads=7)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    freq = np.bincount(np.log2(a.ravel()).astype(int), minlength=4) / a.size
    np.testing.assert_allclose(freq, f, atol=0.01)
    # two tips joined by a path of length t: P(same state) = sum_i pi_i P_ii(t)
    L2 = np.array([-1, -1, 0]); R2 = np.array([-1, -1, 1]); B2 = np.array([0.15, 0.25, 0.0])
    m = plk.simulate(L2, R2, B2, Q, f, np.ones(1), 200000, seed=5)
    same = np.mean(m[0] == m[1])
    P = plk.pmat_host(Q, 0.4, plk.PLK_P_EXACT, f, True)
    expect = float(np.dot(f, np.diag(P)))
    assert abs(same - expect) < 4 * np.sqrt(expect * (1 - expect) / 200000)
