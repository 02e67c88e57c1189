"""The FP64 network oracle checked against itself: analytic back-propagation
against central differences, the bfloat16 rounding against its definition,
and the host-side pieces of the warm start that need no device."""
import numpy as np

from oracle import mlp as M
from phylommand_gb300 import warmstart


def _net(seed, dims):
    rng = np.random.default_rng(seed)
    p = rng.normal(0.0, 0.5, M.n_params(dims))
    x = rng.normal(size=(9, dims[0]))
    t = rng.normal(size=(9, dims[-1]))
    return p, x, t


def test_analytic_gradient_matches_finite_differences():
    dims = [5, 7, 6, 3]
    p, x, t = _net(1, dims)
    loss, g = M.loss_and_grad(p, dims, x, t)
    assert np.isclose(loss, np.mean((M.forward(p, dims, x)[0] - t) ** 2))
    idx = np.arange(M.n_params(dims))
    fd = M.finite_difference(p, dims, x, t, idx)
    np.testing.assert_allclose(g, fd, rtol=1e-6, atol=1e-8)


def test_gradient_of_a_linear_layer_is_closed_form():
    dims = [4, 2]
    p, x, t = _net(2, dims)
    W, b = M.unpack(p, dims)[0]
    y = x @ W.T + b
    d = 2 * (y - t) / y.size
    _, g = M.loss_and_grad(p, dims, x, t)
    np.testing.assert_allclose(g[:8].reshape(2, 4), d.T @ x, rtol=1e-12)
    np.testing.assert_allclose(g[8:], d.sum(0), rtol=1e-12)


def test_bf16_rounding():
    # exactly representable values stay, halfway cases go to even
    assert M.bf16(1.0) == 1.0
    assert M.bf16(1.0 + 2 ** -8) == 1.0                 # halfway, even mantissa below
    assert M.bf16(1.0 + 3 * 2 ** -8) == 1.0 + 2 ** -6    # halfway, odd below: up
    assert M.bf16(1.0 + 2 ** -7) == 1.0 + 2 ** -7
    assert M.bf16(-2.5) == -2.5
    r = np.random.default_rng(3).normal(size=1000)
    assert np.all(np.abs(M.bf16(r) - r) <= np.abs(r) * 2 ** -8)


def test_adam_first_step_moves_by_lr():
    p = np.array([1.0, -2.0, 0.5])
    g = np.array([0.3, -4.0, 1e-3])
    p1, m, v = M.adam(p, g, np.zeros(3), np.zeros(3), 1, 0.01)
    np.testing.assert_allclose(p1, p - 0.01 * np.sign(g), rtol=1e-4)


def test_parameter_count_of_the_warm_start_network():
    dims = [warmstart.N_FEATURES, 256, 256, 256, warmstart.N_PARAMS]
    assert M.n_params(dims) == 43 * 256 + 256 + 2 * (256 * 256 + 256) + 256 * 7 + 7


def test_empirical_frequencies_are_floored_and_normalised():
    f = np.zeros((2, 43), dtype=np.float32)
    f[0, :4] = [0.5, 0.5, 0.0, 0.0]
    f[1, :4] = [0.1, 0.2, 0.3, 0.4]
    e = warmstart.empirical_freqs(f)
    np.testing.assert_allclose(e.sum(1), 1.0)
    assert np.all(e > 0)
    np.testing.assert_allclose(e[1], [0.1, 0.2, 0.3, 0.4], rtol=1e-6)
