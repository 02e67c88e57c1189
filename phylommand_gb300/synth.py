"""Seeded synthetic workloads (the reference's own simulator, simpleML::
simulate_chars at src/simpleML.cpp:233-292, draws from rand() seeded by the
clock; this one is reproducible from a seed).

* Yule topology: repeatedly join two uniformly chosen lineages.
* Branch lengths: i.i.d. Exponential(mean).
* Sequences: simulated down the tree, one rate category per site drawn
  uniformly.

Two backends make the same shapes and distributions:
  "engine"  Q, Gamma rates, P(t) and the simulation from libplk (the native
            seeded multithreaded simulator, ``plk_simulate``);
  "numpy"   the same quantities in numpy / scipy only (Q by the sub_model
            formula, Yang's mean-per-category Gamma rates from scipy's
            incomplete gamma, P(t) by a symmetric eigendecomposition, the
            simulation vectorised over sites), so a process that must not load
            libplk -- the benchmark's reference arm -- builds the identical
            workload, and the engine's arm uses it too.

Node numbering follows the C ABI: tips 0..n-1 (alignment rows), internal
nodes n..2n-2 in creation order (children before parents), root last.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class Workload:
    name: str
    left: np.ndarray
    right: np.ndarray
    bl: np.ndarray
    masks: np.ndarray          # uint32 [n_tips, n_sites]
    n_states: int
    Q: np.ndarray
    freqs: np.ndarray
    cat_rates: np.ndarray
    cat_weights: np.ndarray
    exchange: np.ndarray
    alpha: float | None
    seed: int
    info: dict = field(default_factory=dict)

    @property
    def n_tips(self) -> int:
        return int(self.masks.shape[0])

    @property
    def n_sites(self) -> int:
        return int(self.masks.shape[1])

    @property
    def n_nodes(self) -> int:
        return int(self.left.shape[0])


def yule_tree(n_tips: int, mean_bl: float, rng: np.random.Generator):
    n_nodes = 2 * n_tips - 1
    left = np.full(n_nodes, -1, dtype=np.int32)
    right = np.full(n_nodes, -1, dtype=np.int32)
    lineages = list(range(n_tips))
    nxt = n_tips
    while len(lineages) > 1:
        i, j = rng.choice(len(lineages), size=2, replace=False)
        a, b = lineages[i], lineages[j]
        left[nxt], right[nxt] = a, b
        for idx in sorted((i, j), reverse=True):
            lineages.pop(idx)
        lineages.append(nxt)
        nxt += 1
    bl = rng.exponential(mean_bl, size=n_nodes)
    bl[n_nodes - 1] = 0.0
    return left, right, bl


def reversible_q(n_states: int, exchange: np.ndarray, freqs: np.ndarray, normalise: bool = True,
                 backend: str = "engine") -> np.ndarray:
    """Q through the engine's sub_model-style builder (or its numpy
    restatement), rate spec = identity (upper triangle row-major),
    optionally normalised to mean rate 1."""
    npos = n_states * (n_states - 1) // 2
    if backend == "engine":
        from . import plk
        Q = plk.q_matrix(n_states, True, np.arange(npos), exchange, freqs[:-1])
    else:
        # Q_ij = r_pos(i,j) pi_j, the last frequency 1 - sum of the others,
        # Q_ii = -sum of the row (src/sub_model.cpp:44-53, 99-114)
        pi = np.append(np.asarray(freqs[:-1], dtype=np.float64), 1.0 - float(np.sum(freqs[:-1])))
        R = np.zeros((n_states, n_states))
        iu = np.triu_indices(n_states, 1)
        R[iu] = np.asarray(exchange, dtype=np.float64)[:npos]
        R = R + R.T
        Q = R * pi[None, :]
        np.fill_diagonal(Q, 0.0)
        np.fill_diagonal(Q, -Q.sum(axis=1))
    if normalise:
        mu = -float(np.dot(freqs, np.diag(Q)))
        Q = Q / mu
    return Q


def discrete_gamma_numpy(alpha: float, K: int) -> np.ndarray:
    """Mean rate of each of K equal-probability categories of Gamma(alpha,
    rate alpha) (Yang 1994): r_k = K [I(b_k alpha, alpha + 1) - I(a_k alpha,
    alpha + 1)] with a_k, b_k the k/K and (k+1)/K quantiles and I the
    regularised lower incomplete gamma function."""
    from scipy import special
    q = special.gammaincinv(alpha, np.arange(1, K) / K) / alpha
    cdf1 = np.concatenate(([0.0], special.gammainc(alpha + 1.0, q * alpha), [1.0]))
    return K * np.diff(cdf1)


def pmat_numpy(Q: np.ndarray, t: float, freqs: np.ndarray) -> np.ndarray:
    """exp(Q t) of a reversible Q: eigendecomposition of the symmetric
    D^1/2 Q D^-1/2 (D = diag(freqs))."""
    d = np.sqrt(np.asarray(freqs, dtype=np.float64))
    A = Q * d[:, None] / d[None, :]
    A = 0.5 * (A + A.T)
    lam, V = np.linalg.eigh(A)
    return (V / d[:, None]) @ np.diag(np.exp(lam * t)) @ (V.T * d[None, :])


def simulate(left, right, bl, Q, freqs, cat_rates, n_sites: int, rng: np.random.Generator,
             backend: str = "engine"):
    """State indices [n_tips, n_sites] simulated down the tree."""
    n_nodes = left.shape[0]
    n_tips = int(np.sum((left < 0) & (right < 0)))
    S = Q.shape[0]
    C = len(cat_rates)
    cat = rng.integers(0, C, size=n_sites)
    states = np.zeros((n_nodes, n_sites), dtype=np.int64)
    root = n_nodes - 1
    cum_pi = np.cumsum(freqs)
    cum_pi[-1] = 1.0
    states[root] = np.searchsorted(cum_pi, rng.random(n_sites), side="right")
    # internal nodes are numbered children-first, so descending ids is pre-order
    for u in range(n_nodes - 1, n_tips - 1, -1):
        for v in (left[u], right[u]):
            if v < 0:
                continue
            cumP = np.empty((C, S, S))
            for k in range(C):
                if backend == "engine":
                    from . import plk
                    P = plk.pmat_host(Q, bl[v] * cat_rates[k], plk.PLK_P_EXACT, freqs, True)
                else:
                    P = pmat_numpy(Q, bl[v] * cat_rates[k], freqs)
                P = np.clip(P, 0.0, None)
                P /= P.sum(axis=1, keepdims=True)
                cumP[k] = np.cumsum(P, axis=1)
                cumP[k][:, -1] = 1.0
            rows = cumP[cat, states[u]]                      # [n_sites, S]
            u01 = rng.random(n_sites)
            states[v] = np.minimum((u01[:, None] >= rows).sum(axis=1), S - 1)
    return states[:n_tips]


def to_masks(states: np.ndarray) -> np.ndarray:
    return (np.uint32(1) << states.astype(np.uint32)).astype(np.uint32)


def _model(rng, S, exch_kind, dirichlet, alpha, K, backend):
    npos = S * (S - 1) // 2
    if exch_kind == "uniform":
        exch = rng.uniform(0.5, 5.0, size=npos)
    elif exch_kind == "lognormal":
        exch = rng.lognormal(0.0, 1.0, size=npos)
    else:
        exch = np.ones(npos)
    freqs = rng.dirichlet(np.full(S, dirichlet)) if dirichlet else np.full(S, 1.0 / S)
    if alpha is None:
        cat_rates = np.ones(1)
    elif backend == "engine":
        from . import plk
        cat_rates = plk.discrete_gamma(alpha, K)
    else:
        cat_rates = discrete_gamma_numpy(alpha, K)
    cat_w = np.full(len(cat_rates), 1.0 / len(cat_rates))
    return exch, freqs, cat_rates, cat_w


def make(name: str, seed: int = 1, n_sites: int | None = None, n_tips: int | None = None,
         backend: str = "engine") -> Workload:
    """Seeded workloads of the benchmark shapes (backend: "engine" or
    "numpy", see the module docstring).

    cfg1   16 tips, Exp(mean 0.1), 1,000 DNA sites, JC69 (rates 4/3, freqs 1/4)
    cfg2   128 tips, Exp(mean 0.05), 100,000 DNA sites, GTR exch. U(0.5,5),
           freqs Dir(10^4), Gamma alpha 0.5 in 4 categories, 2% missing cells
    cfg3   64 tips, Exp(mean 0.1), 20,000 sites of 20 states, exch.
           LogNormal(0,1), freqs Dir(5^20), Gamma alpha 1.0 in 4 categories
    """
    rng = np.random.default_rng(seed)
    if name == "cfg1":
        n, mean, N, S = 16, 0.1, 1000, 4
        exch, freqs, cr, cw = np.ones(6), np.full(4, 0.25), np.ones(1), np.ones(1)
        Q = reversible_q(4, exch * (4.0 / 3.0), freqs, normalise=False, backend=backend)
        missing = 0.0
        alpha = None
        exch = exch * (4.0 / 3.0)
    elif name == "cfg2":
        n, mean, N, S = 128, 0.05, 100_000, 4
        alpha = 0.5
        exch, freqs, cr, cw = _model(rng, S, "uniform", 10.0, alpha, 4, backend)
        Q = reversible_q(S, exch, freqs, backend=backend)
        missing = 0.02
    elif name == "cfg3":
        n, mean, N, S = 64, 0.1, 20_000, 20
        alpha = 1.0
        exch, freqs, cr, cw = _model(rng, S, "lognormal", 5.0, alpha, 4, backend)
        Q = reversible_q(S, exch, freqs, backend=backend)
        missing = 0.0
    else:
        raise ValueError(f"unknown workload {name}")
    if n_sites is not None:
        N = int(n_sites)
    if n_tips is not None:
        n = int(n_tips)
    left, right, bl = yule_tree(n, mean, rng)
    sim_seed = int(rng.integers(1 << 62))
    if backend == "engine":
        from . import plk
        masks = plk.simulate(left, right, bl, Q, freqs, cr, N, seed=sim_seed)
    else:
        masks = to_masks(simulate(left, right, bl, Q, freqs, cr, N, np.random.default_rng(sim_seed),
                                  backend="numpy"))
    if missing > 0:
        hole = rng.random(masks.shape) < missing
        masks[hole] = np.uint32((1 << S) - 1)
    return Workload(name, left, right, bl, masks, S, Q, freqs, cr, cw, exch, alpha, seed,
                    {"mean_bl": mean, "missing": missing})
