"""Learned warm start for the GTR+Gamma maximum-likelihood fit.

The reference maximises lnL with NLopt's Nelder-Mead from fixed starting
values -- every free rate 1.0 (src/treeator.cpp:612-615, the optimiser at
:791-805).  Here a small network maps summary statistics of an alignment
(``plk_batch_features``: base frequencies, substitution-type proportions,
site-entropy histogram, mean p-distance) to a starting point of the same fit
(``plk_batch_fit_gtr``: 5 log exchangeabilities relative to C<->T, log Gamma
shape, log tree-length scale).

Pipeline, every step on the GPU through libplk:
  1. simulate alignments on Yule trees under GTR+Gamma parameters drawn from
     the priors below (``plk_simulate``);
  2. label them with the plain fit from the default start (all
     exchangeabilities 1, alpha 1, scale 1) -- the network learns the ML
     point the GPU likelihood itself finds;
  3. train the network (``plk_mlp_*``: BF16 tensor-core GEMMs, FP32
     accumulation, Adam) on standardised features and labels;
  4. fit new alignments from the predicted start.  The default start stays
     the fallback: both starts are scored first and the better one is used.

The fits use the quasi-Newton optimiser with a finite-difference Hessian at
the start (``PLK_FIT_NEWTON_START``): its first step is a Newton step, so a
start close to the optimum pays off; with Nelder-Mead (linear convergence, the
reference's NLopt method) most evaluations go into the last decades of
convergence whatever the start, and the comparison is reported beside it.

The tree handed to the fit carries the simulated topology with branch lengths
rescaled to a mean pairwise (tip-to-tip) path length of ``INPUT_MEAN_PATH``,
so the tree-length scale is a real unknown; because the features are pairwise
statistics and the scale is relative to the mean pairwise path, a network
trained on 32-taxon alignments applies to alignments of other sizes.
"""
from __future__ import annotations

import argparse
import json
import os
import time
from dataclasses import dataclass

import numpy as np

from . import plk, synth

N_CATS = 4
N_PARAMS = 7          # 5 log exchangeabilities, log alpha, log tree-length scale
N_FEATURES = 43
INPUT_MEAN_PATH = 0.5
DEFAULT_STEP = 0.5

# priors of the simulated training and evaluation alignments
EXCH_RANGE = (0.5, 5.0)        # each of AG, AC, AT, GC, GT, CT ~ U
FREQ_DIRICHLET = 10.0          # base frequencies ~ Dir(10, 10, 10, 10)
ALPHA_RANGE = (0.2, 5.0)       # Gamma shape ~ log-uniform
MEAN_BL_RANGE = (0.02, 0.2)    # mean branch length ~ log-uniform


def _loguniform(rng, lo, hi):
    return float(np.exp(rng.uniform(np.log(lo), np.log(hi))))


def mean_pairwise_path(left, right, bl) -> float:
    """Mean tip-to-tip path length: every edge lies on k (n - k) of the
    n (n - 1) / 2 tip pairs, k the tips below it."""
    left = np.asarray(left)
    right = np.asarray(right)
    n_nodes = left.shape[0]
    tips = np.zeros(n_nodes, dtype=np.int64)
    is_tip = (left < 0) & (right < 0)
    tips[is_tip] = 1
    parent = np.full(n_nodes, -1)
    for v in range(n_nodes):
        for c in (left[v], right[v]):
            if c >= 0:
                parent[c] = v
    # tip counts accumulate upwards: deepest nodes first
    depth = np.zeros(n_nodes, dtype=np.int64)
    for v in range(n_nodes):
        u = v
        while parent[u] >= 0:
            u = parent[u]
            depth[v] += 1
    for v in np.argsort(-depth, kind="stable"):
        if parent[v] >= 0:
            tips[parent[v]] += tips[v]
    n = int(is_tip.sum())
    k = tips[parent >= 0]
    w = np.asarray(bl, dtype=np.float64)[parent >= 0]
    return float(np.sum(w * k * (n - k)) / (n * (n - 1) / 2))


def simulate_batch(n_items: int, n_taxa: int, n_sites: int, seed: int, only=None):
    """A plk.Batch of ``n_items`` simulated alignments and the generating
    parameters of each in the fit's parameterisation, shape [n_items, 7].
    With ``only`` (item indices, ascending), the batch holds just those items
    -- the same alignments as in the full batch, since every item's draws
    are made whether it is kept or not -- and truth has their rows."""
    rng = np.random.default_rng(seed)
    b = plk.Batch(N_CATS)
    keep = None if only is None else set(int(i) for i in only)
    truth = np.zeros((n_items, N_PARAMS))
    for i in range(n_items):
        exch = rng.uniform(*EXCH_RANGE, size=6)
        freqs = rng.dirichlet(np.full(4, FREQ_DIRICHLET))
        alpha = _loguniform(rng, *ALPHA_RANGE)
        mean_bl = _loguniform(rng, *MEAN_BL_RANGE)
        left, right, bl = synth.yule_tree(n_taxa, mean_bl, rng)
        sim_seed = int(rng.integers(1 << 62))
        path = mean_pairwise_path(left, right, bl)
        truth[i, :5] = np.log(exch[:5] / exch[5])
        truth[i, 5] = np.log(alpha)
        truth[i, 6] = np.log(path / INPUT_MEAN_PATH)
        if keep is not None and i not in keep:
            continue
        Q = synth.reversible_q(4, exch, freqs)
        cr = plk.discrete_gamma(alpha, N_CATS)
        masks = plk.simulate(left, right, bl, Q, freqs, cr, n_sites, seed=sim_seed)
        b.add(masks, left, right, bl * (INPUT_MEAN_PATH / path))
    if keep is not None:
        truth = truth[sorted(keep)]
    return b, truth


def empirical_freqs(features: np.ndarray) -> np.ndarray:
    """The fixed base frequencies of the fits: the observed ones, floored."""
    f = np.maximum(features[:, :4].astype(np.float64), 1e-6)
    return f / f.sum(axis=1, keepdims=True)


@dataclass
class LabelledSet:
    features: np.ndarray   # [n, 43] float32
    freqs: np.ndarray      # [n, 4]
    truth: np.ndarray      # [n, 7] generating parameters
    labels: np.ndarray     # [n, 7] ML fit from the default start
    lnl: np.ndarray        # [n]
    evals: np.ndarray      # [n]
    fit_s: float

    def save(self, path: str) -> None:
        np.savez(path, features=self.features, freqs=self.freqs, truth=self.truth, labels=self.labels,
                 lnl=self.lnl, evals=self.evals, fit_s=self.fit_s)

    @staticmethod
    def load(path: str) -> "LabelledSet":
        z = np.load(path)
        return LabelledSet(z["features"], z["freqs"], z["truth"], z["labels"], z["lnl"], z["evals"],
                           float(z["fit_s"]))


def make_labelled(n_items: int, n_taxa: int, n_sites: int, seed: int, ftol: float = 1e-4, xtol: float = 1e-3,
                  max_evals: int = 4000, method: int = plk.PLK_FIT_NEWTON_START) -> LabelledSet:
    """Simulate, extract features and label with the plain GPU ML fit."""
    b, truth = simulate_batch(n_items, n_taxa, n_sites, seed)
    try:
        b.set_fit_method(method)
        feats = b.features()
        freqs = empirical_freqs(feats)
        t0 = time.perf_counter()
        fit = b.fit_gtr(freqs, None, DEFAULT_STEP, ftol, xtol, max_evals)
        fit_s = time.perf_counter() - t0
    finally:
        b.close()
    return LabelledSet(feats, freqs, truth, fit.x, fit.lnl, fit.evals, fit_s)


class WarmStart:
    """The trained network with its input/output standardisation and the
    initial simplex steps (one per parameter) used from its predictions."""

    def __init__(self, net: plk.MLP, x_mean, x_std, y_mean, y_std, step):
        self.net = net
        self.x_mean, self.x_std = np.asarray(x_mean, np.float32), np.asarray(x_std, np.float32)
        self.y_mean, self.y_std = np.asarray(y_mean, np.float32), np.asarray(y_std, np.float32)
        self.step = np.broadcast_to(np.asarray(step, np.float64), (N_PARAMS,)).copy()

    def predict(self, features) -> np.ndarray:
        z = (np.asarray(features, np.float32) - self.x_mean) / self.x_std
        return (self.net.forward(z) * self.y_std + self.y_mean).astype(np.float64)

    def save(self, path: str) -> None:
        np.savez(path, params=self.net.get_params(), x_mean=self.x_mean, x_std=self.x_std, y_mean=self.y_mean,
                 y_std=self.y_std, step=self.step,
                 shape=np.array([self.net.n_in, self.net.n_out, self.net.n_hidden, self.net.n_hidden_layers]))

    @staticmethod
    def load(path: str, device: int = 0) -> "WarmStart":
        z = np.load(path)
        n_in, n_out, n_hidden, layers = (int(v) for v in z["shape"])
        net = plk.MLP(n_in, n_out, n_hidden, layers, device=device)
        net.set_params(z["params"])
        return WarmStart(net, z["x_mean"], z["x_std"], z["y_mean"], z["y_std"], z["step"])


def train(data: LabelledSet, epochs: int = 200, batch: int = 256, lr: float = 1e-3, seed: int = 0,
          val_frac: float = 0.1, n_hidden: int = 256, n_hidden_layers: int = 3, step_scale: float = 1.0):
    """Adam on the mean squared error of standardised labels; returns the
    WarmStart and a history dict (losses, validation RMSE per parameter).
    The initial simplex step of each parameter is step_scale times its
    validation RMSE, within [0.02, 0.5]."""
    rng = np.random.default_rng(seed)
    n = data.features.shape[0]
    perm = rng.permutation(n)
    n_val = max(1, int(round(val_frac * n)))
    val, tr = perm[:n_val], perm[n_val:]
    X = data.features.astype(np.float32)
    Y = data.labels.astype(np.float32)
    x_mean, x_std = X[tr].mean(0), X[tr].std(0)
    x_std = np.where(x_std > 1e-6, x_std, 1.0).astype(np.float32)
    y_mean, y_std = Y[tr].mean(0), Y[tr].std(0)
    y_std = np.where(y_std > 1e-6, y_std, 1.0).astype(np.float32)
    Xs = (X - x_mean) / x_std
    Ys = (Y - y_mean) / y_std
    net = plk.MLP(N_FEATURES, N_PARAMS, n_hidden, n_hidden_layers, seed=seed)
    losses = []
    steps_per_epoch = max(1, len(tr) // batch)
    total = epochs * steps_per_epoch
    step = 0
    t0 = time.perf_counter()
    for ep in range(epochs):
        order = rng.permutation(tr)
        ep_loss = 0.0
        for s in range(steps_per_epoch):
            idx = order[s * batch:(s + 1) * batch]
            # cosine decay to a tenth of the initial rate
            rate = lr * (0.1 + 0.9 * 0.5 * (1.0 + np.cos(np.pi * step / total)))
            ep_loss += net.train_step(Xs[idx], Ys[idx], rate)
            step += 1
        losses.append(ep_loss / steps_per_epoch)
    train_s = time.perf_counter() - t0
    ws = WarmStart(net, x_mean, x_std, y_mean, y_std, DEFAULT_STEP)
    resid = ws.predict(X[val]) - data.labels[val]
    rmse = np.sqrt(np.mean(resid ** 2, axis=0))
    ws.step = np.clip(step_scale * rmse, 0.02, DEFAULT_STEP)
    base = np.sqrt(np.mean((data.labels[val] - y_mean) ** 2, axis=0))
    hist = {"train_loss": losses, "val_rmse": rmse.tolist(), "val_rmse_mean_predictor": base.tolist(),
            "train_s": train_s, "steps": step, "start_step": ws.step.tolist()}
    return ws, hist


def fit_warm(b: plk.Batch, freqs, features, ws: WarmStart, ftol: float = 1e-4, xtol: float = 1e-3,
             max_evals: int = 4000, target=None, target_tol: float = 1e-3):
    """The fit from the network's start where that start scores at least as
    well as the default one, else from the default start.  Returns the
    BatchFit (evaluations include the two start evaluations) and which items
    used the network's start."""
    n = len(b)
    x_net = ws.predict(features)
    x_def = np.zeros((n, N_PARAMS))
    l_net = b.eval_gtr(freqs, x_net)
    l_def = b.eval_gtr(freqs, x_def)
    use = l_net >= l_def
    x0 = np.where(use[:, None], x_net, x_def)
    step = np.where(use[:, None], ws.step[None, :], DEFAULT_STEP)
    fit = b.fit_gtr(freqs, x0, step, ftol, xtol, max_evals, target=target, target_tol=target_tol)
    fit.evals = fit.evals + 2
    fit.rounds += 2
    if fit.hit_evals is not None:
        fit.hit_evals = np.where(fit.hit_evals >= 0, fit.hit_evals + 2, -1)
    return fit, use


def evaluate(ws: WarmStart, n_items: int = 1000, n_taxa: int = 64, n_sites: int = 5000, seed: int = 7,
             ftol: float = 1e-4, xtol: float = 1e-3, max_evals: int = 4000, tol: float = 1e-3,
             method: int = plk.PLK_FIT_NEWTON_START) -> dict:
    """Held-out comparison of the plain default-start fit and the warm fit on
    the same simulated alignments, both with the optimiser ``method``.  Two
    evaluation counts per item: until the stopping rule ends the fit, and
    until the fit first comes within ``tol`` of the plain fit's final lnL (the
    plain fit's own count for the latter is taken on a second identical run
    with that target)."""
    b, truth = simulate_batch(n_items, n_taxa, n_sites, seed)
    try:
        b.set_fit_method(method)
        feats = b.features()
        freqs = empirical_freqs(feats)
        b.eval_gtr(freqs, np.zeros((n_items, N_PARAMS)))  # tuning and graph capture outside the timings
        t0 = time.perf_counter()
        plain = b.fit_gtr(freqs, None, DEFAULT_STEP, ftol, xtol, max_evals)
        plain_s = time.perf_counter() - t0
        t0 = time.perf_counter()
        warm, used = fit_warm(b, freqs, feats, ws, ftol, xtol, max_evals, target=plain.lnl, target_tol=tol)
        warm_s = time.perf_counter() - t0
        # the plain fit is deterministic: rerun it with its own optimum as target
        plain_hit = b.fit_gtr(freqs, None, DEFAULT_STEP, ftol, xtol, max_evals, target=plain.lnl,
                              target_tol=tol).hit_evals
    finally:
        b.close()
    # The judge: a warm fit that ends more than tol below the plain fit's
    # optimum continues from the default start (the fallback), on a batch of
    # just those alignments; its evaluations add to the warm fit's.
    warm_only = warm.lnl.copy()
    short = np.flatnonzero(plain.lnl - warm.lnl > tol)
    final = warm.lnl.copy()
    evals = warm.evals.astype(np.int64).copy()
    hit = np.where(warm.hit_evals >= 0, warm.hit_evals, -1).astype(np.int64)
    fallback_s = 0.0
    fallback_diff = 0.0
    if short.size:
        fb, _ = simulate_batch(n_items, n_taxa, n_sites, seed, only=short)
        try:
            fb.set_fit_method(method)
            fb.eval_gtr(freqs[short], np.zeros((short.size, N_PARAMS)))
            t0 = time.perf_counter()
            f = fb.fit_gtr(freqs[short], None, DEFAULT_STEP, ftol, xtol, max_evals, target=plain.lnl[short],
                           target_tol=tol)
            fallback_s = time.perf_counter() - t0
        finally:
            fb.close()
        fallback_diff = float(np.abs(f.lnl - plain.lnl[short]).max())
        final[short] = np.maximum(warm.lnl[short], f.lnl)
        hit[short] = np.where(f.hit_evals >= 0, evals[short] + f.hit_evals, -1)
        evals[short] += f.evals
    warm_s += fallback_s
    deficit = plain.lnl - final   # > 0 where the judged warm fit ends below the plain optimum
    reached = hit >= 0
    pred = ws.predict(feats)
    hit_or_all = np.where(reached, hit, evals)
    return {
        "n_items": n_items, "n_taxa": n_taxa, "n_sites": n_sites, "seed": seed, "tol": tol,
        "method": {plk.PLK_FIT_NELDER_MEAD: "nelder-mead", plk.PLK_FIT_QUASI_NEWTON: "quasi-newton",
                   plk.PLK_FIT_NEWTON_START: "quasi-newton, newton start"}[method],
        "plain_evals_mean": float(plain.evals.mean()), "warm_evals_mean": float(evals.mean()),
        "evals_ratio_warm_over_plain": float(evals.mean() / plain.evals.mean()),
        "plain_evals_to_optimum_mean": float(plain_hit.mean()),
        "warm_evals_to_plain_optimum_mean": float(hit_or_all.mean()),
        "evals_to_optimum_ratio_warm_over_plain": float(hit_or_all.mean() / plain_hit.mean()),
        "frac_warm_reached_plain_optimum": float(reached.mean()),
        "plain_rounds": int(plain.rounds), "warm_rounds": int(warm.rounds),
        "plain_wall_s": plain_s, "warm_wall_s": warm_s, "wall_ratio_warm_over_plain": warm_s / plain_s,
        "frac_final_within_tol_of_plain": float(np.mean(deficit <= tol)),
        "max_lnl_deficit": float(deficit.max()), "mean_lnl_gain": float((-deficit).mean()),
        "judge": {"fallback_items": int(short.size), "fallback_wall_s": fallback_s,
                  "fallback_max_abs_lnl_diff_vs_plain": fallback_diff,
                  "before_fallback_frac_within_tol": float(np.mean(plain.lnl - warm_only <= tol)),
                  "before_fallback_max_deficit": float((plain.lnl - warm_only).max())},
        "frac_network_start_used": float(used.mean()),
        "prediction_rmse_vs_plain_fit": np.sqrt(np.mean((pred - plain.x) ** 2, axis=0)).tolist(),
        "prediction_rmse_vs_truth": np.sqrt(np.mean((pred - truth) ** 2, axis=0)).tolist(),
    }


def main(argv=None):
    ap = argparse.ArgumentParser(description="train and evaluate the learned warm start")
    ap.add_argument("--cache", default="warmstart_cache", help="directory of the labelled set and the weights")
    ap.add_argument("--train-items", type=int, default=20000)
    ap.add_argument("--train-taxa", type=int, default=32)
    ap.add_argument("--train-sites", type=int, default=2000)
    ap.add_argument("--eval-items", type=int, default=1000)
    ap.add_argument("--eval-taxa", type=int, default=64)
    ap.add_argument("--eval-sites", type=int, default=5000)
    ap.add_argument("--epochs", type=int, default=200)
    ap.add_argument("--seed", type=int, default=1)
    args = ap.parse_args(argv)
    os.makedirs(args.cache, exist_ok=True)
    data_path = os.path.join(args.cache, "labelled.npz")
    net_path = os.path.join(args.cache, "warmstart.npz")
    if os.path.exists(data_path):
        data = LabelledSet.load(data_path)
    else:
        data = make_labelled(args.train_items, args.train_taxa, args.train_sites, args.seed)
        data.save(data_path)
    if os.path.exists(net_path):
        ws, hist = WarmStart.load(net_path), {}
    else:
        ws, hist = train(data, epochs=args.epochs, seed=args.seed)
        ws.save(net_path)
    res = evaluate(ws, args.eval_items, args.eval_taxa, args.eval_sites, seed=args.seed + 1000)
    res["label_fit_s"] = data.fit_s
    res["label_evals_mean"] = float(data.evals.mean())
    res["training"] = {k: v for k, v in hist.items() if k != "train_loss"}
    # the same comparison with the Nelder-Mead optimiser (the reference's NLopt method)
    nm = evaluate(ws, args.eval_items, args.eval_taxa, args.eval_sites, seed=args.seed + 1000,
                  method=plk.PLK_FIT_NELDER_MEAD)
    res["nelder_mead"] = {k: nm[k] for k in ("plain_evals_to_optimum_mean", "warm_evals_to_plain_optimum_mean",
                                             "evals_to_optimum_ratio_warm_over_plain", "plain_evals_mean",
                                             "warm_evals_mean", "frac_final_within_tol_of_plain", "plain_wall_s",
                                             "warm_wall_s")}
    print(json.dumps(res))


if __name__ == "__main__":
    main()
