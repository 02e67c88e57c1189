"""Shared test helpers: golden fixtures, engine and oracle set-up."""
from __future__ import annotations

import glob
import os

import numpy as np

from oracle import oracle as O
from phylommand_gb300 import plk

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def fixture_names():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def load_fixture(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    return {k: z[k] for k in z.files}


def fixture_teff(fx):
    """Effective lengths of a fixture through the oracle's rate model."""
    con = fx["clade_of_node"]
    return O.effective_lengths(fx["left"], fx["right"], fx["bl"],
                               root_dist0=0.0 if int(fx["root_quirk"]) else 1e-30,
                               cut_off=fx["cut_off"], cut_rate=fx["cut_rate"],
                               clade_of_node=con if (con >= 0).any() else None,
                               clade_rate=fx["clade_rate"])


def oracle_for_fixture(fx, p_mode=O.P_TAYLOR20, **kw):
    return O.loglik(fx["left"], fx["right"], fx["masks"], fixture_teff(fx), fx["Q"], fx["root_w"],
                    fx["cat_rates"], fx["cat_weights"], p_mode=p_mode, **kw)


def normalise_cond(node_cond, cat_w):
    """[n_int, sites, C, S] raw conditionals -> per-site normalised mix."""
    mix = np.einsum("nics,c->nis", node_cond, cat_w) if node_cond.ndim == 4 else node_cond
    return mix / mix.sum(axis=-1, keepdims=True)


def engine_for_fixture(fx, p_mode=plk.PLK_P_TAYLOR20, device=0):
    h = plk.Handle(device)
    h.set_alignment(fx["masks"], int(fx["n_states"]))
    h.set_tree(fx["left"], fx["right"], fx["bl"])
    con = fx["clade_of_node"]
    h.set_rate_model(bool(int(fx["root_quirk"])), fx["cut_off"], fx["cut_rate"],
                     con if (con >= 0).any() else None, fx["clade_rate"])
    h.set_model(fx["Q"], fx["root_w"], bool(int(fx["tr"])), fx["cat_rates"], fx["cat_weights"], p_mode)
    return h
