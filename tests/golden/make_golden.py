"""Regenerates the golden fixtures in this folder from the reference itself.

Each fixture is the output of the reference's own simpleML / sub_model /
rate_model code, run through ``oracle/_ref/ref_harness`` (built from the
reference sources by ``make -C oracle ref``), on either the reference's example
files (a 100-site excerpt) or seeded synthetic inputs written out as FASTA and
Newick.  The tree arrays stored are the reference parser's own parse, so the
branch lengths are bit-identical to what the reference used.

    python tests/golden/make_golden.py          # needs the reference sources

Fixture keys (npz): left, right, bl (tips first, internal nodes in post-order),
masks [n_tips, n_sites] (uint32 state sets), n_states, tr, Q, root_w,
cat_rates, cat_weights, root_quirk, cut_off, cut_rate, clade_of_node,
clade_rate, lnl, site_lnl, node_sites (site indices of the node vectors),
node_cond [n_int, len(node_sites), C, S] raw conditionals, pmat_t, pmat.
"""
from __future__ import annotations

import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from phylommand_gb300 import synth  # noqa: E402

from oracle import refpath  # noqa: E402

EXAMPLES = refpath.REF_EXAMPLES
PROTEIN = "ACDEFGHIKLMNPQRSTVWY"


def newick(left, right, bl, labels, v=None) -> str:
    root = left.shape[0] - 1 if v is None else v

    def rec(u):
        if left[u] < 0 and right[u] < 0:
            return f"{labels[u]}:{float(bl[u])!r}"
        kids = [rec(c) for c in (left[u], right[u]) if c >= 0]
        return "(" + ",".join(kids) + f"):{float(bl[u])!r}"

    return rec(root)[: -len(f":{float(bl[root])!r}")] + ";"


def write_fasta(path, names, states_or_text):
    with open(path, "w") as f:
        for n, s in zip(names, states_or_text):
            f.write(f">{n}\n{s}\n")


def dna_text(masks):
    inv = {1: "A", 2: "G", 4: "C", 8: "T", 15: "N", 5: "M", 3: "R", 10: "K", 12: "Y", 6: "S", 9: "W",
           14: "B", 13: "H", 11: "D", 7: "V"}
    return ["".join(inv[int(m)] for m in row) for row in masks]


def protein_text(masks):
    out = []
    for row in masks:
        s = []
        for m in row:
            m = int(m)
            if m == (1 << 20) - 1:
                s.append("-")
            else:
                s.append(PROTEIN[m.bit_length() - 1])
        out.append("".join(s))
    return out


def capture(name, fasta, tree, *, specs, rates, freqs=None, tr=None, alphabet=None, cat_rates=None,
            cat_weights=None, root_quirk=True, nsites=None, node_sites=8, pmats=(0.05, 0.3),
            time_rates=None, clade_rates=None, cut_off=(), cut_rate=()):
    h = O.run_harness(fasta, tree, specs, rates, freqs=freqs, tr=tr, alphabet=alphabet,
                      cat_rates=cat_rates, cat_weights=cat_weights, root_quirk=root_quirk,
                      nodes=True, sites=True, pmats=list(pmats), nsites=nsites, dump_tips=True,
                      time_rates=time_rates, clade_rates=clade_rates)
    names = h.names
    masks = h.masks
    left, right, bl, perm = O.reorder_tips_first(h.tree, names)
    n_nodes = left.shape[0]
    clade_of_node = np.full(n_nodes, -1, dtype=np.int32)
    new_of_old = np.empty(n_nodes, dtype=np.int64)
    new_of_old[perm] = np.arange(n_nodes)
    for old, c in h.clades.items():
        clade_of_node[new_of_old[old]] = c
    S = h.Q.shape[0]
    C = 1 if cat_rates is None else len(cat_rates)
    n_int = n_nodes - masks.shape[0]
    k = min(node_sites, masks.shape[1])
    node_cond = np.zeros((n_int, k, C, S))
    for (rank, cat), arr in h.nodes.items():
        node_cond[rank, :, cat, :] = arr[:k]
    is_tr = bool(freqs is not None) if tr is None else bool(tr)
    if is_tr:
        fr = list(freqs) if freqs is not None else [1.0 / S] * S
        last = 1.0
        for f in fr[: S - 1]:
            last -= f
        root_w = np.array(fr[: S - 1] + [last])
    else:
        root_w = np.ones(S)
    clade_rate = []
    if clade_rates:
        for part in clade_rates.split(";"):
            clade_rate.append(float(part.split(":")[0]))
    out = dict(left=left, right=right, bl=bl, masks=masks, n_states=S, tr=int(is_tr), Q=h.Q, root_w=root_w,
               cat_rates=np.array(cat_rates if cat_rates is not None else [1.0]),
               cat_weights=np.array(cat_weights if cat_weights is not None else [1.0]),
               root_quirk=int(root_quirk), cut_off=np.array(cut_off, dtype=np.float32),
               cut_rate=np.array(cut_rate, dtype=np.float32), clade_of_node=clade_of_node,
               clade_rate=np.array(clade_rate, dtype=np.float32), lnl=h.lnl, site_lnl=h.site_lnl,
               node_sites=np.arange(k), node_cond=node_cond,
               pmat_t=np.array(sorted(h.pmats)), pmat=np.array([h.pmats[t] for t in sorted(h.pmats)]))
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(f"{name}: {masks.shape[0]} tips x {masks.shape[1]} sites, S={S}, C={C}, lnL={h.lnl!r}")


def synthetic(tmp, tag, n_tips, n_sites, S, seed, mean_bl=0.1, ambig=0.0):
    rng = np.random.default_rng(seed)
    left, right, bl = synth.yule_tree(n_tips, mean_bl, rng)
    if S == 4:
        freqs = rng.dirichlet(np.full(4, 10.0))
        Q = synth.reversible_q(4, rng.uniform(0.5, 5.0, 6), freqs)
    else:
        freqs = rng.dirichlet(np.full(S, 5.0))
        Q = synth.reversible_q(S, rng.lognormal(0.0, 1.0, S * (S - 1) // 2), freqs)
    states = synth.simulate(left, right, bl, Q, freqs, np.ones(1), n_sites, rng)
    masks = synth.to_masks(states)
    if ambig > 0:
        hole = rng.random(masks.shape) < ambig
        masks[hole] = np.uint32((1 << S) - 1)
        if S == 4:
            amb = rng.random(masks.shape) < ambig
            masks[amb] = rng.choice(np.array([3, 5, 6, 9, 10, 12, 7, 11, 13, 14], dtype=np.uint32), size=int(amb.sum()))
    labels = [f"t{i}" for i in range(n_tips)] + [None] * (left.shape[0] - n_tips)
    tree_path = os.path.join(tmp, tag + ".tree")
    fasta_path = os.path.join(tmp, tag + ".fst")
    with open(tree_path, "w") as f:
        f.write(newick(left, right, bl, labels) + "\n")
    write_fasta(fasta_path, labels[:n_tips], dna_text(masks) if S == 4 else protein_text(masks))
    return fasta_path, tree_path


def main():
    if not O.harness_available():
        O.build()
        import subprocess
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", f"REFSRC={refpath.REF_SRC}"],
                       check=True)
    fa = os.path.join(EXAMPLES, "alignment_file.fst")
    tr = os.path.join(EXAMPLES, "tree_file.tree")
    capture("ex_jc100", fa, tr, specs=[0] * 6, rates=[1.0], freqs=[0.25] * 4, nsites=100)
    capture("ex_gtr100", fa, tr, specs=range(6), rates=[1, 2, 3, 4, 5, 6], freqs=[0.1, 0.2, 0.3, 0.4], nsites=100)
    g = list(O.discrete_gamma(0.5, 4))
    capture("ex_gtr_gamma_noquirk", fa, tr, specs=range(6), rates=[1, 2, 3, 4, 5, 6],
            freqs=[0.1, 0.2, 0.3, 0.4], nsites=100, cat_rates=g, cat_weights=[0.25] * 4, root_quirk=False)
    with tempfile.TemporaryDirectory() as tmp:
        # the JC69 shape of the 16-taxon, 1,000-site compat workload
        w = synth.make("cfg1", seed=11)
        labels = [f"t{i}" for i in range(w.n_tips)] + [None] * (w.n_nodes - w.n_tips)
        tp = os.path.join(tmp, "cfg1.tree")
        fp = os.path.join(tmp, "cfg1.fst")
        with open(tp, "w") as f:
            f.write(newick(w.left, w.right, w.bl, labels) + "\n")
        write_fasta(fp, labels[: w.n_tips], dna_text(w.masks))
        capture("cfg1_jc16x1000", fp, tp, specs=[0] * 6, rates=[4.0 / 3.0], freqs=[0.25] * 4, node_sites=64)

        fp, tp = synthetic(tmp, "gtr", 24, 400, 4, seed=5, ambig=0.04)
        g = list(O.discrete_gamma(0.7, 4))
        capture("syn_gtr_gamma_ambig", fp, tp, specs=range(6), rates=[1.3, 2.9, 0.7, 1.1, 3.7, 1.0],
                freqs=[0.3, 0.2, 0.15, 0.35], cat_rates=g, cat_weights=[0.25] * 4, root_quirk=False, node_sites=16)

        fp, tp = synthetic(tmp, "nontr", 10, 200, 4, seed=6)
        rng = np.random.default_rng(66)
        capture("syn_nontr", fp, tp, specs=range(12), rates=list(rng.uniform(0.1, 1.0, 12)), tr=0, node_sites=16)

        fp, tp = synthetic(tmp, "prot", 12, 150, 20, seed=7, ambig=0.03)
        alpha_path = os.path.join(tmp, "protein.alphabet")
        with open(alpha_path, "w") as f:
            for i, c in enumerate(PROTEIN):
                f.write(f"{c} {i}\n")
            f.write("- " + " ".join(str(i) for i in range(20)) + "\n")
        rng = np.random.default_rng(77)
        pf = rng.dirichlet(np.full(20, 5.0))
        capture("syn_protein20", fp, tp, specs=range(190), rates=list(rng.lognormal(0, 1, 190)),
                freqs=list(pf), alphabet=alpha_path, node_sites=8)

        # multifurcations: resolved by zero-length nodes; the root quirk then
        # zeroes every edge hanging below a zero-length root child
        rng = np.random.default_rng(8)
        names = [f"m{i}" for i in range(7)]
        states = rng.integers(0, 4, size=(7, 60))
        write_fasta(os.path.join(tmp, "mf.fst"), names, dna_text(synth.to_masks(states)))
        with open(os.path.join(tmp, "mf.tree"), "w") as f:
            f.write("((m0:0.11,m1:0.07,m2:0.2):0.05,m3:0.3,(m4:0.1,(m5:0.02,m6:0.09):0.04):0.12);\n")
        capture("syn_multifurc", os.path.join(tmp, "mf.fst"), os.path.join(tmp, "mf.tree"),
                specs=[0, 1, 0, 0, 1, 0], rates=[1.0, 2.5], freqs=[0.25, 0.25, 0.25, 0.25], node_sites=60)

        # rate model: two time slices and one clade rate (treeator -U / -V)
        fp, tp = synthetic(tmp, "rm", 20, 200, 4, seed=9)
        capture("syn_ratemodel", fp, tp, specs=range(6), rates=[1.0, 2.0, 1.0, 1.0, 2.0, 1.0],
                freqs=[0.25] * 4, time_rates="0.5:0.05,2.0:0.15", clade_rates="3.0:t1,t2",
                cut_off=(0.05, 0.15), cut_rate=(0.5, 2.0), node_sites=16)

        # the root quirk: root-edge lengths do not change the reference's lnL
        write_fasta(os.path.join(tmp, "q.fst"), ["A", "B", "C", "D"], ["ACGTA", "ACGTT", "AGGCA", "TCGTA"])
        for tag, x, y in (("quirk_a", 0.3, 0.5), ("quirk_b", 0.9, 0.2)):
            with open(os.path.join(tmp, tag + ".tree"), "w") as f:
                f.write(f"((A:0.1,B:0.2):{x},(C:0.1,D:0.1):{y});\n")
            capture(tag, os.path.join(tmp, "q.fst"), os.path.join(tmp, tag + ".tree"), specs=[0] * 6,
                    rates=[1.0], freqs=[0.25] * 4, node_sites=5)


if __name__ == "__main__":
    main()
