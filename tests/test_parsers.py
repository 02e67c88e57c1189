"""The native FASTA / PHYLIP / NEXUS and Newick parsers (host only) against
the oracle's restatement of the reference's parsers and against the data they
were written from."""
import numpy as np
import pytest

from oracle import oracle as O
from phylommand_gb300 import plk, synth

DNA = "AGCT"
IUPAC = "RYSWKMBDHVN-."


def _random_rows(rng, n_taxa, n_sites):
    rows = []
    for _ in range(n_taxa):
        r = rng.choice(list(DNA), size=n_sites)
        amb = rng.random(n_sites) < 0.05
        r[amb] = rng.choice(list(IUPAC), size=int(amb.sum()))
        low = rng.random(n_sites) < 0.1
        r[low] = np.char.lower(r[low])
        rows.append("".join(r))
    return rows


def _expected(rows):
    out = np.zeros((len(rows), max(len(r) for r in rows)), dtype=np.uint32)
    for i, r in enumerate(rows):
        for j, c in enumerate(r):
            out[i, j] = O.DNA_ALPHABET.get(c, 0)
    out[out == 0] = 15
    return out


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_fasta_matches_oracle_and_data(seed):
    rng = np.random.default_rng(seed)
    rows = _random_rows(rng, 7, 93)
    names = [f"taxon_{i}" for i in range(7)]
    # sequences wrapped at 60 columns, blanks and CRLF line ends
    text = "".join(f">{n}\r\n" + "\n".join(r[k:k + 60] for k in range(0, len(r), 60)) + "\n"
                   for n, r in zip(names, rows))
    got_names, masks = plk.parse_alignment(text)
    o_names, o_masks = O.parse_fasta(text)
    assert got_names == names == o_names
    np.testing.assert_array_equal(masks, o_masks)
    np.testing.assert_array_equal(masks, _expected(rows))


def test_phylip_and_nexus():
    rng = np.random.default_rng(9)
    rows = _random_rows(rng, 5, 40)
    names = ["a", "bb", "c_3", "d", "e"]
    phy = f"5 40\n" + "".join(f"{n} {r}\n" for n, r in zip(names, rows))
    n1, m1 = plk.parse_alignment(phy, plk.PLK_FORMAT_PHYLIP)
    nex = ("#NEXUS\nBEGIN DATA;\n  DIMENSIONS NTAX=5 NCHAR=40;\n  FORMAT DATATYPE=DNA GAP=-;\nMATRIX\n"
           + "".join(f"  {n}   {r}\n" for n, r in zip(names, rows)) + ";\nEND;\n")
    n2, m2 = plk.parse_alignment(nex, plk.PLK_FORMAT_NEXUS)
    assert n1 == n2 == names
    np.testing.assert_array_equal(m1, _expected(rows))
    np.testing.assert_array_equal(m2, m1)
    with pytest.raises(plk.PlkError):
        plk.parse_alignment("4 40\n" + "".join(f"{n} {r}\n" for n, r in zip(names, rows)), plk.PLK_FORMAT_PHYLIP)
    with pytest.raises(plk.PlkError):
        plk.parse_alignment("#NEXUS\nbegin data;\nend;\n", plk.PLK_FORMAT_NEXUS)


def test_custom_alphabet():
    alpha = {c: 1 << i for i, c in enumerate("ARNDCQEGHILKMFPSTWYV")}
    alpha["-"] = 0
    names, m = plk.parse_alignment(">p\nARN-V\n>q\nWYXAA\n", alphabet=alpha)
    assert names == ["p", "q"]
    full = (1 << 20) - 1
    np.testing.assert_array_equal(m, [[1, 2, 4, full, 1 << 19], [1 << 17, 1 << 18, full, 1, 1]])


def _newick(left, right, bl, names, v, rng):
    if left[v] < 0:
        lab = names[v]
        if rng.random() < 0.3:
            lab = f"'{lab}'"
        return f"{lab}:{float(bl[v])!r}"
    inner = f"({_newick(left, right, bl, names, left[v], rng)},{_newick(left, right, bl, names, right[v], rng)})"
    if rng.random() < 0.2:
        inner += "[&comment]"
    return f"{inner}:{float(bl[v])!r}"


@pytest.mark.parametrize("n_tips", [2, 5, 17, 64])
def test_newick_matches_oracle(n_tips):
    rng = np.random.default_rng(n_tips)
    left, right, bl = synth.yule_tree(n_tips, 0.1, rng)
    names = [f"t{i}" for i in range(n_tips)]
    root = len(left) - 1
    text = _newick(left, right, bl, names, root, rng) + ";\n"
    order = rng.permutation(n_tips)
    taxa = [names[i] for i in order]
    L, R, B = plk.parse_newick(text, taxa)
    ol, orr, ob, _ = O.reorder_tips_first(O.parse_newick(text), taxa)
    np.testing.assert_array_equal(L, ol)
    np.testing.assert_array_equal(R, orr)
    np.testing.assert_array_equal(B, ob)
    # the parsed tree is the generating tree up to renumbering: same total length
    assert B.sum() == pytest.approx(bl.sum())


def test_newick_multifurcation_and_errors():
    text = "(a:1,b:2,c:3,d:4)root;"
    L, R, B = plk.parse_newick(text, ["a", "b", "c", "d"])
    ol, orr, ob, _ = O.reorder_tips_first(O.parse_newick(text), ["a", "b", "c", "d"])
    np.testing.assert_array_equal(L, ol)
    np.testing.assert_array_equal(R, orr)
    np.testing.assert_array_equal(B, ob)
    assert len(L) == 7  # two zero-length nodes resolve the four-way split
    for bad in ("(a:1,b:2)", "(a:1,b:2));", "(a,b);"):
        with pytest.raises(plk.PlkError):
            plk.parse_newick(bad, ["a", "x"])
