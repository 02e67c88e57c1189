"""Test infrastructure: Python access to the CPU oracle and to the reference harness.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module, to check results or to time a CPU baseline.
The product (``phylommand_gb300`` / ``libplk``) never imports it.

* ``load()`` binds ``_build/liborc.so`` (built from ``orc.c`` by ``make orc``),
  the FP64 C restatement of the reference likelihood path.
* ``parse_newick`` restates ``tree::tree_file_parser`` (src/tree.cpp:69-237),
  including the zero-length node it inserts to resolve a multifurcation.
* ``parse_fasta`` restates ``matrix_parser::pars_fasta``
  (src/matrix_parser.cpp:93-139) with the built-in DNA alphabet
  (src/matrix_parser.cpp:282-323: A=0, G=1, C=2, T=3) or an alphabet map.
* ``run_harness`` runs ``_ref/ref_harness`` (the reference's own code, built by
  ``make ref`` where the reference sources exist) and parses its output.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liborc.so")
HARNESS = os.path.join(HERE, "_ref", "ref_harness")

P_TAYLOR20, P_EXACT, P_GIVEN = 0, 1, 2

_lib = None


def build() -> None:
    subprocess.run(["make", "-s", "-C", HERE, "orc"], check=True)


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        build()
    lib = ctypes.CDLL(LIB_PATH)
    dp = ctypes.POINTER(ctypes.c_double)
    ip = ctypes.POINTER(ctypes.c_int)
    up = ctypes.POINTER(ctypes.c_uint)
    fp = ctypes.POINTER(ctypes.c_float)
    u32p = ctypes.POINTER(ctypes.c_uint32)
    lib.orc_rate_pos.restype = ctypes.c_uint
    lib.orc_rate_pos.argtypes = [ctypes.c_uint, ctypes.c_int, ctypes.c_uint, ctypes.c_uint]
    lib.orc_q_matrix.restype = None
    lib.orc_q_matrix.argtypes = [ctypes.c_uint, ctypes.c_int, up, dp, dp, dp]
    lib.orc_pmat_taylor20.restype = None
    lib.orc_pmat_taylor20.argtypes = [ctypes.c_uint, dp, ctypes.c_double, dp]
    lib.orc_pmat_exact.restype = None
    lib.orc_pmat_exact.argtypes = [ctypes.c_uint, dp, ctypes.c_double, dp]
    lib.orc_effective_lengths.restype = None
    lib.orc_effective_lengths.argtypes = [ctypes.c_int, ip, ip, dp, ctypes.c_double, ctypes.c_int,
                                          fp, fp, ip, ctypes.c_int, fp, dp]
    lib.orc_discrete_gamma.restype = None
    lib.orc_discrete_gamma.argtypes = [ctypes.c_double, ctypes.c_int, dp]
    lib.orc_loglik.restype = ctypes.c_double
    lib.orc_loglik.argtypes = [ctypes.c_int, ctypes.c_int, ip, ip, ctypes.c_int, ctypes.c_int,
                               u32p, dp, dp, dp, ctypes.c_int, dp, dp, ctypes.c_int, dp,
                               ctypes.c_int, ctypes.c_int, dp, dp, dp, dp]
    lib.orc_internal_postorder.restype = ctypes.c_int
    lib.orc_internal_postorder.argtypes = [ctypes.c_int, ip, ip, ip]
    _lib = lib
    return lib


def _p(a, ct):
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.POINTER(ct))


# ---------------------------------------------------------------- model parts
def rate_pos(n: int, tr: bool, row: int, col: int) -> int:
    return int(load().orc_rate_pos(n, int(tr), row, col))


def q_matrix(n: int, tr: bool, spec, rates, freqs=None) -> np.ndarray:
    spec = np.ascontiguousarray(spec, dtype=np.uint32)
    rates = np.ascontiguousarray(rates, dtype=np.float64)
    fr = None if freqs is None else np.ascontiguousarray(freqs, dtype=np.float64)
    Q = np.zeros((n, n))
    load().orc_q_matrix(n, int(tr), _p(spec, ctypes.c_uint), _p(rates, ctypes.c_double),
                        _p(fr, ctypes.c_double), _p(Q, ctypes.c_double))
    return Q


def pmat_taylor20(Q: np.ndarray, t: float) -> np.ndarray:
    Q = np.ascontiguousarray(Q, dtype=np.float64)
    P = np.zeros_like(Q)
    load().orc_pmat_taylor20(Q.shape[0], _p(Q, ctypes.c_double), float(t), _p(P, ctypes.c_double))
    return P


def pmat_exact(Q: np.ndarray, t: float) -> np.ndarray:
    Q = np.ascontiguousarray(Q, dtype=np.float64)
    P = np.zeros_like(Q)
    load().orc_pmat_exact(Q.shape[0], _p(Q, ctypes.c_double), float(t), _p(P, ctypes.c_double))
    return P


def discrete_gamma(alpha: float, K: int) -> np.ndarray:
    r = np.zeros(K)
    load().orc_discrete_gamma(float(alpha), int(K), _p(r, ctypes.c_double))
    return r


def effective_lengths(left, right, bl, root_dist0=0.0, cut_off=(), cut_rate=(),
                      clade_of_node=None, clade_rate=()) -> np.ndarray:
    left = np.ascontiguousarray(left, dtype=np.int32)
    right = np.ascontiguousarray(right, dtype=np.int32)
    bl = np.ascontiguousarray(bl, dtype=np.float64)
    n = left.shape[0]
    co = np.ascontiguousarray(cut_off, dtype=np.float32)
    cr = np.ascontiguousarray(cut_rate, dtype=np.float32)
    crate = np.ascontiguousarray(clade_rate, dtype=np.float32)
    con = None if clade_of_node is None else np.ascontiguousarray(clade_of_node, dtype=np.int32)
    out = np.zeros(n)
    load().orc_effective_lengths(n, _p(left, ctypes.c_int), _p(right, ctypes.c_int),
                                 _p(bl, ctypes.c_double), float(root_dist0), len(co),
                                 _p(co, ctypes.c_float) if len(co) else None,
                                 _p(cr, ctypes.c_float) if len(cr) else None,
                                 _p(con, ctypes.c_int) if con is not None else None,
                                 len(crate), _p(crate, ctypes.c_float) if len(crate) else None,
                                 _p(out, ctypes.c_double))
    return out


def internal_postorder(left, right) -> np.ndarray:
    left = np.ascontiguousarray(left, dtype=np.int32)
    right = np.ascontiguousarray(right, dtype=np.int32)
    out = np.zeros(left.shape[0], dtype=np.int32)
    n = load().orc_internal_postorder(left.shape[0], _p(left, ctypes.c_int), _p(right, ctypes.c_int),
                                      _p(out, ctypes.c_int))
    return out[:n].copy()


@dataclass
class OracleResult:
    lnl: float
    site_lnl: np.ndarray
    cond: np.ndarray | None = None
    cond_norm: np.ndarray | None = None
    marginal: np.ndarray | None = None


def loglik(left, right, tips, t_eff, Q, root_w, cat_rate=(1.0,), cat_weight=(1.0,),
           p_mode=P_TAYLOR20, P=None, per_site_pmat=False, threads=1,
           want_cond=False, want_cond_norm=False, want_marginal=False) -> OracleResult:
    """FP64 likelihood of the flattened tree (see orc.h for the layout)."""
    left = np.ascontiguousarray(left, dtype=np.int32)
    right = np.ascontiguousarray(right, dtype=np.int32)
    tips = np.ascontiguousarray(tips, dtype=np.uint32)
    t_eff = np.ascontiguousarray(t_eff, dtype=np.float64)
    Q = np.ascontiguousarray(Q, dtype=np.float64)
    root_w = np.ascontiguousarray(root_w, dtype=np.float64)
    cr = np.ascontiguousarray(cat_rate, dtype=np.float64)
    cw = np.ascontiguousarray(cat_weight, dtype=np.float64)
    n_nodes = left.shape[0]
    n_tips, n_sites = tips.shape
    S = Q.shape[0]
    C = cr.shape[0]
    n_int = n_nodes - n_tips
    Pg = None if P is None else np.ascontiguousarray(P, dtype=np.float64)
    site = np.zeros(n_sites)
    cond = np.zeros((n_int, n_sites, C, S)) if want_cond else None
    cn = np.zeros((n_int, n_sites, S)) if want_cond_norm else None
    mg = np.zeros((n_int, n_sites, S)) if want_marginal else None
    lnl = load().orc_loglik(n_tips, n_nodes, _p(left, ctypes.c_int), _p(right, ctypes.c_int), n_sites, S,
                            _p(tips, ctypes.c_uint32), _p(t_eff, ctypes.c_double), _p(Q, ctypes.c_double),
                            _p(root_w, ctypes.c_double), C, _p(cr, ctypes.c_double), _p(cw, ctypes.c_double),
                            int(p_mode), _p(Pg, ctypes.c_double), int(per_site_pmat), int(threads),
                            _p(site, ctypes.c_double), _p(cond, ctypes.c_double), _p(cn, ctypes.c_double),
                            _p(mg, ctypes.c_double))
    return OracleResult(lnl, site, cond, cn, mg)


# ------------------------------------------------------------------ parsing
@dataclass
class _Node:
    bl: float = 0.0
    label: str | None = None
    left: "_Node | None" = None
    right: "_Node | None" = None
    parent: "_Node | None" = None


@dataclass
class FlatTree:
    """Nodes in post-order (left subtree, right subtree, node)."""
    left: np.ndarray
    right: np.ndarray
    bl: np.ndarray
    labels: list = field(default_factory=list)

    @property
    def n_nodes(self) -> int:
        return int(self.left.shape[0])

    def is_tip(self, v: int) -> bool:
        return self.left[v] < 0 and self.right[v] < 0


def parse_newick(text: str) -> FlatTree:
    """Restates tree::tree_file_parser (src/tree.cpp:69-237) for one tree."""
    chars = [c for c in text if not c.isspace()]
    root = _Node()
    present = root
    label = ""
    bl_text = ""
    mode = "s"
    i = 0

    def flush(node):
        nonlocal label, bl_text
        if label:
            node.label = label
            label = ""
        if bl_text:
            node.bl = _atof(bl_text)
            bl_text = ""

    while i < len(chars):
        c = chars[i]
        if c == "[":
            depth = 1
            i += 1
            while i < len(chars) and depth > 0:
                if chars[i] == "[":
                    depth += 1
                elif chars[i] == "]":
                    depth -= 1
                i += 1
            continue
        if c == "(":
            mode = "l"
            present.left = _Node(parent=present)
            present = present.left
            label = ""
        elif c == ",":
            mode = "l"
            flush(present)
            present = present.parent
            if present.right is None:
                present.right = _Node(parent=present)
                present = present.right
            else:
                extra = _Node(parent=present)
                extra.left, extra.right = present.left, present.right
                extra.left.parent = extra
                extra.right.parent = extra
                present.left = extra
                present.right = _Node(parent=present)
                present = present.right
        elif c == ")":
            mode = "l"
            flush(present)
            present = present.parent
        elif c == ":":
            mode = "b"
        elif c == ";":
            flush(present)
            if present.right is None and present.left is not None and present.label is not None:
                present.right = _Node(parent=present, label=present.label, bl=present.bl)
                present.label = None
                present.bl = 0.0
            break
        elif mode == "b":
            bl_text += c
        elif mode == "l":
            if not label and c in "'\"":
                i += 1
                while i < len(chars) and chars[i] != c:
                    label += chars[i]
                    i += 1
            else:
                label += c
        i += 1
    order: list[_Node] = []

    def post(n):
        if n is None:
            return
        post(n.left)
        post(n.right)
        order.append(n)

    post(root)
    idx = {id(n): k for k, n in enumerate(order)}
    left = np.array([idx[id(n.left)] if n.left else -1 for n in order], dtype=np.int32)
    right = np.array([idx[id(n.right)] if n.right else -1 for n in order], dtype=np.int32)
    bl = np.array([n.bl for n in order], dtype=np.float64)
    return FlatTree(left, right, bl, [n.label for n in order])


def _atof(s: str) -> float:
    """atof: the longest leading prefix that reads as a number, else 0."""
    best = 0.0
    for end in range(len(s), 0, -1):
        try:
            best = float(s[:end])
            break
        except ValueError:
            continue
    return best


DNA_ALPHABET = {}
for _c, _bits in [("A", [0]), ("G", [1]), ("C", [2]), ("T", [3]), ("-", []), (".", []),
                  ("R", [0, 1]), ("Y", [2, 3]), ("S", [1, 2]), ("W", [0, 3]), ("K", [1, 3]),
                  ("M", [0, 2]), ("B", [1, 2, 3]), ("D", [0, 1, 3]), ("H", [0, 2, 3]),
                  ("V", [0, 1, 2]), ("N", [0, 1, 2, 3])]:
    _m = 0
    for _b in _bits:
        _m |= 1 << _b
    DNA_ALPHABET[_c] = _m
    if _c.isalpha():
        DNA_ALPHABET[_c.lower()] = _m


def parse_fasta(text: str, alphabet=None):
    """Restates matrix_parser::pars_fasta: returns (names, masks[n_taxa][n_sites]).
    Characters missing from the alphabet read as an empty set; empty cells are
    then set to all states, as treeator does (src/treeator.cpp:463-466)."""
    alphabet = DNA_ALPHABET if alphabet is None else alphabet
    all_states = 0
    for m in alphabet.values():
        all_states |= m
    names, rows = [], []
    cur = None
    for line in text.splitlines():
        line = line.strip("\r")
        if line.startswith(">"):
            names.append(line[1:].replace(" ", "").replace("\t", ""))
            cur = []
            rows.append(cur)
        elif cur is not None:
            for c in line:
                if c in " \t":
                    continue
                cur.append(alphabet.get(c, 0))
    n_sites = max(len(r) for r in rows) if rows else 0
    masks = np.zeros((len(rows), n_sites), dtype=np.uint32)
    for i, r in enumerate(rows):
        masks[i, :len(r)] = r
    masks[masks == 0] = all_states
    return names, masks


def reorder_tips_first(tree: FlatTree, taxa: list) -> tuple:
    """Renumber nodes so tip i is the row of ``taxa`` with its label and the
    internal nodes follow in post-order; returns (left, right, bl, perm) with
    perm[new_id] = old post-order id."""
    pos = {name: i for i, name in enumerate(taxa)}
    n = tree.n_nodes
    new_of_old = np.full(n, -1, dtype=np.int64)
    n_tips = 0
    for v in range(n):
        if tree.is_tip(v):
            new_of_old[v] = pos[tree.labels[v]]
            n_tips += 1
    k = n_tips
    for v in range(n):
        if not tree.is_tip(v):
            new_of_old[v] = k
            k += 1
    perm = np.empty(n, dtype=np.int64)
    perm[new_of_old] = np.arange(n)
    left = np.full(n, -1, dtype=np.int32)
    right = np.full(n, -1, dtype=np.int32)
    bl = np.zeros(n)
    for v in range(n):
        nv = new_of_old[v]
        bl[nv] = tree.bl[v]
        if tree.left[v] >= 0:
            left[nv] = new_of_old[tree.left[v]]
        if tree.right[v] >= 0:
            right[nv] = new_of_old[tree.right[v]]
    return left, right, bl, perm


# ------------------------------------------------------------ reference run
@dataclass
class HarnessResult:
    lnl: float
    site_lnl: np.ndarray | None
    Q: np.ndarray
    tree: FlatTree | None
    nodes: dict          # (rank, cat) -> array [n_sites, S] of raw conditionals
    pmats: dict          # t -> P
    clades: dict         # postorder id -> clade number
    seconds: float | None
    names: list | None = None      # taxa in file order (with dump_tips)
    masks: np.ndarray | None = None  # uint32 [n_taxa, n_sites] (with dump_tips)


def harness_available() -> bool:
    return os.path.exists(HARNESS)


def run_harness(fasta: str, tree: str | None, specs, rates, freqs=None, alphabet=None,
                cat_rates=None, cat_weights=None, root_quirk=True, nodes=False, sites=False,
                pmats=None, nsites=None, time_reps=0, time_rates=None, clade_rates=None,
                tr=None, binary=None, dump_tips=False) -> HarnessResult:
    cmd = [binary or HARNESS, "--fasta", fasta, "--specs", ",".join(str(int(s)) for s in specs),
           "--rates", ",".join(repr(float(r)) for r in rates)]
    if tree:
        cmd += ["--tree", tree]
    if freqs is not None:
        cmd += ["--freqs", ",".join(repr(float(f)) for f in freqs)]
    if tr is not None:
        cmd += ["--tr", str(int(tr))]
    if alphabet:
        cmd += ["--alphabet", alphabet]
    if cat_rates is not None:
        cmd += ["--cat-rates", ",".join(repr(float(r)) for r in cat_rates),
                "--cat-weights", ",".join(repr(float(w)) for w in cat_weights)]
    if not root_quirk:
        cmd.append("--no-root-quirk")
    if nodes:
        cmd.append("--nodes")
    if sites:
        cmd.append("--sites")
    if pmats:
        cmd += ["--pmat", ",".join(repr(float(t)) for t in pmats)]
    if nsites is not None:
        cmd += ["--nsites", str(int(nsites))]
    if time_reps:
        cmd += ["--time", str(int(time_reps))]
    if time_rates:
        cmd += ["--time-rates", time_rates]
    if clade_rates:
        cmd += ["--clade-rates", clade_rates]
    if dump_tips:
        cmd.append("--dump-tips")
    out = subprocess.run(cmd, check=True, capture_output=True, text=True).stdout
    qrows, trows, srows, node_rows, prow, clades = {}, [], {}, {}, {}, {}
    lnl, secs = None, None
    dnames, drows = [], []
    for line in out.splitlines():
        f = line.split()
        if not f:
            continue
        tag = f[0]
        if tag == "Q":
            qrows[int(f[1])] = [float(x) for x in f[2:]]
        elif tag == "T":
            trows.append((int(f[1]), int(f[2]), int(f[3]), int(f[4]), float(f[5]), f[6]))
        elif tag == "S":
            srows[int(f[1])] = float(f[2])
        elif tag == "L":
            lnl = float(f[1])
        elif tag == "N":
            node_rows.setdefault((int(f[1]), int(f[2])), {})[int(f[3])] = [float(x) for x in f[4:]]
        elif tag == "P":
            prow.setdefault(float(f[1]), {})[int(f[2])] = [float(x) for x in f[3:]]
        elif tag == "C":
            clades[int(f[1])] = int(f[2])
        elif tag == "TIME":
            secs = float(f[1])
        elif tag == "D":
            dnames.append(f[2])
            drows.append([int(x, 16) for x in f[3].split(",")] if len(f) > 3 else [])
    Q = np.array([qrows[i] for i in sorted(qrows)])
    ft = None
    if trows:
        trows.sort()
        ft = FlatTree(np.array([r[2] for r in trows], dtype=np.int32),
                      np.array([r[3] for r in trows], dtype=np.int32),
                      np.array([r[4] for r in trows]),
                      [r[5] if r[1] else (None if r[5] == "-" else r[5]) for r in trows])
    nodes_out = {k: np.array([v[s] for s in sorted(v)]) for k, v in node_rows.items()}
    pm = {t: np.array([rows[i] for i in sorted(rows)]) for t, rows in prow.items()}
    site = np.array([srows[i] for i in sorted(srows)]) if srows else None
    dm = np.array(drows, dtype=np.uint32) if drows else None
    return HarnessResult(lnl, site, Q, ft, nodes_out, pm, clades, secs,
                         dnames if dnames else None, dm)
