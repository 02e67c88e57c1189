"""ctypes binding of libplk (include/plk.h).

The engine itself is the C ABI; this module only marshals numpy arrays across
it.  Loading fails loudly when ``lib/libplk.so`` has not been built: there is
no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libplk.so")

PLK_OK = 0
PLK_ERR_ARG = -1
PLK_ERR_ALLOC = -2
PLK_ERR_CUDA = -3
PLK_ERR_STATE = -4
PLK_ERR_TIMEOUT = -5
PLK_ERR_NUMERIC = -6
PLK_ERR_TIP = -7
PLK_ERR_NODEV = -8
PLK_ERR_UNSUPPORTED = -9

PLK_FP64 = 0
PLK_FP32S = 1
PLK_P_TAYLOR20 = 0
PLK_P_EXACT = 1
PLK_NODES_COND = 0
PLK_NODES_MARGINAL = 1
PLK_FIT_NELDER_MEAD = 0
PLK_FIT_QUASI_NEWTON = 1
PLK_FIT_NEWTON_START = 2

# Every symbol include/plk.h declares (checked by the tests).
EXPORTS = [
    "plk_create", "plk_destroy", "plk_last_error", "plk_status_string", "plk_api_version",
    "plk_set_alignment", "plk_set_alignment8", "plk_set_tree", "plk_set_rate_model", "plk_set_model",
    "plk_loglik", "plk_site_loglik", "plk_node_states", "plk_n_internal",
    "plk_q_matrix", "plk_pmat_host", "plk_discrete_gamma", "plk_effective_lengths",
    "plk_loglik_async", "plk_loglik_result", "plk_set_stream", "plk_set_profiling", "plk_kernel_times",
    "plk_sum_sites_noalloc", "plk_prune_variant", "plk_test_withhold_stage", "plk_set_patterns", "plk_n_patterns",
    "plk_fit_gtr", "plk_fit_n_params",
    "plk_batch_create", "plk_batch_destroy", "plk_batch_last_error", "plk_batch_n_items", "plk_batch_add",
    "plk_batch_set_model", "plk_batch_loglik", "plk_batch_tuning", "plk_batch_form",
    "plk_batch_nni_count", "plk_batch_nni_moves", "plk_batch_nni_loglik", "plk_simulate", "plk_nni_moves_host",
    "plk_batch_features", "plk_batch_fit_gtr", "plk_batch_eval_gtr", "plk_batch_set_fit_method",
    "plk_set_fit_method", "plk_batch_edge_derivatives", "plk_batch_optimize_branches", "plk_batch_branch_lengths",
    "plk_parse_alignment", "plk_parse_newick",
    "plk_mlp_create", "plk_mlp_destroy", "plk_mlp_last_error", "plk_mlp_n_params", "plk_mlp_get_params",
    "plk_mlp_set_params", "plk_mlp_forward", "plk_mlp_gradients", "plk_mlp_train_step",
    "plk_measure_fp32_peak", "plk_loglik_err", "plk_node_states_err", "plk_batch_device_ms",
]

_lib = None


class PlkError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"plk status {status}: {message}")
        self.status = status
        self.message = message


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"libplk.so not built at {LIB_PATH}: run `python -m phylommand_gb300.build`")
    L = ctypes.CDLL(LIB_PATH)
    c_int, c_double, c_void_p = ctypes.c_int, ctypes.c_double, ctypes.c_void_p
    dp = ctypes.POINTER(ctypes.c_double)
    ip = ctypes.POINTER(ctypes.c_int)
    fp = ctypes.POINTER(ctypes.c_float)
    up = ctypes.POINTER(ctypes.c_uint)
    u32p = ctypes.POINTER(ctypes.c_uint32)
    hp = ctypes.c_void_p
    L.plk_create.argtypes = [ctypes.POINTER(ctypes.c_void_p), c_int]
    L.plk_destroy.argtypes = [hp]
    L.plk_destroy.restype = None
    L.plk_last_error.argtypes = [hp]
    L.plk_last_error.restype = ctypes.c_char_p
    L.plk_status_string.argtypes = [c_int]
    L.plk_status_string.restype = ctypes.c_char_p
    L.plk_api_version.argtypes = []
    L.plk_set_alignment.argtypes = [hp, c_int, c_int, c_int, u32p]
    L.plk_set_alignment8.argtypes = [hp, c_int, c_int, c_int, ctypes.POINTER(ctypes.c_uint8)]
    L.plk_set_tree.argtypes = [hp, c_int, ip, ip, dp]
    L.plk_set_rate_model.argtypes = [hp, c_int, c_int, fp, fp, ip, c_int, fp]
    L.plk_set_model.argtypes = [hp, c_int, dp, dp, c_int, c_int, dp, dp, c_int]
    L.plk_loglik.argtypes = [hp, c_int, dp]
    L.plk_site_loglik.argtypes = [hp, dp]
    L.plk_node_states.argtypes = [hp, c_int, c_int, dp]
    L.plk_n_internal.argtypes = [hp]
    L.plk_q_matrix.argtypes = [c_int, c_int, up, dp, dp, dp]
    L.plk_pmat_host.argtypes = [c_int, dp, dp, c_int, c_double, c_int, dp]
    L.plk_discrete_gamma.argtypes = [c_double, c_int, dp]
    L.plk_effective_lengths.argtypes = [c_int, ip, ip, dp, c_int, c_int, fp, fp, ip, c_int, fp, dp]
    L.plk_loglik_async.argtypes = [hp, c_int]
    L.plk_loglik_result.argtypes = [hp, dp]
    L.plk_set_stream.argtypes = [hp, c_void_p]
    L.plk_set_profiling.argtypes = [hp, c_int]
    L.plk_kernel_times.argtypes = [hp, dp, ip, c_int]
    L.plk_prune_variant.argtypes = [hp]
    L.plk_test_withhold_stage.argtypes = [hp]
    L.plk_set_patterns.argtypes = [hp, c_int]
    L.plk_n_patterns.argtypes = [hp]
    L.plk_sum_sites_noalloc.argtypes = [c_void_p, c_int, c_void_p, c_void_p]
    L.plk_measure_fp32_peak.argtypes = [c_int, c_int, c_int, dp, dp]
    L.plk_loglik_err.argtypes = [hp, dp, dp, dp, dp]
    L.plk_node_states_err.argtypes = [hp, c_int, dp, dp]
    L.plk_batch_device_ms.argtypes = [c_void_p, dp, dp]
    L.plk_fit_gtr.argtypes = [hp, c_int, dp, c_int, dp, c_double, c_double, c_double, c_int, dp, dp, ip]
    L.plk_fit_n_params.argtypes = [c_int, c_int]
    L.plk_batch_create.argtypes = [ctypes.POINTER(ctypes.c_void_p), c_int, c_int]
    L.plk_batch_destroy.argtypes = [hp]
    L.plk_batch_destroy.restype = None
    L.plk_batch_last_error.argtypes = [hp]
    L.plk_batch_last_error.restype = ctypes.c_char_p
    L.plk_batch_n_items.argtypes = [hp]
    L.plk_batch_add.argtypes = [hp, c_int, c_int, u32p, c_int, ip, ip, dp, ip]
    L.plk_batch_set_model.argtypes = [hp, c_int, dp, dp, dp, dp]
    L.plk_batch_loglik.argtypes = [hp, dp]
    L.plk_batch_tuning.argtypes = [hp, ip, ip, dp, ip]
    L.plk_batch_form.argtypes = [hp, ip, ip]
    L.plk_batch_nni_count.argtypes = [hp, c_int]
    L.plk_batch_nni_moves.argtypes = [hp, c_int, ip]
    L.plk_batch_nni_loglik.argtypes = [hp, dp]
    L.plk_simulate.argtypes = [c_int, ip, ip, dp, c_int, dp, dp, c_int, dp, c_int, ctypes.c_uint64, c_int, u32p]
    L.plk_nni_moves_host.argtypes = [c_int, ip, ip, ip, ip]
    L.plk_batch_features.argtypes = [hp, fp]
    L.plk_batch_fit_gtr.argtypes = [hp, dp, dp, dp, c_double, c_double, c_int, dp, dp, ip, ip, dp, c_double, ip]
    L.plk_batch_eval_gtr.argtypes = [hp, dp, dp, dp]
    L.plk_batch_set_fit_method.argtypes = [hp, c_int]
    L.plk_set_fit_method.argtypes = [hp, c_int]
    L.plk_batch_edge_derivatives.argtypes = [hp, dp]
    L.plk_batch_optimize_branches.argtypes = [hp, c_int, c_double, dp, ip]
    L.plk_batch_branch_lengths.argtypes = [hp, c_int, dp]
    L.plk_parse_alignment.argtypes = [ctypes.c_char_p, ctypes.c_size_t, c_int, ctypes.POINTER(ctypes.c_int32), ip,
                                      ip, u32p, ctypes.c_char_p, ctypes.c_size_t]
    L.plk_parse_newick.argtypes = [ctypes.c_char_p, ctypes.c_size_t, c_int, ctypes.c_char_p, ip, ip, ip, dp]
    L.plk_mlp_create.argtypes = [ctypes.POINTER(ctypes.c_void_p), c_int, c_int, c_int, c_int, c_int, ctypes.c_uint64]
    L.plk_mlp_destroy.argtypes = [hp]
    L.plk_mlp_destroy.restype = None
    L.plk_mlp_last_error.argtypes = [hp]
    L.plk_mlp_last_error.restype = ctypes.c_char_p
    L.plk_mlp_n_params.argtypes = [hp]
    L.plk_mlp_get_params.argtypes = [hp, fp]
    L.plk_mlp_set_params.argtypes = [hp, fp]
    L.plk_mlp_forward.argtypes = [hp, c_int, fp, fp]
    L.plk_mlp_gradients.argtypes = [hp, c_int, fp, fp, fp, fp]
    L.plk_mlp_train_step.argtypes = [hp, c_int, fp, fp, ctypes.c_float, fp]
    no_status = ("plk_destroy", "plk_last_error", "plk_status_string", "plk_batch_destroy", "plk_batch_last_error",
                 "plk_mlp_destroy", "plk_mlp_last_error")
    for name in EXPORTS:
        if name not in no_status:
            getattr(L, name).restype = c_int
    _lib = L
    return L


def _p(a, ct):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(ct))


def _check(status: int, handle=None) -> None:
    if status != PLK_OK:
        msg = lib().plk_last_error(handle)
        raise PlkError(status, msg.decode() if msg else "")


# ---------------------------------------------------------------- host helpers
def q_matrix(n_states: int, reversible: bool, rate_spec, rates, freqs=None) -> np.ndarray:
    spec = np.ascontiguousarray(rate_spec, dtype=np.uint32)
    r = np.ascontiguousarray(rates, dtype=np.float64)
    f = None if freqs is None else np.ascontiguousarray(freqs, dtype=np.float64)
    Q = np.zeros((n_states, n_states))
    _check(lib().plk_q_matrix(n_states, int(reversible), _p(spec, ctypes.c_uint), _p(r, ctypes.c_double),
                              _p(f, ctypes.c_double), _p(Q, ctypes.c_double)))
    return Q


def pmat_host(Q, t: float, p_mode: int = PLK_P_EXACT, root_weights=None, reversible: bool = True) -> np.ndarray:
    Q = np.ascontiguousarray(Q, dtype=np.float64)
    w = None if root_weights is None else np.ascontiguousarray(root_weights, dtype=np.float64)
    P = np.zeros_like(Q)
    _check(lib().plk_pmat_host(Q.shape[0], _p(Q, ctypes.c_double), _p(w, ctypes.c_double), int(reversible),
                               float(t), int(p_mode), _p(P, ctypes.c_double)))
    return P


def simulate(left, right, branch_length, Q, freqs, cat_rates, n_sites: int, seed: int, threads: int = 0) -> np.ndarray:
    """Seeded simulation down a tree; returns state-set masks [n_tips, n_sites]."""
    l = np.ascontiguousarray(left, dtype=np.int32)
    r = np.ascontiguousarray(right, dtype=np.int32)
    b = np.ascontiguousarray(branch_length, dtype=np.float64)
    Q = np.ascontiguousarray(Q, dtype=np.float64)
    f = np.ascontiguousarray(freqs, dtype=np.float64)
    cr = np.ascontiguousarray(cat_rates, dtype=np.float64)
    n_tips = int(np.sum((l < 0) & (r < 0)))
    out = np.zeros((n_tips, int(n_sites)), dtype=np.uint32)
    _check(lib().plk_simulate(l.shape[0], _p(l, ctypes.c_int), _p(r, ctypes.c_int), _p(b, ctypes.c_double), Q.shape[0],
                              _p(Q, ctypes.c_double), _p(f, ctypes.c_double), cr.shape[0], _p(cr, ctypes.c_double),
                              int(n_sites), ctypes.c_uint64(seed), int(threads or os.cpu_count() or 1),
                              _p(out, ctypes.c_uint32)))
    return out


PLK_FORMAT_FASTA = 0
PLK_FORMAT_PHYLIP = 1
PLK_FORMAT_NEXUS = 2


def parse_alignment(text, fmt: int = PLK_FORMAT_FASTA, alphabet=None):
    """(names, masks[n_taxa, n_sites]) from FASTA / PHYLIP / NEXUS text
    (alphabet: dict char -> state-set mask, default DNA with IUPAC codes)."""
    data = text.encode() if isinstance(text, str) else bytes(text)
    table = None
    if alphabet is not None:
        table = np.full(256, -1, dtype=np.int32)
        for c, m in alphabet.items():
            table[ord(c)] = int(m)
    tp = _p(table, ctypes.c_int32)
    nt, ns = ctypes.c_int(0), ctypes.c_int(0)
    _check(lib().plk_parse_alignment(data, len(data), int(fmt), tp, ctypes.byref(nt), ctypes.byref(ns), None, None, 0))
    masks = np.zeros((nt.value, ns.value), dtype=np.uint32)
    cap = len(data) + nt.value + 1
    names = ctypes.create_string_buffer(cap)
    _check(lib().plk_parse_alignment(data, len(data), int(fmt), tp, ctypes.byref(nt), ctypes.byref(ns),
                                     _p(masks, ctypes.c_uint32), names, cap))
    out, off = [], 0
    raw = names.raw
    for _ in range(nt.value):
        end = raw.index(b"\0", off)
        out.append(raw[off:end].decode())
        off = end + 1
    return out, masks


def parse_newick(text, names=None):
    """(left, right, bl) of the first tree; tip i = names[i] when given."""
    data = text.encode() if isinstance(text, str) else bytes(text)
    packed = None if names is None else b"".join(n.encode() + b"\0" for n in names)
    n_taxa = 0 if names is None else len(names)
    nn = ctypes.c_int(0)
    _check(lib().plk_parse_newick(data, len(data), n_taxa, packed, ctypes.byref(nn), None, None, None))
    left = np.zeros(nn.value, dtype=np.int32)
    right = np.zeros(nn.value, dtype=np.int32)
    bl = np.zeros(nn.value)
    _check(lib().plk_parse_newick(data, len(data), n_taxa, packed, ctypes.byref(nn), _p(left, ctypes.c_int),
                                  _p(right, ctypes.c_int), _p(bl, ctypes.c_double)))
    return left, right, bl


def nni_moves(left, right) -> np.ndarray:
    """[n_moves, 2]: (node v, which) of every NNI move of a tree (host only)."""
    l = np.ascontiguousarray(left, dtype=np.int32)
    r = np.ascontiguousarray(right, dtype=np.int32)
    n = ctypes.c_int(0)
    _check(lib().plk_nni_moves_host(l.shape[0], _p(l, ctypes.c_int), _p(r, ctypes.c_int), None, ctypes.byref(n)))
    out = np.zeros((n.value, 2), dtype=np.int32)
    if n.value:
        _check(lib().plk_nni_moves_host(l.shape[0], _p(l, ctypes.c_int), _p(r, ctypes.c_int), _p(out, ctypes.c_int),
                                        ctypes.byref(n)))
    return out


def discrete_gamma(alpha: float, K: int) -> np.ndarray:
    out = np.zeros(K)
    _check(lib().plk_discrete_gamma(float(alpha), int(K), _p(out, ctypes.c_double)))
    return out


def effective_lengths(left, right, branch_length, root_quirk: bool = True, cut_off=(), cut_rate=(),
                      clade_of_node=None, clade_rate=()) -> np.ndarray:
    l = np.ascontiguousarray(left, dtype=np.int32)
    r = np.ascontiguousarray(right, dtype=np.int32)
    b = np.ascontiguousarray(branch_length, dtype=np.float64)
    co = np.ascontiguousarray(cut_off, dtype=np.float32)
    cr = np.ascontiguousarray(cut_rate, dtype=np.float32)
    crt = np.ascontiguousarray(clade_rate, dtype=np.float32)
    con = None if clade_of_node is None else np.ascontiguousarray(clade_of_node, dtype=np.int32)
    out = np.zeros(l.shape[0])
    _check(lib().plk_effective_lengths(l.shape[0], _p(l, ctypes.c_int), _p(r, ctypes.c_int), _p(b, ctypes.c_double),
                                       int(root_quirk), len(co), _p(co, ctypes.c_float) if len(co) else None,
                                       _p(cr, ctypes.c_float) if len(cr) else None, _p(con, ctypes.c_int),
                                       len(crt), _p(crt, ctypes.c_float) if len(crt) else None,
                                       _p(out, ctypes.c_double)))
    return out


# ---------------------------------------------------------------------- handle
class Handle:
    """One alignment + tree + model resident on one GPU."""

    def __init__(self, device: int = 0):
        self._h = ctypes.c_void_p()
        _check(lib().plk_create(ctypes.byref(self._h), int(device)), None)
        self.n_states = 0
        self.n_sites = 0

    def close(self) -> None:
        if self._h:
            lib().plk_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def raw(self):
        return self._h

    def set_patterns(self, on: bool) -> None:
        """Evaluate distinct site patterns once, weighted by their counts
        (takes effect at the next set_alignment)."""
        _check(lib().plk_set_patterns(self._h, int(bool(on))), self._h)

    @property
    def n_patterns(self) -> int:
        return int(lib().plk_n_patterns(self._h))

    def set_alignment(self, masks: np.ndarray, n_states: int) -> None:
        """State-set masks [n_tips, n_sites]; uint8 masks (<= 8 states) take
        the byte path (plk_set_alignment8), anything else the 32-bit one."""
        if isinstance(masks, np.ndarray) and masks.dtype == np.uint8 and masks.flags.c_contiguous:
            _check(lib().plk_set_alignment8(self._h, masks.shape[0], masks.shape[1], int(n_states),
                                            _p(masks, ctypes.c_uint8)), self._h)
            m = masks
        else:
            m = np.ascontiguousarray(masks, dtype=np.uint32)
            _check(lib().plk_set_alignment(self._h, m.shape[0], m.shape[1], int(n_states), _p(m, ctypes.c_uint32)),
                   self._h)
        self.n_states = int(n_states)
        self.n_sites = int(m.shape[1])

    def set_tree(self, left, right, branch_length) -> None:
        l = np.ascontiguousarray(left, dtype=np.int32)
        r = np.ascontiguousarray(right, dtype=np.int32)
        b = np.ascontiguousarray(branch_length, dtype=np.float64)
        _check(lib().plk_set_tree(self._h, l.shape[0], _p(l, ctypes.c_int), _p(r, ctypes.c_int), _p(b, ctypes.c_double)), self._h)

    def set_rate_model(self, root_quirk: bool = True, cut_off=(), cut_rate=(), clade_of_node=None, clade_rate=()) -> None:
        co = np.ascontiguousarray(cut_off, dtype=np.float32)
        cr = np.ascontiguousarray(cut_rate, dtype=np.float32)
        crt = np.ascontiguousarray(clade_rate, dtype=np.float32)
        con = None if clade_of_node is None else np.ascontiguousarray(clade_of_node, dtype=np.int32)
        _check(lib().plk_set_rate_model(self._h, int(root_quirk), len(co), _p(co, ctypes.c_float) if len(co) else None,
                                        _p(cr, ctypes.c_float) if len(cr) else None,
                                        _p(con, ctypes.c_int), len(crt), _p(crt, ctypes.c_float) if len(crt) else None), self._h)

    def set_model(self, Q, root_weights, reversible: bool = True, cat_rates=(1.0,), cat_weights=(1.0,),
                  p_mode: int = PLK_P_TAYLOR20) -> None:
        Q = np.ascontiguousarray(Q, dtype=np.float64)
        w = np.ascontiguousarray(root_weights, dtype=np.float64)
        cr = np.ascontiguousarray(cat_rates, dtype=np.float64)
        cw = np.ascontiguousarray(cat_weights, dtype=np.float64)
        _check(lib().plk_set_model(self._h, Q.shape[0], _p(Q, ctypes.c_double), _p(w, ctypes.c_double), int(reversible),
                                   cr.shape[0], _p(cr, ctypes.c_double), _p(cw, ctypes.c_double), int(p_mode)), self._h)

    def loglik(self, precision: int = PLK_FP64) -> float:
        out = ctypes.c_double(0.0)
        _check(lib().plk_loglik(self._h, int(precision), ctypes.byref(out)), self._h)
        return out.value

    def loglik_status(self, precision: int = PLK_FP64) -> tuple[int, float]:
        out = ctypes.c_double(0.0)
        st = lib().plk_loglik(self._h, int(precision), ctypes.byref(out))
        return st, out.value

    def loglik_async(self, precision: int = PLK_FP32S) -> None:
        _check(lib().plk_loglik_async(self._h, int(precision)), self._h)

    def loglik_result(self) -> float:
        out = ctypes.c_double(0.0)
        _check(lib().plk_loglik_result(self._h, ctypes.byref(out)), self._h)
        return out.value

    def set_stream(self, cuda_stream: int | None) -> None:
        """Run on an existing CUDA stream (e.g. torch.cuda.Stream().cuda_stream)."""
        _check(lib().plk_set_stream(self._h, ctypes.c_void_p(cuda_stream or 0)), self._h)

    def set_profiling(self, on: bool) -> None:
        _check(lib().plk_set_profiling(self._h, int(on)), self._h)

    def kernel_times(self, reset: bool = True) -> tuple[np.ndarray, int]:
        """Summed ms of (P(t), post-order, reduction) and the evaluation count."""
        ms = np.zeros(3)
        n = ctypes.c_int(0)
        _check(lib().plk_kernel_times(self._h, _p(ms, ctypes.c_double), ctypes.byref(n), int(reset)), self._h)
        return ms, n.value

    PRUNE_KERNELS = {
        4: {0: "prune4_kernel", 1: "prune4s_kernel (1 site/thread)", 2: "prune4s_kernel (2 sites/thread)",
            3: "prune4p_kernel (category pairs on FP32x2, 1 site/thread)",
            4: "prune4p_kernel (category pairs on FP32x2, 2 sites/thread)",
            5: "prune4p_kernel (category pairs on FP32x2, 1 site/thread, tip codes from global)",
            6: "prune4p_kernel (category pairs on FP32x2, 2 sites/thread, tip codes from global)",
            7: "prune4p_kernel (category pairs on FP32x2, 2 threads/site, tip codes from global)",
            8: "prune4p_kernel (category pairs on FP32x2, 2 threads/site)",
            9: "prune4p_bulk_kernel (category pairs on FP32x2, TMA bulk-copy stage ring, mbarrier pipeline)",
            10: "prune4p_kernel (category pairs on FP32x2, 1 site/thread, tip codes staged with each op)",
            11: "prune4p_kernel (category pairs on FP32x2, 2 sites/thread, tip codes staged with each op)",
            12: "prune4w_kernel (category pairs on FP32x2, warp-independent, 1 site/thread, spills in TMEM)",
            13: "prune4w_kernel (category pairs on FP32x2, warp-independent, 2 sites/thread, spills in TMEM)",
            14: "prune4w_kernel (category pairs on FP32x2, warp-independent, 4 sites/thread, spills in TMEM)",
            15: "prune4w_kernel (category pairs on FP32x2, warp-independent, 1 site/thread, tables in shared memory)",
            16: "prune4w_kernel (category pairs on FP32x2, warp-independent, 2 sites/thread, tables in shared memory)",
            17: "prune4w_kernel (category pairs on FP32x2, warp-independent, 4 sites/thread, tables in shared memory)",
            18: "prune4w_kernel (category pairs on FP32x2, warp-independent, 2 sites per 2 threads, tables in shared memory)"},
        20: {1: "prune20_kernel (CUDA cores, 4 warps/tile)", 2: "prune20_kernel (tensor cores, split TF32, 4 warps/tile)",
             3: "prune20_kernel (CUDA cores, 8 warps/tile)", 4: "prune20_kernel (tensor cores, split TF32, 8 warps/tile)",
             5: "prune20u_kernel (tcgen05 tensor cores, TMEM accumulators, split TF32)",
             6: "prune20v_kernel (tcgen05 tensor cores, compact: three CTAs per SM, split TF32)",
             7: "prune20v_kernel (tcgen05 tensor cores, compact, split BF16)"},
    }

    def test_withhold_stage(self) -> None:
        """Arm the failure-path test of the TMA-fed post-order form (see
        plk_test_withhold_stage)."""
        _check(lib().plk_test_withhold_stage(self._h), self._h)

    def prune_variant(self) -> int:
        """Number of the autotuned FP32 post-order form (-1: none tuned)."""
        return int(lib().plk_prune_variant(self._h))

    def prune_kernel(self) -> str:
        """Name of the autotuned FP32 post-order kernel, or 'other' where no
        tuned choice applies (FP64, other state counts, untuned)."""
        v = int(lib().plk_prune_variant(self._h))
        return self.PRUNE_KERNELS.get(getattr(self, "n_states", 0), {}).get(v, "other")

    def site_loglik(self) -> np.ndarray:
        out = np.zeros(self.n_sites)
        _check(lib().plk_site_loglik(self._h, _p(out, ctypes.c_double)), self._h)
        return out

    def set_fit_method(self, method: int) -> None:
        """PLK_FIT_NELDER_MEAD (default) or PLK_FIT_QUASI_NEWTON for fit_gtr."""
        _check(lib().plk_set_fit_method(self._h, int(method)), self._h)

    def fit_gtr(self, freqs, n_cats: int = 4, x0=None, precision: int = PLK_FP32S, step: float = 0.5,
                ftol: float = 1e-4, xtol: float = 1e-3, max_evals: int = 2000):
        """Nelder-Mead ML fit of GTR(+Gamma) exchangeabilities, Gamma shape and
        tree-length scale; returns (x, lnL, evaluations)."""
        f = np.ascontiguousarray(freqs, dtype=np.float64)
        n = int(lib().plk_fit_n_params(self.n_states, int(n_cats)))
        x = np.zeros(n)
        x0a = None if x0 is None else np.ascontiguousarray(x0, dtype=np.float64)
        lnl = ctypes.c_double(0.0)
        ne = ctypes.c_int(0)
        _check(lib().plk_fit_gtr(self._h, int(precision), _p(f, ctypes.c_double), int(n_cats), _p(x0a, ctypes.c_double),
                                 float(step), float(ftol), float(xtol), int(max_evals), _p(x, ctypes.c_double),
                                 ctypes.byref(lnl), ctypes.byref(ne)), self._h)
        return x, lnl.value, ne.value

    def n_internal(self) -> int:
        return int(lib().plk_n_internal(self._h))

    def node_states(self, mode: int = PLK_NODES_COND, precision: int = PLK_FP64) -> np.ndarray:
        out = np.zeros((self.n_internal(), self.n_sites, self.n_states))
        _check(lib().plk_node_states(self._h, int(mode), int(precision), _p(out, ctypes.c_double)), self._h)
        return out

    def loglik_err(self) -> tuple[float, float, float, float]:
        """(fast lnL, FP64 lnL, |delta|, |delta| / |FP64 lnL|)."""
        v = [ctypes.c_double() for _ in range(4)]
        _check(lib().plk_loglik_err(self._h, *[ctypes.byref(x) for x in v]), self._h)
        return tuple(x.value for x in v)

    def node_states_err(self, mode: int = PLK_NODES_COND) -> tuple[np.ndarray, float]:
        """Fast-form node states and their largest absolute difference from
        the FP64 plain form's."""
        out = np.zeros((self.n_internal(), self.n_sites, self.n_states))
        err = ctypes.c_double()
        _check(lib().plk_node_states_err(self._h, int(mode), _p(out, ctypes.c_double), ctypes.byref(err)), self._h)
        return out, err.value



def sum_sites_noalloc(d_site_lnl: int, n_sites: int, d_lnl_out: int, cuda_stream: int | None = None) -> None:
    """Compensated sum of per-site log-likelihoods in device memory into one
    device double, allocating nothing (device addresses as integers)."""
    _check(lib().plk_sum_sites_noalloc(ctypes.c_void_p(d_site_lnl), int(n_sites), ctypes.c_void_p(d_lnl_out),
                                       ctypes.c_void_p(cuda_stream or 0)))


@dataclass
class BatchFit:
    """Result of Batch.fit_gtr: per item the parameter vector, lnL and
    evaluation count; the batch evaluations (rounds) used; with a target, the
    evaluations each item needed to come within the tolerance of it."""
    x: np.ndarray
    lnl: np.ndarray
    evals: np.ndarray
    rounds: int
    hit_evals: np.ndarray | None = None


class Batch:
    """Many 4-state alignments, trees and models scored in one launch."""

    def __init__(self, n_cats: int = 4, device: int = 0):
        self._b = ctypes.c_void_p()
        _check(lib().plk_batch_create(ctypes.byref(self._b), int(device), int(n_cats)), None)
        self.n_cats = int(n_cats)
        self._n_nodes = []

    def _check(self, status: int) -> None:
        if status != PLK_OK:
            msg = lib().plk_batch_last_error(self._b)
            raise PlkError(status, msg.decode() if msg else "")

    def close(self) -> None:
        if self._b:
            lib().plk_batch_destroy(self._b)
            self._b = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __len__(self) -> int:
        return int(lib().plk_batch_n_items(self._b))

    def add(self, masks, left, right, branch_length) -> int:
        m = np.ascontiguousarray(masks, dtype=np.uint32)
        l = np.ascontiguousarray(left, dtype=np.int32)
        r = np.ascontiguousarray(right, dtype=np.int32)
        b = np.ascontiguousarray(branch_length, dtype=np.float64)
        item = ctypes.c_int(-1)
        self._check(lib().plk_batch_add(self._b, m.shape[0], m.shape[1], _p(m, ctypes.c_uint32), l.shape[0],
                                        _p(l, ctypes.c_int), _p(r, ctypes.c_int), _p(b, ctypes.c_double),
                                        ctypes.byref(item)))
        self._n_nodes.append(int(l.shape[0]))
        return item.value

    def set_model(self, item: int, Q, freqs, cat_rates, cat_weights) -> None:
        Q = np.ascontiguousarray(Q, dtype=np.float64)
        f = np.ascontiguousarray(freqs, dtype=np.float64)
        cr = np.ascontiguousarray(cat_rates, dtype=np.float64)
        cw = np.ascontiguousarray(cat_weights, dtype=np.float64)
        self._check(lib().plk_batch_set_model(self._b, int(item), _p(Q, ctypes.c_double), _p(f, ctypes.c_double),
                                              _p(cr, ctypes.c_double), _p(cw, ctypes.c_double)))

    def loglik(self) -> np.ndarray:
        out = np.zeros(len(self))
        self._check(lib().plk_batch_loglik(self._b, _p(out, ctypes.c_double)))
        return out

    def features(self) -> np.ndarray:
        """[n_items, 43] summary statistics (see plk_batch_features)."""
        out = np.zeros((len(self), 43), dtype=np.float32)
        self._check(lib().plk_batch_features(self._b, _p(out, ctypes.c_float)))
        return out

    def fit_gtr(self, freqs, x0=None, step=None, ftol: float = 1e-4, xtol: float = 1e-3, max_evals: int = 3000,
                target=None, target_tol: float = 1e-3) -> "BatchFit":
        """Lockstep Nelder-Mead ML fits of every item (see plk_batch_fit_gtr)."""
        n = len(self)
        np_ = int(lib().plk_fit_n_params(4, self.n_cats))
        f = np.ascontiguousarray(freqs, dtype=np.float64).reshape(n, 4)
        x0a = None if x0 is None else np.ascontiguousarray(x0, dtype=np.float64).reshape(n, np_)
        st = None
        if step is not None:
            # a scalar, one step per item, one per parameter, or [n_items, n_params]
            s = np.asarray(step, dtype=np.float64)
            if s.ndim == 1 and s.shape[0] == n and n != np_:
                s = s[:, None]
            st = np.ascontiguousarray(np.broadcast_to(s, (n, np_)), dtype=np.float64)
        tg = None if target is None else np.ascontiguousarray(target, dtype=np.float64).reshape(n)
        x = np.zeros((n, np_))
        lnl = np.zeros(n)
        ev = np.zeros(n, dtype=np.int32)
        hits = np.full(n, -1, dtype=np.int32)
        rounds = ctypes.c_int(0)
        self._check(lib().plk_batch_fit_gtr(self._b, _p(f, ctypes.c_double), _p(x0a, ctypes.c_double),
                                            _p(st, ctypes.c_double), float(ftol), float(xtol), int(max_evals),
                                            _p(x, ctypes.c_double), _p(lnl, ctypes.c_double), _p(ev, ctypes.c_int),
                                            ctypes.byref(rounds), _p(tg, ctypes.c_double), float(target_tol),
                                            _p(hits, ctypes.c_int)))
        return BatchFit(x, lnl, ev, rounds.value, hits if tg is not None else None)

    def set_fit_method(self, method: int) -> None:
        """PLK_FIT_NELDER_MEAD (default) or PLK_FIT_QUASI_NEWTON for fit_gtr."""
        self._check(lib().plk_batch_set_fit_method(self._b, int(method)))

    def edge_derivatives(self) -> list:
        """Per item an [n_nodes, 2] array: d lnL / dt and d2 lnL / dt2 for the
        edge above every node (caller's node ids; the root's row is 0)."""
        counts = self._n_nodes
        out = np.zeros(2 * max(sum(counts), 1))
        self._check(lib().plk_batch_edge_derivatives(self._b, _p(out, ctypes.c_double)))
        res, o = [], 0
        for n in counts:
            res.append(out[o:o + 2 * n].reshape(n, 2).copy())
            o += 2 * n
        return res

    def optimize_branches(self, max_iter: int = 50, tol: float = 1e-4):
        """ML branch lengths of every item; returns (lnL per item, iterations)."""
        lnl = np.zeros(len(self))
        iters = ctypes.c_int(0)
        self._check(lib().plk_batch_optimize_branches(self._b, int(max_iter), float(tol), _p(lnl, ctypes.c_double),
                                                      ctypes.byref(iters)))
        return lnl, iters.value

    def branch_lengths(self, item: int) -> np.ndarray:
        out = np.zeros(self._n_nodes[item])
        self._check(lib().plk_batch_branch_lengths(self._b, int(item), _p(out, ctypes.c_double)))
        return out

    def eval_gtr(self, freqs, x) -> np.ndarray:
        """lnL of every item at its GTR parameter vector x[n_items, n_params]."""
        n = len(self)
        np_ = int(lib().plk_fit_n_params(4, self.n_cats))
        f = np.ascontiguousarray(freqs, dtype=np.float64).reshape(n, 4)
        xa = np.ascontiguousarray(x, dtype=np.float64).reshape(n, np_)
        out = np.zeros(n)
        self._check(lib().plk_batch_eval_gtr(self._b, _p(f, ctypes.c_double), _p(xa, ctypes.c_double),
                                             _p(out, ctypes.c_double)))
        return out

    def nni_moves(self, item: int) -> np.ndarray:
        """[n_moves, 2]: (node v, which) of every NNI move of an item."""
        n = int(lib().plk_batch_nni_count(self._b, int(item)))
        out = np.zeros((n, 2), dtype=np.int32)
        if n:
            self._check(lib().plk_batch_nni_moves(self._b, int(item), _p(out, ctypes.c_int)))
        return out

    def device_ms(self) -> tuple[float, float]:
        """CUDA-event device time (ms) of the last loglik() and nni_loglik()."""
        a, b = ctypes.c_double(), ctypes.c_double()
        self._check(lib().plk_batch_device_ms(self._b, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def nni_loglik(self) -> list:
        """lnL of every NNI neighbour, one array per item."""
        counts = [int(lib().plk_batch_nni_count(self._b, i)) for i in range(len(self))]
        out = np.zeros(max(sum(counts), 1))
        self._check(lib().plk_batch_nni_loglik(self._b, _p(out, ctypes.c_double)))
        res, o = [], 0
        for c in counts:
            res.append(out[o:o + c].copy())
            o += c
        return res

    def tuning(self) -> dict:
        spt, grid, graph = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_int(0)
        ms = ctypes.c_double(0.0)
        self._check(lib().plk_batch_tuning(self._b, ctypes.byref(spt), ctypes.byref(grid), ctypes.byref(ms),
                                           ctypes.byref(graph)))
        paired, codes = ctypes.c_int(0), ctypes.c_int(0)
        self._check(lib().plk_batch_form(self._b, ctypes.byref(paired), ctypes.byref(codes)))
        return {"sites_per_thread": spt.value, "grid": grid.value, "postorder_ms": ms.value, "graph": bool(graph.value),
                "paired": bool(paired.value), "codes_smem": bool(codes.value)}


class MLP:
    """The warm-start network (see plk_mlp_create): n_in -> n_hidden x layers
    (ReLU) -> n_out, BF16 tensor-core GEMMs, FP32 master weights, Adam."""

    def __init__(self, n_in: int, n_out: int, n_hidden: int = 256, n_hidden_layers: int = 3, seed: int = 0,
                 device: int = 0):
        self._m = ctypes.c_void_p()
        _check(lib().plk_mlp_create(ctypes.byref(self._m), int(device), int(n_in), int(n_hidden),
                                    int(n_hidden_layers), int(n_out), int(seed)), None)
        self.n_in, self.n_out = int(n_in), int(n_out)
        self.n_hidden, self.n_hidden_layers = int(n_hidden), int(n_hidden_layers)

    def _check(self, status: int) -> None:
        if status != PLK_OK:
            msg = lib().plk_mlp_last_error(self._m)
            raise PlkError(status, msg.decode() if msg else "")

    def close(self) -> None:
        if self._m:
            lib().plk_mlp_destroy(self._m)
            self._m = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def n_params(self) -> int:
        return int(lib().plk_mlp_n_params(self._m))

    def layer_shapes(self) -> list:
        dims = [self.n_in] + [self.n_hidden] * self.n_hidden_layers + [self.n_out]
        return [(dims[i + 1], dims[i]) for i in range(len(dims) - 1)]

    def get_params(self) -> np.ndarray:
        out = np.zeros(self.n_params, dtype=np.float32)
        self._check(lib().plk_mlp_get_params(self._m, _p(out, ctypes.c_float)))
        return out

    def set_params(self, p) -> None:
        a = np.ascontiguousarray(p, dtype=np.float32)
        if a.size != self.n_params:
            raise ValueError(f"expected {self.n_params} parameters, got {a.size}")
        self._check(lib().plk_mlp_set_params(self._m, _p(a, ctypes.c_float)))

    def forward(self, x) -> np.ndarray:
        xa = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, self.n_in)
        y = np.zeros((xa.shape[0], self.n_out), dtype=np.float32)
        self._check(lib().plk_mlp_forward(self._m, xa.shape[0], _p(xa, ctypes.c_float), _p(y, ctypes.c_float)))
        return y

    def gradients(self, x, t):
        xa = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, self.n_in)
        ta = np.ascontiguousarray(t, dtype=np.float32).reshape(-1, self.n_out)
        g = np.zeros(self.n_params, dtype=np.float32)
        loss = ctypes.c_float(0.0)
        self._check(lib().plk_mlp_gradients(self._m, xa.shape[0], _p(xa, ctypes.c_float), _p(ta, ctypes.c_float),
                                            _p(g, ctypes.c_float), ctypes.byref(loss)))
        return g, float(loss.value)

    def train_step(self, x, t, lr: float) -> float:
        xa = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, self.n_in)
        ta = np.ascontiguousarray(t, dtype=np.float32).reshape(-1, self.n_out)
        loss = ctypes.c_float(0.0)
        self._check(lib().plk_mlp_train_step(self._m, xa.shape[0], _p(xa, ctypes.c_float), _p(ta, ctypes.c_float),
                                             float(lr), ctypes.byref(loss)))
        return float(loss.value)
