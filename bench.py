"""Benchmark: lnL evaluations per second of the DNA GTR+Gamma4 workload
(128 taxa, Yule tree with Exp(mean 0.05) branch lengths, 100,000 sites, 2% of
tip cells missing) on one GB300, FP32 partials with per-site scaling.

A step is one full likelihood evaluation through the C ABI: P(t) for every
edge and category (FP64 eigen form), the post-order pass over all sites and
the compensated reduction of the site log-likelihoods to one number.

    python bench.py [--steps K] [--warmup W] [--gpus N] [--impl ours|reference]

Prints one JSON line.  Multi-GPU runs (torchrun, one rank per GPU) are
independent replicas of the workload: the path does not shard within one
evaluation here, so there is no collective on the data path.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = "cfg2"
ORACLE_CELLS = 20_000_000  # tip cells up to which the DNA bench runs the FP64 oracle on the full workload
SEED = 2
FALLBACK_HBM_GBS = 6800.0
FALLBACK_BF16_TFLOPS = 1900.0
SM_COUNT = 152
FP32_LANES_PER_SM = 128


def algorithmic_bytes_per_site(n_tips: int, S: int, C: int, b: int) -> int:
    """Bytes one lnL evaluation must move per site in a level-by-level pass:
    internal-child partials read, 1-byte tip codes, each internal node's
    partials written plus a 4-byte scaler."""
    n_int = n_tips - 1
    internal_child_edges = n_int - 1
    return internal_child_edges * S * C * b + n_tips * 1 + n_int * (S * C * b + 4)


def algorithmic_flops_per_site(n_tips: int, S: int, C: int) -> int:
    """2 flops per multiply-add of every internal-child P(t) product, plus the
    per-node combine; tip children are table look-ups."""
    n_int = n_tips - 1
    return (n_int - 1) * 2 * C * S * S + n_int * C * S


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), float(d["bf16_tflops"]), "measured"
    return FALLBACK_HBM_GBS, FALLBACK_BF16_TFLOPS, "fallback"


def load_traffic(kernel: str):
    """DRAM bytes per launch of the named post-order kernel on this workload
    from its committed ncu summary (None when none has been summarised)."""
    p = os.path.join(ROOT, "profiles", f"{kernel.split()[0]}_dna_gtr_g4_128x100k.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("dram_bytes_per_launch")
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 7:
                continue
            try:
                rows.append((float(f[0]), float(f[1]), f[3:7]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, r in rows for i, v in enumerate(r) if v.lower().startswith("active")})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


def cpu_port_seconds(w, n_sites_sample: int, threads: int) -> float:
    """The oracle port of the reference path on a bounded sample of sites:
    P(t) rebuilt by Taylor-plus-20-squarings for every (site, edge,
    category), as simpleML::branch_likelihood does."""
    from oracle import oracle as O
    teff = O.effective_lengths(w.left, w.right, w.bl, root_dist0=1e-30)
    t0 = time.perf_counter()
    O.loglik(w.left, w.right, np.ascontiguousarray(w.masks[:, :n_sites_sample]), teff, w.Q, w.freqs,
             w.cat_rates, w.cat_weights, p_mode=O.P_TAYLOR20, per_site_pmat=True, threads=threads)
    return time.perf_counter() - t0


def dist_setup(n_gpus: int):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if os.environ.get("PLK_BENCH_GLOO") is None else "gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def reduce_max(world, x: float, device) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(args, world, rank):
    """The reference's CPU path on the host cores: the oracle port (the
    reference's sources do not travel to the GPU host) on all threads, each
    step a bounded sample of the same workload."""
    if rank != 0:
        return
    from phylommand_gb300 import synth  # the numpy backend: this process never loads libplk
    w = synth.make(WORKLOAD, seed=SEED, n_sites=args.sites, n_tips=args.taxa, backend="numpy")
    threads = os.cpu_count() or 1
    sample = max(threads * 40, 256)
    for _ in range(args.warmup):
        cpu_port_seconds(w, sample, threads)
    secs = [cpu_port_seconds(w, sample, threads) for _ in range(args.steps)]
    per_eval = (sum(secs) / len(secs)) * (w.n_sites / sample)
    value = 1.0 / per_eval
    line = {
        "impl": "reference", "metric": "lnL evals/s", "value": value, "unit": "evals/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(secs) / len(secs),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(w),
        "cpu_baseline": {"value": value, "unit": "evals/s", "cores": threads, "kind": "port",
                         "sample": f"{sample} of {w.n_sites} sites per step, {threads} threads, P(t) rebuilt per "
                                   f"(site, edge, category) by the reference's Taylor-plus-20-squarings; "
                                   f"time scaled linearly to all sites"},
        "e2e": {"value": value, "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "gsite_node_updates_per_s": value * (w.n_tips - 1) * w.n_sites / 1e9,
    }
    print(json.dumps(line), flush=True)


def workload_config(w):
    """The workload both arms run (the same dict in both lines)."""
    return {"workload": f"DNA GTR+Gamma4, {w.n_tips}-taxon Yule tree, {w.n_sites:,} sites, 2% missing cells",
            "n_taxa": w.n_tips, "n_sites": w.n_sites, "n_states": w.n_states, "n_categories": len(w.cat_rates),
            "alpha": w.alpha, "branch_lengths": "Exp(mean 0.05)", "seed": w.seed,
            "generator": "numpy (phylommand_gb300.synth, backend numpy)",
            "p_matrix": "FP64 eigen form", "partials": "FP32, per-site power-of-two scaling",
            "site_sum": "FP64 compensated", "parallelism": "replicas",
            "l2": "GPU arm: 256 MiB written before every timed step (L2 flushed), outside the events"}


def measure_fp32_peak(device: int):
    """The FP32 multiply-add peak of this GPU, measured by the library's
    microbenchmark (fma.rn.f32x2 chains over 4 CTAs per SM, CUDA events):
    TFLOP/s, or None when it fails."""
    import ctypes
    from phylommand_gb300 import plk
    t, ms = ctypes.c_double(), ctypes.c_double()
    best = None
    for packed in (1, 0):
        if plk.lib().plk_measure_fp32_peak(device, packed, 1 << 16, ctypes.byref(t), ctypes.byref(ms)) == 0:
            best = t.value if best is None else max(best, t.value)
    return best


def measure_fp64_peak(device: int):
    """The FP64 multiply-add rate of this GPU, measured by the library's
    microbenchmark (fma.rn.f64 chains over 4 CTAs per SM, CUDA events):
    TFLOP/s, or None when it fails."""
    import ctypes
    from phylommand_gb300 import plk
    t, ms = ctypes.c_double(), ctypes.c_double()
    if plk.lib().plk_measure_fp32_peak(device, 2, 1 << 10, ctypes.byref(t), ctypes.byref(ms)) == 0:
        return t.value
    return None


def required_bytes(w, C: int, grid_blocks: int) -> int:
    """Bytes one fused post-order pass must move through HBM: the 1-byte tip
    codes (rows padded to 16 bytes), the paired P(t) and tip tables it reads,
    the FP64 per-site values it writes and its block sums."""
    stride = (w.n_sites + 15) // 16 * 16
    codes = w.n_tips * stride
    tables = w.n_nodes * C * 16 * 4 + w.n_tips * C * 16 * 4 * 4
    return codes + tables + 8 * w.n_sites + 16 * grid_blocks


def time_steps(h, stream, flush, steps: int, precision: int):
    """CUDA-event time (ms, summed over steps) of `steps` evaluations on the
    engine's stream, L2 flushed before each outside the events."""
    import torch
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    for k in range(steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        starts[k].record(stream)
        h.loglik_async(precision)
        ends[k].record(stream)
    torch.cuda.synchronize()
    return sum(s.elapsed_time(e) for s, e in zip(starts, ends))


def run_ours(args, world, rank, local):
    import torch
    from phylommand_gb300 import plk, synth
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    w = synth.make(WORKLOAD, seed=SEED, n_sites=args.sites, n_tips=args.taxa, backend="numpy")
    C = len(w.cat_rates)
    fp32_peak = measure_fp32_peak(local)
    h = plk.Handle(local)
    h.set_alignment(w.masks, w.n_states)
    h.set_tree(w.left, w.right, w.bl)
    h.set_rate_model(False)
    h.set_model(w.Q, w.freqs, True, w.cat_rates, w.cat_weights, plk.PLK_P_EXACT)
    stream = torch.cuda.Stream(device=dev)
    h.set_stream(stream.cuda_stream)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)  # larger than the 129 MB L2

    lnl64 = h.loglik(plk.PLK_FP64)
    for _ in range(max(args.warmup, 3)):
        h.loglik_async(plk.PLK_FP32S)
    h.loglik_result()

    clocks = ClockSampler(local)
    clocks.start()
    barrier(world)
    torch.cuda.synchronize()
    t_wall = time.perf_counter()
    dev_ms = time_steps(h, stream, flush, args.steps, plk.PLK_FP32S)
    barrier(world)
    wall = time.perf_counter() - t_wall
    # the same steps again with the engine's per-kernel events (an event
    # between two kernels keeps the second from starting until the first has
    # drained, about 2 us each, so the steps above carry none): the kernel
    # durations of the roofline
    h.set_profiling(True)
    prof_ms = reduce_max(world, time_steps(h, stream, flush, args.steps, plk.PLK_FP32S), dev)
    kern_ms, n_evals = h.kernel_times(reset=True)
    h.set_profiling(False)
    clk = clocks.stop()
    lnl_timed = h.loglik_result()
    h_variant = h.prune_kernel()
    max_ms = reduce_max(world, dev_ms, dev)
    value = world * args.steps / (max_ms / 1e3)

    # the FP64 plain form (reference operation order for the P(t)-independent
    # part, FP64 partials) on the same workload: the like-for-like precision
    # of the reference's CPU path
    for _ in range(3):
        h.loglik_async(plk.PLK_FP64)
    h.loglik_result()
    steps64 = max(3, args.steps // 2)
    # (the engine's per-kernel events are on here: about 2 us each against a
    # 4 ms step)
    h.set_profiling(True)
    ms64 = reduce_max(world, time_steps(h, stream, flush, steps64, plk.PLK_FP64), dev)
    kern64, n64 = h.kernel_times(reset=True)
    h.set_profiling(False)
    lnl64_timed = h.loglik_result()
    value64 = world * steps64 / (ms64 / 1e3)
    fp64_peak = measure_fp64_peak(local)

    # end to end through the C ABI with host buffers: upload the alignment,
    # tree and model from pinned host memory, evaluate, read the lnL back
    # (byte masks, plk_set_alignment8; the 32-bit masks of plk_set_alignment
    # are timed the same way beside it)
    h.set_stream(None)
    pinned8 = torch.empty(w.masks.shape, dtype=torch.uint8, pin_memory=True)
    masks8 = pinned8.numpy()
    masks8[...] = w.masks.astype(np.uint8)
    pinned32 = torch.empty(w.masks.shape, dtype=torch.int32, pin_memory=True)
    masks32 = pinned32.numpy().view(np.uint32)
    masks32[...] = w.masks
    small = w.left.nbytes + w.right.nbytes + w.bl.nbytes + w.Q.nbytes + w.freqs.nbytes \
        + w.cat_rates.nbytes + w.cat_weights.nbytes
    e2e_steps = max(3, args.steps // 2)

    # The steps call the C ABI (include/plk.h) as a C or C++ caller such as
    # the simpleML drop-in does: the ctypes argument objects are built once,
    # every step passes the same host buffers and the library copies them
    # again (alignment, tree, rate model, model) before the evaluation.
    import ctypes
    L, hh = plk.lib(), h.raw
    c_i, c_d = ctypes.c_int, ctypes.c_double
    tl, tr = np.ascontiguousarray(w.left, np.int32), np.ascontiguousarray(w.right, np.int32)
    tb = np.ascontiguousarray(w.bl, np.float64)
    mq, mf = np.ascontiguousarray(w.Q, np.float64), np.ascontiguousarray(w.freqs, np.float64)
    mr, mw = np.ascontiguousarray(w.cat_rates, np.float64), np.ascontiguousarray(w.cat_weights, np.float64)
    tree_args = (hh, len(tl), tl.ctypes.data_as(ctypes.POINTER(c_i)), tr.ctypes.data_as(ctypes.POINTER(c_i)),
                 tb.ctypes.data_as(ctypes.POINTER(c_d)))
    rate_args = (hh, 0, 0, None, None, None, 0, None)
    model_args = (hh, mq.shape[0], mq.ctypes.data_as(ctypes.POINTER(c_d)), mf.ctypes.data_as(ctypes.POINTER(c_d)), 1,
                  len(mr), mr.ctypes.data_as(ctypes.POINTER(c_d)), mw.ctypes.data_as(ctypes.POINTER(c_d)),
                  plk.PLK_P_EXACT)
    out = ctypes.c_double(0.0)

    def e2e_run(masks, precision=plk.PLK_FP32S):
        if masks.dtype == np.uint8:
            aln = (L.plk_set_alignment8, (hh, masks.shape[0], masks.shape[1], w.n_states,
                                          masks.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))))
        else:
            aln = (L.plk_set_alignment, (hh, masks.shape[0], masks.shape[1], w.n_states,
                                         masks.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))))
        def step():
            st = aln[0](*aln[1])
            st |= L.plk_set_tree(*tree_args)
            st |= L.plk_set_rate_model(*rate_args)
            st |= L.plk_set_model(*model_args)
            st |= L.plk_loglik(hh, precision, ctypes.byref(out))
            if st != plk.PLK_OK:
                raise plk.PlkError(st, (L.plk_last_error(hh) or b"").decode())

        for _ in range(2):  # warm-up through the same entry points (buffers sized, forms tuned)
            step()
        barrier(world)
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            step()
        return world * e2e_steps / reduce_max(world, time.perf_counter() - t0, dev), out.value

    e2e_value, lnl_e2e = e2e_run(masks8)
    e2e32_value, _ = e2e_run(masks32)
    e2e64_value, _ = e2e_run(masks8, plk.PLK_FP64)
    # where an end-to-end step goes: the host time of each call (the uploads
    # are asynchronous, so their device work overlaps the calls after them;
    # plk_loglik waits for everything)
    aln8 = (hh, masks8.shape[0], masks8.shape[1], w.n_states, masks8.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)))
    calls = (("set_alignment8", lambda: L.plk_set_alignment8(*aln8)),
             ("set_tree", lambda: L.plk_set_tree(*tree_args)),
             ("set_rate_model", lambda: L.plk_set_rate_model(*rate_args)),
             ("set_model", lambda: L.plk_set_model(*model_args)),
             ("loglik", lambda: L.plk_loglik(hh, plk.PLK_FP32S, ctypes.byref(out))))
    e2e_parts = {name: 0.0 for name, _ in calls}
    for _ in range(e2e_steps):
        for name, call in calls:
            t0 = time.perf_counter()
            call()
            e2e_parts[name] += time.perf_counter() - t0
    e2e_parts = {name: 1e3 * t / e2e_steps for name, t in e2e_parts.items()}
    h2d = masks8.nbytes + small

    # errors of the fast form: the lnL and the ancestral probabilities (the
    # conditional and the marginal node states), as the C ABI reports them
    # against the FP64 plain form, and against the FP64 oracle
    fast, f64, abs_err_abi, rel_err_abi = h.loglik_err()
    cells = w.n_tips * w.n_sites
    node_err = {}
    if cells <= ORACLE_CELLS:
        from oracle import oracle as O
        teff = plk.effective_lengths(w.left, w.right, w.bl, False)
        orc = O.loglik(w.left, w.right, w.masks, teff, w.Q, w.freqs, w.cat_rates, w.cat_weights,
                       p_mode=O.P_EXACT, threads=os.cpu_count() or 1, want_cond_norm=True, want_marginal=True)
        ref_lnl = orc.lnl
        ref_name = "error_vs_fp64_oracle"
        for name, mode, ref in (("cond", plk.PLK_NODES_COND, orc.cond_norm),
                                ("marginal", plk.PLK_NODES_MARGINAL, orc.marginal)):
            n32, e_abi = h.node_states_err(mode)
            node_err[name] = {"max_abs_vs_fp64_oracle": float(np.abs(n32 - ref).max()),
                              "max_abs_vs_fp64_engine_abi": e_abi}
            del n32
        del orc
    else:
        ref_lnl = lnl64
        ref_name = "error_vs_fp64_engine"
    h.close()

    if rank != 0:
        return
    hbm_peak, _, peak_src = load_peaks()
    flops_per_launch = algorithmic_flops_per_site(w.n_tips, w.n_states, C) * w.n_sites
    prune_ms = kern_ms[1] / max(n_evals, 1)
    post64_ms = kern64[1] / max(n64, 1)
    fp64_achieved = flops_per_launch / (post64_ms / 1e3) / 1e12
    grid = (w.n_sites + 127) // 128
    req = required_bytes(w, C, grid)
    fp32_achieved = flops_per_launch / (prune_ms / 1e3) / 1e12
    level_bytes = algorithmic_bytes_per_site(w.n_tips, w.n_states, C, 4) * w.n_sites

    # CPU baseline: the reference's algorithm (oracle port), one core, on a
    # bounded sample of this workload
    sample = 1200
    cpu_s = cpu_port_seconds(w, sample, 1)
    cpu_value = 1.0 / (cpu_s * w.n_sites / sample)

    err = {"abs": abs(lnl_timed - ref_lnl), "rel": abs(lnl_timed - ref_lnl) / abs(ref_lnl),
           "e2e_rel": abs(lnl_e2e - ref_lnl) / abs(ref_lnl),
           "fp64_engine_rel": abs(lnl64_timed - ref_lnl) / abs(ref_lnl),
           "abi_plk_loglik_err": {"abs": abs_err_abi, "rel": rel_err_abi},
           "node_states": node_err}
    line = {
        "metric": "lnL evals/s", "value": value, "unit": "evals/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": max_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded simulation of the workload's shapes)",
        "config": workload_config(w),
        "gsite_node_updates_per_s": value * (w.n_tips - 1) * w.n_sites / 1e9,
        "wall_s_timed_region": wall,
        "kernel_ms_per_eval": {"pmat": kern_ms[0] / max(n_evals, 1), "postorder_and_total": prune_ms,
                               "after": kern_ms[2] / max(n_evals, 1),
                               "source": "a second run of the timed steps with the engine's per-kernel events",
                               "ms_per_step_with_kernel_events": prof_ms / args.steps},
        "roofline": {"bound": "hbm", "achieved": req / (prune_ms / 1e3) / 1e9, "peak": hbm_peak, "unit": "GB/s",
                     "frac": req / (prune_ms / 1e3) / 1e9 / hbm_peak, "traffic": load_traffic(h_variant),
                     "kernel": f"{h_variant} (post-order pass)", "required_bytes_per_launch": req,
                     "peak_source": peak_src,
                     "bytes": "tip codes + paired P(t) and tip tables + FP64 site values + block sums; the pass "
                              "keeps every partial vector on chip",
                     "level_by_level_model_bytes": level_bytes,
                     "bound_that_applies": "fp32 (roofline_fp32): the pass is instruction-issue bound, not HBM bound"},
        "roofline_fp32": {"bound": "fp32", "achieved": fp32_achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                          "frac": fp32_achieved / fp32_peak if fp32_peak else None,
                          "flops_per_launch": flops_per_launch,
                          "peak_source": "measured: plk_measure_fp32_peak (fma.rn.f32x2 and fma.rn.f32 chains, "
                                         "4 CTAs per SM, CUDA events), the larger"},
        "fp64_plain_form": {"value": value64, "unit": "evals/s", "ms_per_step": ms64 / steps64, "steps": steps64,
                            "e2e": e2e64_value, "postorder_ms": post64_ms,
                            "roofline_fp64": {
                                "bound": "fp64", "achieved": fp64_achieved, "peak": fp64_peak, "unit": "TFLOP/s",
                                "frac": (fp64_achieved / fp64_peak) if fp64_peak else None,
                                "peak_source": "measured: plk_measure_fp32_peak(packed = 2), fma.rn.f64 chains over "
                                               "4 CTAs per SM, CUDA events",
                                "note": "the plain form multiplies and adds separately in the reference's operation "
                                        "order, one FP64 instruction per flop, so the FP64 issue rate caps it at half "
                                        "of this FMA peak"}},
        "cpu_baseline": {"value": cpu_value, "unit": "evals/s", "cores": 1, "kind": "port",
                         "sample": f"{sample} of {w.n_sites} sites, P(t) rebuilt per (site, edge, category) by the "
                                   f"reference's Taylor-plus-20-squarings, scaled linearly to all sites"},
        "e2e": {"value": e2e_value, "unit": "evals/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": 12,
                "path": "C ABI: plk_set_alignment8 (pinned byte masks) + plk_set_tree + plk_set_rate_model + "
                        "plk_set_model + plk_loglik, every step",
                "with_32bit_masks": {"value": e2e32_value, "h2d_bytes_per_step": int(masks32.nbytes + small),
                                     "path": "plk_set_alignment (pinned 32-bit masks) + the same calls"},
                "host_ms_per_call": e2e_parts},
        # per evaluation: P(t) (which also writes the paired layouts of the
        # tuned form) and the post-order pass, whose last CTA adds up the total
        "gpu_launches": 2 * args.steps,
        ref_name: err,
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)


def load_profile(name: str):
    """Counters of a committed ncu summary (profiles/<name>.json), or None."""
    p = os.path.join(ROOT, "profiles", f"{name}.json")
    if os.path.exists(p):
        return json.load(open(p))
    return None


def run_protein(args):
    """lnL evals/s of the 20-state workload (64 taxa, 20,000 sites, Gamma4):
    each 20-state form forced in turn (CUDA cores, mma.sync split TF32,
    tcgen05 split TF32, tcgen05 split BF16), the FP64 form, then the
    autotuner's choice; per form the post-order time against the FP32 and
    tensor rooflines, its pipe utilisation from the committed ncu summaries,
    and the error against the FP64 oracle."""
    import torch
    from phylommand_gb300 import plk, synth
    from oracle import oracle as O
    w = synth.make("cfg3", seed=3, backend="numpy")
    teff = plk.effective_lengths(w.left, w.right, w.bl, False)
    orc = O.loglik(w.left, w.right, w.masks, teff, w.Q, w.freqs, w.cat_rates, w.cat_weights, p_mode=O.P_EXACT,
                   threads=os.cpu_count() or 1)
    n_int = w.n_tips - 1
    S, C = 20, len(w.cat_rates)
    bytes_per_eval = algorithmic_bytes_per_site(w.n_tips, S, C, 4) * w.n_sites
    flops_per_eval = algorithmic_flops_per_site(w.n_tips, S, C) * w.n_sites
    hbm_peak, bf16_peak, peak_src = load_peaks()
    fp32_peak = measure_fp32_peak(0)
    fp64_peak = measure_fp64_peak(0)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.Stream()
    res = {}
    names = {"1": "prune20_kernel, CUDA cores, 4 warps/tile", "2": "prune20_kernel, tensor cores (split TF32), 4 warps/tile",
             "3": "prune20_kernel, CUDA cores, 8 warps/tile", "4": "prune20_kernel, tensor cores (split TF32), 8 warps/tile",
             "5": "prune20u_kernel, tcgen05 tensor cores (split TF32, TMEM accumulators)",
             "6": "prune20v_kernel, tcgen05 tensor cores, compact form (three CTAs per SM)",
             "7": "prune20v_kernel, tcgen05 tensor cores, compact form, split BF16 (kind::f16)",
             "fp64": "prune_generic_kernel, FP64 partials (the plain form)", "auto": "autotuned"}
    profiles = {"1": "prune20_kernel_protein_64x20k", "3": "prune20_kernel_protein_64x20k",
                "5": "prune20u_kernel_protein_64x20k", "6": "prune20v_kernel_protein_64x20k",
                "7": "prune20v_bf16_kernel_protein_64x20k"}
    clocks = ClockSampler(0)
    clocks.start()
    forms = ("1", "2", "3", "4", "5", "6", "7", "fp64", "auto") if args.form is None else (args.form,)
    for v in forms:
        if v in ("auto", "fp64"):
            os.environ.pop("PLK_PRUNE_VARIANT", None)
        else:
            os.environ["PLK_PRUNE_VARIANT"] = v
        precision = plk.PLK_FP64 if v == "fp64" else plk.PLK_FP32S
        with plk.Handle() as h:
            h.set_alignment(w.masks, S)
            h.set_tree(w.left, w.right, w.bl)
            h.set_rate_model(False)
            h.set_model(w.Q, w.freqs, True, w.cat_rates, w.cat_weights, plk.PLK_P_EXACT)
            h.set_stream(stream.cuda_stream)
            for _ in range(max(args.warmup, 3)):
                h.loglik_async(precision)
            h.loglik_result()
            if v not in ("auto", "fp64") and h.prune_variant() != int(v):
                continue  # the form does not apply to this workload
            torch.cuda.synchronize()
            ms = time_steps(h, stream, flush, args.steps, precision) / args.steps
            # the kernel durations from the same steps again with per-kernel
            # events (kept out of the steps above, where each costs ~2 us)
            h.set_profiling(True)
            time_steps(h, stream, flush, args.steps, precision)
            kern, n = h.kernel_times(reset=True)
            h.set_profiling(False)
            lnl = h.loglik_result()
            post_ms = kern[1] / max(n, 1)
            tflops = flops_per_eval / (post_ms / 1e3) / 1e12
            res[v] = {"kernel": names[v], "evals_per_s": 1e3 / ms, "ms_per_eval": ms, "postorder_ms": post_ms,
                      "gsite_node_updates_per_s": n_int * w.n_sites / (ms / 1e3) / 1e9,
                      "achieved_tflops": tflops,
                      "frac_of_fp32_peak": tflops / fp32_peak if fp32_peak else None,
                      "frac_of_bf16_dense_peak": tflops / bf16_peak,
                      "frac_of_fp64_peak": (tflops / fp64_peak) if (v == "fp64" and fp64_peak) else None,
                      "rel_err_vs_fp64_oracle": abs(lnl - orc.lnl) / abs(orc.lnl),
                      "abs_err_vs_fp64_oracle": abs(lnl - orc.lnl)}
            if v == "auto":
                res[v]["variant"] = h.prune_variant()
            prof = load_profile(profiles.get(v, ""))
            if prof:
                res[v]["ncu"] = prof
    clk = clocks.stop()
    os.environ.pop("PLK_PRUNE_VARIANT", None)
    if args.form is not None:  # one form only (e.g. for a profile of its kernel)
        print(json.dumps({"metric": "lnL evals/s (20 states)", "form": args.form, "variants": res, "clocks": clk}),
              flush=True)
        return
    best = res["auto"]
    tuned = str(best["variant"])
    prof = load_profile(profiles.get(tuned, "")) or {}
    line = {"metric": "lnL evals/s (20 states)", "value": best["evals_per_s"], "unit": "evals/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": best["ms_per_eval"], "higher_is_better": True,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": "20-state, 64-taxon Yule tree, 20,000 sites, exchangeabilities LogNormal(0,1), "
                                   "Gamma4 alpha 1", "l2": "flushed before every step"},
            "roofline": {"bound": "tensor", "achieved": best["achieved_tflops"], "peak": bf16_peak,
                         "unit": "TFLOP/s", "frac": best["achieved_tflops"] / bf16_peak,
                         "traffic": prof.get("dram_bytes_per_launch"), "peak_source": f"{peak_src} (cuBLAS bf16)",
                         "flops_per_launch": flops_per_eval,
                         "note": "algorithmic flops of the 20x20 products; the split forms issue 3x as many "
                                 "tensor products"},
            "roofline_fp32": {"achieved": best["achieved_tflops"], "peak": fp32_peak, "unit": "TFLOP/s",
                              "frac": best["achieved_tflops"] / fp32_peak if fp32_peak else None,
                              "peak_source": "measured: plk_measure_fp32_peak"},
            "algorithmic_bytes_per_eval": bytes_per_eval, "algorithmic_flops_per_eval": flops_per_eval,
            "tuned_form": tuned, "variants": res, "clocks": clk}
    print(json.dumps(line), flush=True)


def run_warmstart(args):
    """Time-to-ML-fit, learned vs plain: 20,000 simulated 32 x 2,000 training
    alignments labelled by the GPU fit, the network trained on them, then
    1,000 held-out 64 x 5,000 alignments fitted from the default start and
    from the network's start (the Newton-start quasi-Newton fit); evaluations
    until each fit first comes within 1e-3 of the plain fit's optimum."""
    import tempfile
    from phylommand_gb300 import warmstart as W
    from phylommand_gb300 import plk
    t0 = time.perf_counter()
    data = W.make_labelled(args.ws_train, 32, 2000, seed=1)
    ws, hist = W.train(data, epochs=200, seed=1)
    prep_s = time.perf_counter() - t0
    clocks = ClockSampler(0)
    clocks.start()
    r = W.evaluate(ws, args.ws_eval, 64, 5000, seed=1001)
    clk = clocks.stop()
    # the same held-out comparison under Nelder-Mead, the reference's NLopt
    # method (LN_NELDERMEAD, src/treeator.cpp:791-805)
    nm = W.evaluate(ws, args.ws_eval, 64, 5000, seed=1001, method=plk.PLK_FIT_NELDER_MEAD)
    with tempfile.TemporaryDirectory() as d:  # the checkpoint round trip
        ws.save(os.path.join(d, "w.npz"))
        again = W.WarmStart.load(os.path.join(d, "w.npz"))
        feats = np.random.default_rng(0).random((4, W.N_FEATURES)).astype(np.float32)
        same = bool(np.array_equal(ws.predict(feats), again.predict(feats)))
    line = {"metric": "lnL evaluations to reach the ML fit, learned start / default start",
            "value": r["evals_to_optimum_ratio_warm_over_plain"], "unit": "ratio", "higher_is_better": False,
            "n_gpus": 1, "dtype": "f32 lnL, bf16 network", "data": "synthetic",
            "config": {"workload": f"train {args.ws_train:,} x (32 taxa, 2,000 sites); evaluate {args.ws_eval:,} x "
                                   "(64 taxa, 5,000 sites); "
                                   "GTR+Gamma4 priors", "train_items": args.ws_train, "eval_items": args.ws_eval,
                       "optimiser": r["method"]},
            "plain": {"evals_to_optimum": r["plain_evals_to_optimum_mean"], "evals_to_stop": r["plain_evals_mean"],
                      "wall_s": r["plain_wall_s"], "rounds": r["plain_rounds"]},
            "warm": {"evals_to_plain_optimum": r["warm_evals_to_plain_optimum_mean"],
                     "evals_to_stop": r["warm_evals_mean"], "wall_s": r["warm_wall_s"], "rounds": r["warm_rounds"]},
            "time_to_fit_ratio": r["wall_ratio_warm_over_plain"],
            "frac_final_within_1e-3_of_plain": r["frac_final_within_tol_of_plain"],
            "max_lnl_deficit": r["max_lnl_deficit"], "judge": r["judge"], "labelling_and_training_s": prep_s,
            "label_fit_s": data.fit_s, "train_s": hist["train_s"], "checkpoint_round_trip": same,
            "nelder_mead": {k: nm[k] for k in ("evals_to_optimum_ratio_warm_over_plain", "plain_evals_to_optimum_mean",
                                               "warm_evals_to_plain_optimum_mean", "plain_evals_mean",
                                               "warm_evals_mean", "wall_ratio_warm_over_plain",
                                               "frac_final_within_tol_of_plain", "max_lnl_deficit", "judge")},
            "clocks": clk}
    print(json.dumps(line), flush=True)


def nni_batch_workload(n_items: int, seed: int):
    """Uneven batch: taxa U{8..256}, sites log-uniform 200-50,000, each with
    its own Yule tree (Exp(mean 0.05)) and GTR+Gamma4 model (exchangeabilities
    U(0.5, 5), frequencies Dir(10^4), alpha 0.5)."""
    from phylommand_gb300 import plk, synth
    rng = np.random.default_rng(seed)
    cr = plk.discrete_gamma(0.5, 4)
    for i in range(n_items):
        n = int(rng.integers(8, 257))
        N = int(np.exp(rng.uniform(np.log(200), np.log(50000))))
        left, right, bl = synth.yule_tree(n, 0.05, rng)
        f = rng.dirichlet(np.full(4, 10.0))
        Q = synth.reversible_q(4, rng.uniform(0.5, 5.0, 6), f)
        masks = plk.simulate(left, right, bl, Q, f, cr, N, seed=int(rng.integers(1 << 62)))
        yield masks, left, right, bl, Q, f, cr


def run_nni(args):
    """Trees scored per second: every batch tree and all its NNI neighbours,
    batched (one persistent launch for the base trees, one for all the
    neighbours) against one plain launch per tree (set the tree, evaluate),
    the latter timed on a sample of the items and scaled by site-node work."""
    from phylommand_gb300 import plk
    from phylommand_gb300.nni import neighbour_tree
    n_items = args.nni_items
    b = plk.Batch(4)
    sample, work = [], []
    t0 = time.perf_counter()
    for i, (masks, left, right, bl, Q, f, cr) in enumerate(nni_batch_workload(n_items, SEED)):
        b.add(masks, left, right, bl)
        b.set_model(i, Q, f, cr, np.full(4, 0.25))
        work.append((masks.shape[0] - 1) * masks.shape[1])
        if i < args.nni_sample:
            sample.append((masks, left, right, bl, Q, f, cr))
    build_s = time.perf_counter() - t0
    counts = [len(b.nni_moves(i)) for i in range(n_items)]
    trees = n_items + sum(counts)
    for _ in range(max(1, args.warmup)):
        b.loglik()
        b.nni_loglik()
    # device time of each batched pass from the batch's own CUDA events
    # (plk_batch_device_ms: graph launch to result copy, and the NNI scoring)
    clocks = ClockSampler(0)
    clocks.start()
    dev_ms = 0.0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        base = b.loglik()
        nni = b.nni_loglik()
        a_ms, n_ms = b.device_ms()
        dev_ms += a_ms + n_ms
    batched_wall_s = (time.perf_counter() - t0) / args.steps
    clk = clocks.stop()
    batched_s = dev_ms / 1e3 / args.steps
    # plain arm: one evaluation per tree through the single-tree C ABI (set
    # the tree, evaluate), CUDA events on the engine's stream around each
    # item's trees
    import torch
    stream = torch.cuda.Stream()
    plain_s, sample_work, err = 0.0, 0.0, 0.0
    w4 = np.full(4, 0.25)
    with plk.Handle() as h:
        h.set_stream(stream.cuda_stream)
        for i, (masks, left, right, bl, Q, f, cr) in enumerate(sample):
            moves = b.nni_moves(i)
            topologies = [(left, right)] + [neighbour_tree(left, right, int(v), int(w)) for v, w in moves]
            batched = [base[i]] + list(nni[i])
            h.set_alignment(masks, 4)
            h.set_tree(left, right, bl)
            h.set_rate_model(False)
            h.set_model(Q, f, True, cr, w4, plk.PLK_P_EXACT)
            h.loglik(plk.PLK_FP32S)  # tuning for this shape
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(stream)
            for L, R in topologies:
                h.set_tree(L, R, bl)
                h.set_rate_model(False)
                h.loglik(plk.PLK_FP32S)
            e1.record(stream)
            torch.cuda.synchronize()
            plain_s += e0.elapsed_time(e1) / 1e3
            sample_work += work[i] * len(topologies)
            for (L, R), got in list(zip(topologies, batched))[:8]:
                h.set_tree(L, R, bl)
                h.set_rate_model(False)
                ref = h.loglik(plk.PLK_FP64)
                err = max(err, abs(got - ref) / abs(ref))
    total_work = float(sum(w * (1 + c) for w, c in zip(work, counts)))
    plain_total_s = plain_s * total_work / sample_work
    line = {"metric": "trees scored/s (512 uneven alignments + all NNI neighbours)", "value": trees / batched_s,
            "unit": "trees/s", "n_items": n_items, "trees": trees, "batched_s_per_pass": batched_s,
            "timing": "CUDA events: the batch's own (plk_batch_device_ms) for the batched arm, on the engine's "
                      "stream around each sampled item's per-tree calls for the plain arm",
            "batched_wall_s_per_pass": batched_wall_s, "clocks": clk,
            "plain_s_per_pass_estimated": plain_total_s, "plain_trees_per_s": trees / plain_total_s,
            "plain_sample_items": len(sample), "speedup_vs_plain_per_tree": plain_total_s / batched_s,
            "max_rel_err_fp32_batched_vs_fp64_per_tree": err, "build_s": build_s, "tuning": b.tuning(),
            "steps": args.steps, "warmup": args.warmup, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "uneven batch: taxa U{8..256}, sites log-uniform 200-50,000, GTR+Gamma4 each",
                       "seed": SEED}}
    b.close()
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="dna", choices=["dna", "nni", "protein", "warmstart"],
                    help="dna: the headline workload; nni: the uneven batch with NNI neighbours; protein: 20 "
                         "states; warmstart: time-to-ML-fit with the learned start")
    ap.add_argument("--taxa", type=int, default=None, help="dna workload: taxa (default 128)")
    ap.add_argument("--sites", type=int, default=None, help="dna workload: sites (default 100,000)")
    ap.add_argument("--nni-items", type=int, default=512)
    ap.add_argument("--nni-sample", type=int, default=24)
    ap.add_argument("--ws-train", type=int, default=20000)
    ap.add_argument("--ws-eval", type=int, default=1000)
    ap.add_argument("--form", default=None, help="protein workload: time only this 20-state form (1-7, fp64, auto)")
    args = ap.parse_args()
    if args.workload == "nni":
        run_nni(args)
        return
    if args.workload == "protein":
        run_protein(args)
        return
    if args.workload == "warmstart":
        run_warmstart(args)
        return
    world, rank, local = (1, 0, 0) if args.impl == "reference" else dist_setup(args.gpus)
    if args.impl == "reference":
        rank = int(os.environ.get("RANK", "0"))
        run_reference(args, world, rank)
        return
    run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
