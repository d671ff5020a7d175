#!/usr/bin/env python
"""Benchmark: tree-likelihood lnL + gradient evaluations per second on one GB300.

Workload (default ``gtr_g4_t1000_b8``): GTR+Gamma4 on a 1,000-taxon Yule tree
with 100,000 simulated DNA sites (compressed to N unique patterns), a batch of
8 branch-length samples.  One *step* = one batched evaluation: the model
set-up (Gamma category rates by the quantile kernel, the normalised rate
matrix, its FP64 eigen system by the device eigensolver), transition matrices,
post-order pass, pre-order adjoint pass and all reductions, giving lnL and
the full gradient (branch lengths, rate matrix -> exchangeabilities and
frequencies, category rates/weights) for every sample.  One *evaluation*
= lnL + gradient for one sample; ``value`` = evaluations / second over all
ranks.  Inputs stay resident in HBM; the stored partials (tens of GB) exceed
the 129 MB L2, so no explicit L2 flush is used.

``--impl reference`` times the reference path on the host cores (all
threads): torchtree's own ``p_t`` + ``calculate_treelikelihood_discrete_rescaled``
+ ``backward`` in FP64 (the copy installed in ``baseline/_ref``; the oracle
port where torchtree cannot be imported).  A step is one sample's lnL and
gradient over one pattern chunk; consecutive steps walk the chunks of the
whole alignment in order, so every step is measured work of the same
workload and nothing is extrapolated.  That arm loads nothing from this
package's native library (the alignment is compressed with numpy).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "lnL+grad evals/s: FP32-rescaled batched vs FP64 drop-in, 1 GB300; p99 latency"
UNIT = "evals/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("gb300", "reference"), default="gb300")
    ap.add_argument("--workload", default="gtr_g4_t1000_b8")
    ap.add_argument("--precision", choices=("f32", "f64"), default="f32")
    ap.add_argument("--fp64-steps", type=int, default=2, help="steps of the FP64 drop-in comparison (0: skip)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ref-chunk-patterns", type=int, default=10240,
                    help="patterns per chunk of the reference path on the CPU (one chunk per reference step; "
                         "the CPU-baseline leg evaluates every chunk of sample 0)")
    ap.add_argument("--sites", type=int, default=None, help="override the workload's site count")
    ap.add_argument("--tips", type=int, default=None, help="override the workload's tip count")
    ap.add_argument("--batch", type=int, default=None, help="override the workload's batch")
    ap.add_argument("--slab-patterns", type=int, default=None,
                    help="4-state plans: hold this many patterns' partials at once (the gradient recomputes "
                         "the post-order slab by slab)")
    ap.add_argument("--serving", action="store_true",
                    help="serving mix instead of the batched step: Poisson arrivals from many chains over "
                         "resident data sets, continuous batching through captured CUDA graphs")
    ap.add_argument("--serving-datasets", type=int, default=32)
    ap.add_argument("--serving-chains", type=int, default=256)
    ap.add_argument("--serving-requests", type=int, default=1024)
    ap.add_argument("--serving-slots", type=int, default=4)
    ap.add_argument("--serving-fixed-slots", action="store_true",
                    help="every plan gets --serving-slots slots (default: fewer for data sets whose one sample "
                         "fills the GPU, serving.slots_for)")
    ap.add_argument("--serving-merge-depth", type=int, default=2,
                    help="merged DNA steps in flight at once (0: no merging, one graph per data set)")
    ap.add_argument("--serving-max-tips", type=int, default=2000)
    ap.add_argument("--serving-max-sites", type=int, default=50000)
    ap.add_argument("--timetree", action="store_true",
                    help="time-tree prior step instead: node-height ratio transform with log|det J| and the "
                         "constant-size coalescent, values and gradients, for a batch of samples")
    ap.add_argument("--timetree-cpu-batch", type=int, default=32, help="samples in the CPU oracle's sample")
    return ap.parse_args()


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi while running."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.lines:
            return None
        sm, mx, reasons = [], None, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for name, flag in zip(names, parts[4:8]):
                if flag.lower() == "active":
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def replica_throughput(seconds: float, units_per_rank: int, world: int, device=None) -> tuple:
    """Whole-job throughput of ``world`` independent replicas: the slowest
    rank's time (max over ranks) and units/s over all ranks."""
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    slowest = float(t.item())
    return slowest, units_per_rank * world / slowest


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def measured_tensor_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return float(json.loads(p.read_text())["bf16_tflops"])
    return 1900.0


def workload(args):
    from torchtree_gb300 import datatype, patterns, synthetic

    wl = synthetic.named_workload(args.workload, **workload_overrides(args))
    ca = patterns.compress(wl.sequences, datatype.get(wl.data_type))
    return wl, ca


def rate_matrix(model, exch, pi):
    """Unnormalised Q of a workload's model (torch, differentiable)."""
    import torch

    from torchtree_gb300 import substitution

    if model in ("gtr", "hky"):
        return substitution.gtr_q(exch, pi)
    if model == "general":
        return substitution.general_symmetric_q(exch, pi, pi.shape[-1])
    return substitution.mg94_q(torch.ones_like(exch[..., :1]), exch[..., 1:2], exch[..., :1], pi)


def cpu_baseline(wl, chunk_patterns):
    """The reference path on the host cores: one whole evaluation (all
    patterns, pattern chunk by pattern chunk) of sample 0, timed."""
    from oracle import reference_arm as RA

    ref = RA.ReferencePath(wl, chunk_patterns)
    t0 = time.perf_counter()
    lnl, grads = ref.evaluate(0)
    sec = time.perf_counter() - t0
    return {"value": 1.0 / sec, "unit": UNIT, "cores": ref.threads, "kind": ref.kind,
            "sample": (f"{ref.describe()}; one whole evaluation (lnL + gradient) of sample 0 over all "
                       f"{ref.N} patterns in {len(ref.chunks)} chunks, timed once"),
            "seconds_per_eval": sec}, (lnl, grads, ref)


def fp32_error(got, want):
    """FP32 results against the FP64 drop-in on the same inputs (the drop-in
    equals the FP64 oracle to 1e-10 in the parity tests): lnL relative error
    per sample, and each gradient's largest error relative to its largest
    entry (dlnL/dQ, dlnL/dt, dlnL/dr)."""
    lnl, want_lnl = got[0], want[0]
    out = {"vs": "FP64 drop-in on the same inputs",
           "lnl_max_rel_err": float(((lnl - want_lnl).abs() / want_lnl.abs()).max())}
    for name, g, w in zip(("dq", "dbranch", "drate"), got[1:], want[1:]):
        out[f"{name}_max_err_rel_to_max"] = float((g - w).abs().max() / w.abs().max().clamp_min(1e-300))
    return out


def workload_overrides(args):
    over = {}
    if args.sites:
        over["site_count"] = args.sites
    if args.tips:
        over["tip_count"] = args.tips
    if args.batch:
        over["batch"] = args.batch
    return over


def bench_config(args, wl, n_patterns, sites, slab=None):
    """The ``config`` object of both arms' lines (identical for the same workload)."""
    S = wl.state_count
    cfg = {"workload": args.workload, "tips": wl.topology.tip_count, "sites": int(sites),
           "patterns": int(n_patterns), "batch": int(wl.branch_lengths.shape[0]), "categories": wl.categories,
           "states": S,
           "substitution_model": {"gtr": "GTR", "hky": "HKY", "general": "general symmetric 20-state",
                                  "mg94": "MG94 codon (GY94-style)"}[wl.model] + f"+Gamma{wl.categories}",
           "l2": "inputs (stored partials) larger than L2; no flush",
           "parallelism": f"replicas x{args.gpus}"}
    if slab:
        cfg["slab_patterns"] = slab
        cfg["slabs"] = ("partials held one pattern slab at a time; the pre_order_adjoint time includes the "
                        "post-order recompute")
    return cfg


def plugin_e2e(args, wl, dev, steps):
    """lnL + gradient through the torchtree plug-in class, as a torchtree user
    calls it: ``torchtree_gb300.TreeLikelihoodModel`` built by torchtree's JSON
    machinery over torchtree's GTR / HKY model, this package's GammaSiteModel
    and a fixed-topology tree model, parameters as CPU tensors (the class
    copies them to the device, runs the engine and returns lnL to the host;
    ``backward`` brings the gradients back).  None when torchtree cannot be
    imported or the model is not GTR / HKY."""
    import torch

    from oracle import reference as R
    from oracle import reference_arm as RA

    if wl.model not in ("gtr", "hky") or R.import_torchtree() is None:
        return None
    from torchtree import Parameter
    from torchtree.core.utils import process_object
    from torchtree.evolution.substitution_model import GTR, HKY

    from torchtree_gb300.model import GammaSiteModel  # noqa: F401  (registers the class)

    tips, weights = RA.compress(wl.sequences, wl.data_type)
    names = wl.topology.tip_names
    leaf = lambda a: torch.tensor(np.asarray(a), dtype=torch.float64).requires_grad_()  # noqa: E731
    p_bl, p_pi, p_shape = Parameter("bl", leaf(wl.branch_lengths)), Parameter("pi", leaf(wl.pi)), \
        Parameter("shape", leaf(wl.shape))
    if wl.model == "hky":
        p_ex = Parameter("kappa", leaf(wl.exch[:, 1:2]))
        subst = HKY("subst", p_ex, p_pi)
    else:
        p_ex = Parameter("exch", leaf(wl.exch))
        subst = GTR("subst", p_ex, p_pi)
    dic = {"tree": R.fixed_tree_class()(wl.topology.postorder, names, p_bl), "subst": subst,
           "sp": R.PatternSource(tips, weights)}
    dic["site"] = process_object({"id": "site", "type": "torchtree_gb300.GammaSiteModel", "shape": "shape",
                                  "categories": wl.categories}, dict(dic, shape=p_shape))
    like = process_object({"id": "like", "type": "torchtree_gb300.TreeLikelihoodModel", "tree_model": "tree",
                           "site_model": "site", "substitution_model": "subst", "site_pattern": "sp",
                           "precision": args.precision}, dic)
    like.rescale = True
    params = (p_bl, p_ex, p_pi, p_shape)
    hosts = [p.tensor.detach().clone() for p in params]

    def one():
        for p, h in zip(params, hosts):  # new parameter values: listeners invalidate the cached lnL
            p.tensor = h.clone().requires_grad_()
        lnl = like()
        lnl.sum().backward()
        return sum(p.tensor.grad.numel() * 8 for p in params) + lnl.numel() * 8

    for _ in range(2):
        one()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        d2h = one()
    torch.cuda.synchronize()
    sec = time.perf_counter() - t0
    b = int(wl.branch_lengths.shape[0])
    return {"value": b * steps / sec, "unit": UNIT, "h2d_bytes_per_step": int(sum(h.numel() * 8 for h in hosts)),
            "d2h_bytes_per_step": int(d2h),
            "what": "torchtree_gb300.TreeLikelihoodModel from JSON (torchtree GTR/HKY, GammaSiteModel, CPU "
                    "parameters) called and back-propagated like the reference class"}


def reference_error(res, ref_lnl, ref_grads, n_free):
    """A GPU result's sample 0 against the reference path's: lnL relative
    error, and the branch-length and category-rate gradients' largest error
    relative to their largest entry."""
    lnl, _, dbl, dr = (x.double() for x in res)
    g_bl, g_r = ref_grads[0], ref_grads[3]
    return {"lnl_rel_err": float(abs(float(lnl[0]) - ref_lnl) / abs(ref_lnl)),
            "dbranch_err_rel_to_max": float((dbl[0, :n_free] - g_bl).abs().max() / g_bl.abs().max()),
            "drate_err_rel_to_max": float((dr[0] - g_r).abs().max() / g_r.abs().max())}


def run_reference(args):
    """The reference path on the host cores, timed step by step (rank 0 only)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import reference_arm as RA
    from torchtree_gb300 import synthetic

    wl = synthetic.named_workload(args.workload, **workload_overrides(args))
    ref = RA.ReferencePath(wl, args.ref_chunk_patterns)
    b, nch = int(wl.branch_lengths.shape[0]), len(ref.chunks)
    sizes = [hi - lo for lo, hi in ref.chunks]

    def step(i):
        c = i % nch
        ref.evaluate_chunk((i // nch) % b, c)
        return sizes[c]

    for i in range(args.warmup):
        step(i)
    per, done = [], 0
    t0 = time.perf_counter()
    for i in range(args.steps):
        t1 = time.perf_counter()
        done += step(args.warmup + i)
        per.append(time.perf_counter() - t1)
    wall = time.perf_counter() - t0
    value = done / ref.N / wall  # whole evaluations (lnL + gradient of one sample) per second
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": wall / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": f"synthetic (seeded Yule tree, alignment simulated under the model: {wl.data_type})",
        "impl": "reference",
        "config": bench_config(args, wl, ref.N, ref.sites),
        "latency_ms": {"p50": float(np.percentile(per, 50)) * 1e3, "p99": float(np.percentile(per, 99)) * 1e3,
                       "what": "one step: one sample's lnL + gradient over one pattern chunk"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": ref.threads, "kind": ref.kind,
                         "sample": (f"{ref.describe()}; step = one sample over one chunk of <= "
                                    f"{args.ref_chunk_patterns} of the {ref.N} patterns ({nch} chunks), "
                                    f"steps walk the chunks in order ({done} pattern evaluations timed)")},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "setup_s": {"compress": ref.compress_s},
    }
    print(json.dumps(line), flush=True)


def serving_mix(args, rng):
    """Resident data sets of the serving mix: taxa log-uniform in [20, max tips], sites
    log-uniform in [500, max sites], 70 % DNA GTR+G4 / 30 % amino-acid general
    symmetric + G4 (exchangeabilities ~ Gamma(1,1), frequencies ~ Dirichlet(1^20)).
    Tip states are i.i.d. uniform (only the shapes matter for the timing), one
    pattern per site."""
    from torchtree_gb300 import synthetic
    from torchtree_gb300.patterns import CompressedAlignment
    from torchtree_gb300.serving import ModelSpec

    out = []
    for d in range(args.serving_datasets):
        T = int(round(np.exp(rng.uniform(np.log(20), np.log(args.serving_max_tips)))))
        N = int(round(np.exp(rng.uniform(np.log(500), np.log(args.serving_max_sites)))))
        protein = rng.random() < 0.3
        S = 20 if protein else 4
        topo = synthetic.yule_topology(T, rng)
        codes = rng.integers(0, S, size=(T, N), dtype=np.uint8)
        ca = CompressedAlignment(codes=codes, table=np.vstack([np.eye(S), np.ones((1, S))]),
                                 weights=np.ones(N), columns=np.zeros((T, 0), dtype=np.uint8))
        spec = ModelSpec("general" if protein else "gtr")
        out.append((f"ds{d}", topo, ca, S, spec))
    return out


def chain_params(rng, topo, S):
    B = 2 * topo.tip_count - 3
    exch = rng.gamma(1.0, 1.0, S * (S - 1) // 2) if S == 20 else rng.dirichlet(np.ones(6))
    return {"branch_lengths": rng.exponential(0.05, B), "exch": exch, "pi": rng.dirichlet(np.ones(S)),
            "shape": np.array([0.5])}


def run_serving(args):
    import torch

    from torchtree_gb300 import serving
    from torchtree_gb300.likelihood import PhyloLikelihood

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    rng = np.random.default_rng(7)
    mix = serving_mix(args, rng)
    chains = [(c % len(mix), chain_params(rng, mix[c % len(mix)][1], mix[c % len(mix)][3]))
              for c in range(args.serving_chains)]
    srv = serving.LikelihoodServer(slots=args.serving_slots, precision="f32", merge=args.serving_merge_depth > 0,
                                   merge_depth=max(1, args.serving_merge_depth),
                                   size_slots=not args.serving_fixed_slots)
    for name, topo, ca, S, spec in mix:
        srv.add_dataset(name, topo, ca, S, spec)
    srv.start()

    def request(c):
        d, p = chains[c]
        q = dict(p)
        q["branch_lengths"] = p["branch_lengths"] * np.exp(rng.normal(0.0, 0.01, p["branch_lengths"].shape))
        return mix[d][0], q

    # warm-up: every data set once (plan creation, autotuning, graph capture), then a
    # closed-loop burst to estimate capacity
    t0 = time.perf_counter()
    for c in range(len(mix)):
        srv.submit(*request(c)).result()
    setup_s = time.perf_counter() - t0
    srv.reset_stats()
    burst = [srv.submit(*request(c)) for c in range(min(len(chains), 4 * len(mix)))]
    t1 = time.perf_counter()
    for f in burst:
        f.result()
    capacity = len(burst) / (time.perf_counter() - t1)
    burst_stats = srv.latency_stats()
    rate = 0.7 * capacity
    srv.reset_stats()
    # open-loop Poisson arrivals at 70 % of the measured capacity
    gaps = rng.exponential(1.0 / rate, args.serving_requests)
    picks = rng.integers(0, len(chains), args.serving_requests)
    futs = []
    start = time.perf_counter()
    due = start
    for g, c in zip(gaps, picks):
        due += g
        wait = due - time.perf_counter()
        if wait > 0:
            time.sleep(wait)
        futs.append(srv.submit(*request(int(c))))
    for f in futs:
        f.result()
    wall = time.perf_counter() - start
    stats = srv.latency_stats()
    srv.stop()
    # one-at-a-time FP64 drop-in calls (batch 1, eager) on a sample of the same requests
    sample = [request(int(c)) for c in picks[: min(32, len(picks))]]
    lik_cache = {}
    t2 = time.perf_counter()
    for name, p in sample:
        d = next(i for i, m in enumerate(mix) if m[0] == name)
        _, topo, ca, S, spec = mix[d]
        if name not in lik_cache:
            lik_cache.clear()
            torch.cuda.empty_cache()
            lik_cache[name] = PhyloLikelihood(topo, ca, S, 4, batch=1, precision="f64")
        lik = lik_cache[name]
        prep = serving.host_prepare(serving.Dataset(name, topo, ca, S, spec), p)
        dev = lik.device
        q, bls_, r_, p_, pi_ = (prep[k].to(dev).unsqueeze(0) for k in ("q", "bls", "rates", "probs", "pi"))
        lik.rescale = True
        lnl = lik.evaluate_rate_matrix(q, pi_, bls_, r_, p_, pi_)
        lnl.sum().backward()
        torch.cuda.synchronize()
    fp64_rate = len(sample) / (time.perf_counter() - t2)
    lik_cache.clear()
    sizes = [(m[1].tip_count, m[2].pattern_count, m[3]) for m in mix]
    line = {
        "metric": "serving lnL+grad requests/s, Poisson mix over resident data sets, 1 GB300; p50/p99 latency",
        "value": len(futs) / wall, "unit": "requests/s", "higher_is_better": True, "n_gpus": 1,
        "latency_ms": {"p50": stats.get("p50_ms"), "p99": stats.get("p99_ms"), "mean": stats.get("mean_ms"),
                       "queue_wait_p50": stats.get("wait_p50_ms"), "service_p50": stats.get("service_p50_ms")},
        "offered_rate": rate, "capacity_closed_loop": capacity,
        "closed_loop": {"requests": burst_stats.get("count"), "launches": burst_stats.get("launches"),
                        "requests_per_launch": burst_stats.get("requests_per_launch"),
                        "merged_steps": burst_stats.get("merged_steps"),
                        "requests_per_merged_step": burst_stats.get("requests_per_merged_step"),
                        "latency_p50_ms": burst_stats.get("p50_ms"),
                        "what": f"{len(burst)} requests submitted at once (chain c on data set c mod {len(mix)}); "
                                "counters of this phase only"},
        "requests": len(futs),
        "batches": stats.get("batches"), "launches": stats.get("launches"),
        "requests_per_launch": stats.get("requests_per_launch"),
        "merged_steps": stats.get("merged_steps"), "requests_per_merged_step": stats.get("requests_per_merged_step"),
        "merge_host_ms_per_step": stats.get("merge_host_ms_per_step"), "merge_depth": args.serving_merge_depth,
        "admissions": stats.get("admissions"), "evictions": stats.get("evictions"),
        "setup_s": setup_s, "dtype": "f32",
        "fp64_one_at_a_time": {"value": fp64_rate, "unit": "requests/s", "sample": len(sample),
                               "what": "PhyloLikelihood FP64, batch 1, eager, sequential"},
        "speedup_vs_fp64_one_at_a_time": (len(futs) / wall) / fp64_rate,
        "data": "synthetic: Yule trees, i.i.d. uniform tip states, GTR+G4 / general 20-state+G4",
        "config": {"workload": "serving_mix", "datasets": len(mix), "chains": len(chains),
                   "slots": args.serving_slots, "fixed_slots": args.serving_fixed_slots, "dna": sum(1 for s in sizes if s[2] == 4),
                   "protein": sum(1 for s in sizes if s[2] == 20), "tips_range": [min(s[0] for s in sizes),
                                                                                    max(s[0] for s in sizes)],
                   "patterns_range": [min(s[1] for s in sizes), max(s[1] for s in sizes)]},
    }
    print(json.dumps(line), flush=True)


def run_timetree(args):
    """Time-tree prior step for a batch of samples: ratios -> internal heights,
    branch lengths and log|det J| (tree_height_transform.py:7-99), the
    constant-size coalescent log-density of the heights (coalescent.py:86-134),
    and the gradient of log p + log|det J| with respect to the ratios and the
    population size.  The reference times the same operations one sample at a
    time (benchmarks/benchmark.py:441-789)."""
    import torch

    from torchtree_gb300 import synthetic
    from torchtree_gb300.timetree import TimeTree

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    rng = np.random.default_rng(11)
    T = args.tips or 1000
    b = args.batch or 16384
    topo = synthetic.yule_topology(T, rng)
    times = rng.uniform(0.0, 5.0, T)  # heterochronous tips (sampling times before the present)
    lb = np.zeros(T - 1)
    for v, l, r in topo.postorder:
        lb[v - T] = max(times[l] if l < T else lb[l - T], times[r] if r < T else lb[r - T])
    x_host = rng.uniform(0.05, 0.95, (b, T - 1))
    x_host[:, T - 2] = lb[T - 2] + rng.exponential(5.0, b)  # root height above its lower bound
    th_host = rng.lognormal(1.0, 0.3, b)
    tree = TimeTree(topo.postorder, times)
    x = torch.tensor(x_host, device=dev)
    th = torch.tensor(th_host, device=dev)

    def step(xx, tt):
        xx = xx.detach().requires_grad_()
        tt = tt.detach().requires_grad_()
        h, bl, ld = tree.ratio_transform(xx)
        lp = tree.constant_coalescent(h, tt)
        total = lp + ld
        gx, gth = torch.autograd.grad(total.sum(), (xx, tt))
        return total, gx, gth

    for _ in range(max(args.warmup, 3)):
        step(x, th)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    with ClockSampler(local) as clocks:
        ev[0].record(stream)
        for i in range(args.steps):
            step(x, th)
            ev[i + 1].record(stream)
        torch.cuda.synchronize()
    total_ms = ev[0].elapsed_time(ev[-1])
    per = [ev[i].elapsed_time(ev[i + 1]) for i in range(args.steps)]
    value = b * args.steps / (total_ms / 1e3)
    # per-kernel times (the C-ABI calls on the stream)
    e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    xx = x.detach().requires_grad_()
    e[0].record(stream)
    h, bl, ld = tree.ratio_transform(xx)
    e[1].record(stream)
    lp = tree.constant_coalescent(h, th)
    e[2].record(stream)
    torch.autograd.grad((lp + ld).sum(), xx)
    e[3].record(stream)
    torch.cuda.synchronize()
    k_ms = {"ratio_transform": e[0].elapsed_time(e[1]), "constant_coalescent": e[1].elapsed_time(e[2]),
            "backward": e[2].elapsed_time(e[3])}
    # end to end: host ratios and population sizes in (pinned), values and gradients out
    xp, tp = torch.tensor(x_host).pin_memory(), torch.tensor(th_host).pin_memory()
    outs = [torch.empty(b, dtype=torch.float64).pin_memory(), torch.empty(b, T - 1, dtype=torch.float64).pin_memory(),
            torch.empty(b, dtype=torch.float64).pin_memory()]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        res = step(xp.to(dev, non_blocking=True), tp.to(dev, non_blocking=True))
        for o, r in zip(outs, res):
            o.copy_(r, non_blocking=True)
        torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    # CPU oracle (torch FP64 + autograd, all host threads) on a sample of the batch
    from oracle import timetree as OT

    nb = min(args.timetree_cpu_batch, b)
    xc = torch.tensor(x_host[:nb]).requires_grad_()
    tc_ = torch.tensor(th_host[:nb]).requires_grad_()
    t1 = time.perf_counter()
    hc, _, ldc = OT.ratio_transform(topo.postorder_list(), list(times), xc)
    lpc = OT.constant_coalescent(list(times), hc, tc_)
    gxc, _ = torch.autograd.grad((lpc + ldc).sum(), (xc, tc_))
    cpu_s = time.perf_counter() - t1
    res = step(x[:nb], th[:nb])
    check = float(torch.max(torch.abs(res[0].cpu() - (lpc + ldc).detach())))
    I = T - 1
    # bytes a launch sequence must move per sample: ratios in, heights / branch
    # lengths out (ratio transform); heights in, height gradients out
    # (coalescent); ratios, heights and the three incoming gradients in, ratio
    # gradients out (backward)
    per_sample = 8 * (I + I + (2 * T - 2) + 1) + 8 * (I + I + 2) + 8 * (I + I + I + (2 * T - 2) + 1 + I)
    peak, peak_kind = measured_peaks()
    achieved = per_sample * b / (sum(k_ms.values()) / 1e3) / 1e9
    line = {
        "metric": "time-tree prior evals/s: ratio transform + log|det J| + constant coalescent, values and gradients",
        "value": value, "unit": "samples/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded Yule tree, uniform tip dates, uniform ratios)",
        "config": {"workload": f"timetree_t{T}_b{b}", "tips": T, "batch": b,
                   "l2": f"inputs {b * I * 8 / 1e6:.0f} MB per tensor; no flush"},
        "latency_ms": {"p50": float(np.percentile(per, 50)), "p99": float(np.percentile(per, 99))},
        "kernels_ms": k_ms,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind, "traffic": None, "per_launch_bytes": per_sample * b},
        "cpu_baseline": {"value": nb / cpu_s, "unit": "samples/s", "cores": torch.get_num_threads(), "kind": "port",
                         "sample": f"{nb} samples of the same tree and inputs (oracle: torch FP64 + autograd)",
                         "max_abs_diff": check},
        "e2e": {"value": b * args.steps / e2e_s, "unit": "samples/s",
                "h2d_bytes_per_step": int(xp.numel() * 8 + tp.numel() * 8),
                "d2h_bytes_per_step": int(sum(o.numel() for o in outs) * 8)},
        "gpu_launches": 3, "clocks": clocks.summary(),
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.serving:
        run_serving(args)
        return
    if args.timetree:
        run_timetree(args)
        return
    import torch
    import torch.distributed as dist

    from torchtree_gb300 import _native, site_models, substitution
    from torchtree_gb300.engine import LikelihoodEngine
    from torchtree_gb300.likelihood import PhyloLikelihood, batch_inputs

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        dist.init_process_group("nccl", device_id=dev)

    def barrier():
        if world > 1:
            dist.barrier()

    wl, ca = workload(args)
    b = int(wl.branch_lengths.shape[0])
    T, N, K, S = wl.topology.tip_count, ca.pattern_count, wl.categories, ca.table.shape[1]
    bl, exch, pi, shape = batch_inputs(wl, dev)
    zeros = torch.zeros(b, 1, dtype=torch.float64, device=dev)
    bls = torch.cat([bl, zeros], -1).contiguous()

    side = torch.cuda.Stream(device=dev)

    def model_setup():
        """The per-step model work on the device: Gamma category rates
        (quantile kernel, on a side stream: it and the eigensolver are
        independent and each fills only a few SMs), the normalised rate
        matrix (a few torch ops) and its FP64 eigen system (device
        eigensolver)."""
        main = torch.cuda.current_stream()
        side.wait_stream(main)
        with torch.cuda.stream(side):
            r, p = site_models.gamma_rates(shape, K)
            r, p = r.contiguous(), p.expand(b, K).contiguous()
        qn = substitution.normalise(rate_matrix(wl.model, exch, pi), pi)
        lam_, u_, w_ = substitution.device_eigen(qn, pi)
        main.wait_stream(side)
        r.record_stream(main)
        p.record_stream(main)
        return lam_, u_, w_, r, p

    lam, u, w, rates, probs = model_setup()

    def make_engine(precision):
        return LikelihoodEngine(wl.topology.postorder, T, S, K, ca.codes, ca.table, ca.weights, batch=b,
                                precision=precision, device=dev)

    eng = make_engine(args.precision)
    if args.slab_patterns is not None:
        eng.set_option(_native.TT_OPT_SLAB_PATTERNS, args.slab_patterns)
    slab = eng.get_option(_native.TT_OPT_SLAB_PATTERNS)
    stream = torch.cuda.current_stream()

    def step(e):
        lam_, u_, w_, r_, p_ = model_setup()
        e.set_eigen(lam_, u_, w_, bls, r_)
        lnl = e.log_likelihood(p_, pi, rescale=True, keep_partials=True)
        e.gradient(p_, pi)
        return (lnl,) + e.rate_matrix_gradient(lam_, u_, w_, bls, r_)

    for _ in range(max(args.warmup, 3)):
        step(eng)
    torch.cuda.synchronize()
    assert eng.device_status() == 0
    launches0 = eng.launch_count
    barrier()
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    with ClockSampler(local) as clocks:
        ev[0].record(stream)
        for i in range(args.steps):
            step(eng)
            ev[i + 1].record(stream)
        torch.cuda.synchronize()
    barrier()
    launches = eng.launch_count - launches0 + 2 * args.steps  # + the quantile and eigen kernels
    per_step = [ev[i].elapsed_time(ev[i + 1]) for i in range(args.steps)]
    slowest_s, value = replica_throughput(ev[0].elapsed_time(ev[-1]) / 1e3, b * args.steps, world, dev)
    total_ms = slowest_s * 1e3

    # per-call timing of the two pruning kernels (each call: one pruning
    # kernel + its small reduction kernels) for the roofline
    fw, bw, fo = [], [], []
    for _ in range(3):
        e0, e1, e2, e3 = (torch.cuda.Event(enable_timing=True) for _ in range(4))
        eng.set_eigen(lam, u, w, bls, rates)
        e0.record(stream)
        eng.log_likelihood(probs, pi, rescale=True, keep_partials=True)
        e1.record(stream)
        eng.gradient(probs, pi)
        e2.record(stream)
        eng.log_likelihood(probs, pi, rescale=True, keep_partials=False)  # lnL only
        e3.record(stream)
        torch.cuda.synchronize()
        fw.append(e0.elapsed_time(e1))
        bw.append(e1.elapsed_time(e2))
        fo.append(e2.elapsed_time(e3))
    fw_ms, bw_ms, fo_ms = statistics.median(fw), statistics.median(bw), statistics.median(fo)
    elem = 4 if args.precision == "f32" else 8
    I = T - 1
    # algorithmic bytes per launch: the level-by-level pruning model (children
    # read back from HBM, outside partials written and read), per sample
    p_n = K * S * N * elem
    model_fw = b * (I * (p_n + 4 * N) + (I - 1) * p_n + T * N + 4 * N)
    model_bw = b * ((I - 1) * p_n + (I - 1) * p_n + (I - 1) * p_n + I * 4 * N)
    # bytes this design moves: stored partials written once and read once, tip
    # codes, and the per-tile gradient blocks of the adjoint
    tile = 64
    ntiles = -(-N // tile)
    design_fw = b * ((I - 1) * p_n + T * N + 8 * N)
    design_bw = b * ((I - 1) * p_n + T * N + 8 * N + (2 * T - 2) * ntiles * K * S * S * elem)
    if S == 4 and args.precision == "f32" and eng.get_option(_native.TT_OPT_INPLACE_ADJOINT):
        # outside partials stored over the post-order tiles: written once, read once
        sched, _ = _native.schedule(T, wl.topology.postorder)
        design_bw += b * 2 * int((sched[:, 9] & 1).sum()) * p_n
    peak, peak_kind = measured_peaks()

    def entry(ms, model, design):
        return {"ms": ms, "bytes": model, "gbs": model / ms / 1e6, "design_bytes": design,
                "dram_gbs": design / ms / 1e6}

    kernels = {"post_order": entry(fw_ms, model_fw, design_fw),
               "pre_order_adjoint": entry(bw_ms, model_bw, design_bw)}
    lnl_only = {"ms": fo_ms, "evals_per_s": b / (fo_ms / 1e3),
                "what": "post-order pass without storing partials (lnL only, no gradient)"}
    dom = max(kernels, key=lambda k: kernels[k]["ms"])
    achieved = kernels[dom]["gbs"]
    roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": peak_kind, "traffic": None,
                "per_launch_bytes": kernels[dom]["bytes"],
                "bytes_model": "level-by-level pruning traffic (5 partial passes per evaluation)",
                "dram_achieved": kernels[dom]["dram_gbs"], "dram_frac": kernels[dom]["dram_gbs"] / peak,
                "kernels": kernels}
    if S != 4:  # amino-acid / codon: level-scheduled kernels; algorithmic flops of the products
        s_flop = 2 * S * S * K * N * b  # one S x S matrix applied to one category's patterns
        fw_flops = I * 2 * s_flop  # the two children's products of every internal node
        # adjoint: P^T u for every internal child (outside partials) and sum_p u x^T for every
        # branch (gradient blocks); the children's products come from the post-order
        bw_flops = ((I - 1) + (2 * T - 2)) * s_flop
        for name, fl in (("post_order", fw_flops), ("pre_order_adjoint", bw_flops)):
            kernels[name]["flops"] = fl
            kernels[name]["tflops"] = fl / kernels[name]["ms"] / 1e9
        tflops_peak = measured_tensor_peak()
        roofline["tensor_post_order"] = {
            "bound": "tensor", "achieved": kernels["post_order"]["tflops"], "peak": tflops_peak,
            "unit": "TFLOP/s", "frac": kernels["post_order"]["tflops"] / tflops_peak,
            "what": "codon post-order as split-TF32 tcgen05 MMAs (3 MMAs per product, counted once); "
                    "peak = measured dense BF16 (TF32 runs at half that rate)"} if S > 20 else None
        if S > 20 and args.precision == "f32" and eng.get_option(_native.TT_OPT_TENSOR_CORE_ADJOINT):
            roofline["tensor_adjoint"] = {
                "bound": "tensor", "achieved": kernels["pre_order_adjoint"]["tflops"], "peak": tflops_peak,
                "unit": "TFLOP/s", "frac": kernels["pre_order_adjoint"]["tflops"] / tflops_peak,
                "what": "codon adjoint as split-TF32 tcgen05 MMAs (outside partials and gradient blocks, "
                        "3 MMAs per product, counted once); peak = measured dense BF16"}
    traffic_file = ROOT / "profiles" / "traffic.json"
    if traffic_file.exists():
        tr = json.loads(traffic_file.read_text()).get(args.workload, {}).get(dom)
        if tr:
            roofline["traffic"] = tr

    # FP64 drop-in on the same workload; its results measure the FP32 error
    fp64, accuracy, got, want = None, None, None, None
    if args.fp64_steps > 0 and args.precision == "f32":
        got = [x.cpu() for x in step(eng)]
        del eng
        torch.cuda.empty_cache()
        e64 = make_engine("f64")
        want = [x.cpu() for x in step(e64)]
        torch.cuda.synchronize()
        accuracy = fp32_error(got, want)
        a, z = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(args.fp64_steps):
            step(e64)
        z.record(stream)
        torch.cuda.synchronize()
        ms = a.elapsed_time(z) / args.fp64_steps
        fp64 = {"value": b / (ms / 1e3), "unit": UNIT, "ms_per_step": ms, "steps": args.fp64_steps}
        del e64
        torch.cuda.empty_cache()
        eng = None

    # end to end through the public API: host inputs -> H2D -> lnL+grad -> D2H
    e2e = None
    if not args.no_e2e:
        lik = PhyloLikelihood(wl.topology, ca, S, K, batch=b, precision=args.precision, device=dev)
        lik.rescale = True
        hosts = [x.detach().cpu().pin_memory() for x in (bl, exch, pi, shape)]
        h2d = sum(x.numel() * x.element_size() for x in hosts)

        def e2e_step():
            d_bl, d_ex, d_pi, d_sh = (x.to(dev, non_blocking=True) for x in hosts)
            d_bl.requires_grad_()
            d_ex.requires_grad_()
            d_pi.requires_grad_()
            r, p = site_models.gamma_rates(d_sh, K)
            lnl = lik(d_bl, rate_matrix(wl.model, d_ex, d_pi), d_pi, r, p.expand(b, K))
            grads = torch.autograd.grad(lnl.sum(), [d_bl, d_ex, d_pi])
            out = [lnl.detach().cpu()] + [g.cpu() for g in grads]
            return sum(o.numel() * o.element_size() for o in out)

        for _ in range(2):
            e2e_step()
        torch.cuda.synchronize()
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            d2h = e2e_step()
        torch.cuda.synchronize()
        _, e2e_value = replica_throughput(time.perf_counter() - t0, b * args.steps, world, dev)
        e2e = {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h}
        del lik
        torch.cuda.empty_cache()
        if world == 1:
            e2e["plugin"] = plugin_e2e(args, wl, dev, args.steps)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu, (ref_lnl, ref_grads, _) = cpu_baseline(wl, args.ref_chunk_patterns)
        # the same evaluation through the GPU paths: sample 0 of the FP64 drop-in and of the timed precision
        cpu["check"] = {"vs": "the reference path's sample 0 (whole alignment, FP64, CPU)"}
        for name, res in (("fp64_dropin", want), (args.precision, got)):
            if res is not None:
                cpu["check"][name] = reference_error(res, ref_lnl, ref_grads, 2 * T - 3)

    if rank == 0:
        lat = sorted(per_step)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": args.precision,
            "data": f"synthetic (seeded Yule tree, alignment simulated under the model: {wl.data_type})",
            "config": bench_config(args, wl, N, int(sum(ca.weights)), slab),
            "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                           "what": "one batched lnL+gradient call (all samples)"},
            "fp64_dropin": fp64,
            "accuracy": accuracy,
            "speedup_vs_fp64": (value / world / fp64["value"]) if fp64 else None,
            "lnl_only": lnl_only,
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches,
            "clocks": clocks.summary(),
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
