"""Timed CPU baseline: the oracle's restatement of the reference path.

TEST/BENCH INFRASTRUCTURE ONLY (used by ``bench.py``'s CPU-baseline leg and
its ``--impl reference`` arm).  One evaluation = FP64 lnL of one sample with
rescaling (torchtree/evolution/tree_likelihood.py:186-221) plus the autograd
gradient with respect to branch lengths, exchangeabilities and frequencies,
exactly the torch ops the reference runs on the CPU.  Work is bounded by
evaluating a prefix of the pattern columns; rescaling is per pattern, so the
cost of the full workload is the prefix cost times N / n_patterns.
"""
from __future__ import annotations

import os
import time

import numpy as np
import torch

from . import likelihood as OL


def prepare(topology_postorder, codes, table, weights, branch_lengths, exch, pi, category_rates,
            n_patterns: int, model: str = "gtr"):
    n = min(n_patterns, codes.shape[1])
    tips = [torch.tensor(np.ascontiguousarray(table[codes[t, :n]].T)) for t in range(codes.shape[0])]
    return dict(post=[list(map(int, x)) for x in topology_postorder], tips=tips,
                weights=torch.tensor(np.asarray(weights[:n], dtype=np.float64)),
                bl=torch.tensor(branch_lengths), exch=torch.tensor(exch), pi=torch.tensor(pi),
                rates=torch.tensor(category_rates), n=n, model=model)


def _rate_matrix(model, exch, pi):
    """GTR / HKY (6 exchangeabilities), general symmetric, MG94 ((kappa, omega), alpha = 1)."""
    if model in ("gtr", "hky"):
        return OL.q_gtr(exch, pi)
    if model == "general":
        return OL.q_general_symmetric(exch, pi, pi.shape[-1])
    if model == "mg94":
        return OL.q_mg94(torch.ones_like(exch[..., :1]), exch[..., 1:2], exch[..., :1], pi)
    raise ValueError(model)


def one_evaluation(d) -> float:
    bl = d["bl"].clone().requires_grad_()
    exch = d["exch"].clone().requires_grad_()
    pi = d["pi"].clone().requires_grad_()
    k = d["rates"].shape[-1]
    props = torch.full((k, 1, 1), 1.0 / k, dtype=torch.float64)
    mats = OL.p_t_symmetric(_rate_matrix(d.get("model", "gtr"), exch, pi), pi,
                            OL.model_branch_lengths(bl).unsqueeze(-1) * d["rates"].unsqueeze(-2))
    parts = list(d["tips"]) + [None] * (len(d["tips"]) - 1)
    lnl = OL.treelikelihood_discrete_rescaled(parts, d["weights"], d["post"], mats, pi.unsqueeze(-2), props)
    lnl.sum().backward()
    return float(lnl.detach().sum())


def time_evaluations(d, repeats: int = 3, warmup: int = 1, threads: int | None = None):
    """Median seconds per prefix evaluation and the thread count used."""
    threads = threads or os.cpu_count() or 1
    torch.set_num_threads(threads)
    for _ in range(warmup):
        one_evaluation(d)
    times = []
    for _ in range(repeats):
        t0 = time.perf_counter()
        one_evaluation(d)
        times.append(time.perf_counter() - t0)
    return float(np.median(times)), threads, times
