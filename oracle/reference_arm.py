"""Timed CPU run of the reference path on a benchmark workload.

TEST/BENCH INFRASTRUCTURE ONLY: ``bench.py``'s ``cpu_baseline`` leg and its
``--impl reference`` arm.  Nothing here loads the package's native library:
the alignment is compressed with numpy and every likelihood, matrix and
gradient comes from torch CPU ops.

What runs is torchtree's own code when it can be imported (its source tree
or the unmodified copy installed in ``baseline/_ref``, see
``oracle/reference.py``):

* ``GTR`` / ``HKY`` ``.p_t`` (evolution/substitution_model/abstract.py:57-76,
  nucleotide.py:238-264, 328-374) on ``cat(branch_lengths, 0) * rates`` as
  ``TreeLikelihoodModel._call`` forms it (evolution/tree_likelihood.py:313-346);
* ``calculate_treelikelihood_discrete_rescaled``
  (evolution/tree_likelihood.py:186-221);
* ``.backward()`` for the gradient with respect to the branch lengths, the
  exchangeabilities (or kappa), the frequencies and the category rates.

Otherwise the oracle's restatement of the same functions runs
(``oracle/likelihood.py``), and the result says ``kind = "port"``.

The reference has no discretised-Gamma site model; the Gamma category rates
are computed with scipy (the quantiles (2i+1)/(2K), mean one) and fed in as a
tensor, as the GPU path receives them.

A full evaluation of one sample is exact when done in pattern chunks:
rescaling is per pattern (tree_likelihood.py:209-211), so the chunks' lnL and
gradients add up to the whole alignment's.  ``evaluate_chunk`` does one chunk;
a step of the timed loop is one chunk, and consecutive steps walk the chunks
of the alignment in order.
"""
from __future__ import annotations

import os
import time

import numpy as np
import torch

from . import likelihood as OL
from . import patterns as OP
from . import reference


def _byte_matrix(sequences) -> np.ndarray:
    return np.stack([np.frombuffer(s.encode("ascii"), dtype=np.uint8) for s in sequences])


def compress(sequences, data_type: str):
    """Unique alignment columns in the reference's order with their counts.

    The reference sorts the per-taxon character tuples lexicographically
    (site_pattern.py:69-97); ``numpy.unique`` over columns of ASCII bytes
    sorts in the same order.  Codon columns are the per-taxon triplets
    (site_pattern.py:77-82).  Returns ``(tips [T] of float64 [S, N], weights [N])``
    with tip partials as ``compute_tips_partials(use_ambiguities=False)``
    gives them (site_pattern.py:100-124).
    """
    raw = _byte_matrix(sequences)
    T = raw.shape[0]
    if data_type == "codon":
        trip = raw.reshape(T, -1, 3).transpose(0, 2, 1).reshape(3 * T, -1)  # taxon-major triplet rows
        cols, weights = np.unique(trip, axis=1, return_counts=True)
        code = OP.CodonCode(OP.GENETIC_CODES["universal"])
        S = code.state_count
        c3 = cols.reshape(T, 3, -1)
        tips = []
        for t in range(T):
            rows = [code.partial("".join(map(chr, c3[t, :, n])), False) for n in range(cols.shape[1])]
            tips.append(np.ascontiguousarray(np.asarray(rows, dtype=np.float64).T))
        return tips, weights.astype(np.float64)
    cols, weights = np.unique(raw, axis=1, return_counts=True)
    partial = OP.nucleotide_partial if data_type == "nucleotide" else OP.amino_acid_partial
    lut = np.asarray([partial(chr(c), False) for c in range(128)], dtype=np.float64)  # [128, S]
    tips = [np.ascontiguousarray(lut[cols[t]].T) for t in range(T)]
    return tips, weights.astype(np.float64)


def category_rates(wl) -> np.ndarray:
    from scipy.special import gammaincinv

    k, shape = wl.categories, float(wl.shape[0, 0])
    q = (2.0 * np.arange(k) + 1.0) / (2.0 * k)
    if wl.site_model == "gamma":
        r = gammaincinv(shape, q) / shape
    else:  # Weibull (site_model.py:237-247)
        r = np.power(-np.log(1.0 - q), 1.0 / shape)
    return r / r.mean()


class ReferencePath:
    """The reference path's lnL + gradient of one sample, by pattern chunks."""

    def __init__(self, wl, chunk_patterns: int, threads: int | None = None):
        self.threads = threads or os.cpu_count() or 1
        torch.set_num_threads(self.threads)
        t0 = time.perf_counter()
        tips, weights = compress(wl.sequences, wl.data_type)
        self.compress_s = time.perf_counter() - t0
        self.wl = wl
        self.T = wl.topology.tip_count
        self.N = int(weights.shape[0])
        self.sites = int(weights.sum())
        self.post = [list(map(int, x)) for x in wl.topology.postorder]
        n = max(1, min(int(chunk_patterns), self.N))
        bounds = list(range(0, self.N, n)) + [self.N]
        self.chunks = [(bounds[i], bounds[i + 1]) for i in range(len(bounds) - 1)]
        self.tips = [[torch.from_numpy(t[:, a:b].copy()) for t in tips] for a, b in self.chunks]
        self.weights = [torch.from_numpy(weights[a:b].copy()) for a, b in self.chunks]
        self.rates = category_rates(wl)
        self.tt = reference.import_torchtree() if wl.model in ("gtr", "hky") else None
        self.kind = "reference" if self.tt is not None else "port"

    def describe(self) -> str:
        if self.kind == "reference":
            return (f"torchtree 1.0.2 ({reference.describe()}): {self.wl.model.upper()}.p_t + "
                    f"calculate_treelikelihood_discrete_rescaled + backward, FP64")
        return "oracle port of tree_likelihood.py:186-221 + p_t + autograd, FP64"

    def _matrices(self, s: int):
        """Leaf tensors and the transition matrices ``[B, K, S, S]`` of sample s."""
        wl = self.wl
        bl = torch.tensor(wl.branch_lengths[s], requires_grad=True)
        exch = torch.tensor(wl.exch[s], requires_grad=True)
        pi = torch.tensor(wl.pi[s], requires_grad=True)
        rates = torch.tensor(self.rates, requires_grad=True)
        bls = torch.cat([bl, torch.zeros(1, dtype=bl.dtype)])  # unrooted: node 2T-3 gets 0
        times = bls.reshape(-1, 1) * rates
        if self.kind == "reference":
            from torchtree import Parameter
            from torchtree.evolution.substitution_model import GTR, HKY

            if wl.model == "hky":
                kappa = exch[1:2]  # exchangeabilities (1, k, 1, 1, k, 1)
                model = HKY(None, Parameter(None, kappa), Parameter(None, pi))
            else:
                model = GTR(None, Parameter(None, exch), Parameter(None, pi))
            mats = model.p_t(times)
        else:
            if wl.model in ("gtr", "hky"):
                q = OL.q_gtr(exch, pi)
            elif wl.model == "general":
                q = OL.q_general_symmetric(exch, pi, pi.shape[-1])
            else:
                q = OL.q_mg94(torch.ones_like(exch[:1]), exch[1:2], exch[:1], pi)
            mats = OL.p_t_symmetric(q, pi, times)
        return (bl, exch, pi, rates), mats

    def evaluate_chunk(self, s: int, c: int):
        """lnL of chunk c of sample s and its gradients (branch lengths,
        exchangeabilities, frequencies, category rates)."""
        leaves, mats = self._matrices(s)
        pi = leaves[2]
        k = self.rates.shape[0]
        props = torch.full((k, 1, 1), 1.0 / k, dtype=torch.float64)
        parts = list(self.tips[c]) + [None] * (self.T - 1)
        if self.kind == "reference":
            from torchtree.evolution.tree_likelihood import calculate_treelikelihood_discrete_rescaled

            lnl = calculate_treelikelihood_discrete_rescaled(parts, self.weights[c], self.post, mats,
                                                            pi.reshape(1, -1), props)
        else:
            lnl = OL.treelikelihood_discrete_rescaled(parts, self.weights[c], self.post, mats,
                                                      pi.reshape(1, -1), props)
        lnl.sum().backward()
        return float(lnl.detach().sum()), [x.grad for x in leaves]

    def evaluate(self, s: int = 0):
        """Whole-alignment lnL and gradients of sample s (sum over chunks)."""
        total, grads = 0.0, None
        for c in range(len(self.chunks)):
            v, g = self.evaluate_chunk(s, c)
            total += v
            grads = g if grads is None else [a + b for a, b in zip(grads, g)]
        return total, grads
