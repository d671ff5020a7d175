"""Standalone tree likelihood (no torchtree objects needed).

``PhyloLikelihood`` holds one topology and one compressed alignment
resident on the device and evaluates lnL for a batch of parameter samples,
differentiable with respect to every input.  Its glue follows
``TreeLikelihoodModel._call`` (torchtree/evolution/tree_likelihood.py:313-356):
an unrooted tree's ``2T-3`` branch lengths get a trailing zero for node 2T-3,
a clock multiplies time lengths by per-branch rates, and P(t) uses
``branch_length * category_rate``.

The sticky rescaling switch of the reference (tree_likelihood.py:378-388)
is kept for the FP64 drop-in: evaluations run unscaled until one returns
-inf, then rescale from then on.  FP32 always rescales.
"""
from __future__ import annotations

import numpy as np
import torch

from .autograd import EigenLikelihood, GeneralRateMatrixLikelihood, MatrixLikelihood, RateMatrixLikelihood
from .engine import LikelihoodEngine
from .patterns import CompressedAlignment
from .substitution import normalise
from .tree import Topology


class PhyloLikelihood:
    def __init__(self, topology: Topology, alignment: CompressedAlignment, state_count: int,
                 category_count: int, batch: int = 1, precision: str = "f32", device=None):
        self.topology = topology
        self.alignment = alignment
        self.state_count = state_count
        self.category_count = category_count
        self.batch = batch
        self.precision = precision
        self.engine = LikelihoodEngine(topology.postorder, topology.tip_count, state_count,
                                       category_count, alignment.codes, alignment.table,
                                       alignment.weights, batch=batch, precision=precision,
                                       device=device)
        self.device = self.engine.device
        self.rescale = precision == "f32"

    def node_branch_lengths(self, branch_lengths: torch.Tensor, clock_rates=None) -> torch.Tensor:
        """Per-node lengths ``[b, 2T-2]`` (tree_likelihood.py:323-344)."""
        if clock_rates is None:
            zero = torch.zeros(branch_lengths.shape[:-1] + (1,), dtype=branch_lengths.dtype,
                               device=branch_lengths.device)
            return torch.cat((branch_lengths, zero), -1)
        return clock_rates * branch_lengths

    def __call__(self, branch_lengths, q_unnorm, frequencies, rates, props, clock_rates=None):
        """lnL ``[b]``.

        ``branch_lengths [b, 2T-3]`` (unrooted) or ``[b, 2T-2]`` with
        ``clock_rates``; ``q_unnorm [b,S,S]`` reversible rate matrix;
        ``frequencies [b,S]``; ``rates``/``props`` ``[b,K]``.
        """
        bls = self.node_branch_lengths(branch_lengths, clock_rates)
        return self.evaluate_rate_matrix(normalise(q_unnorm, frequencies), frequencies, bls, rates, props,
                                         frequencies)

    def evaluate_rate_matrix(self, q, pi_q, bls, rates, props, frequencies):
        """lnL from the normalised rate matrix; gradients reach ``q`` as dlnL/dQ."""
        if self.rescale:
            return RateMatrixLikelihood.apply(q, pi_q, bls, rates, props, frequencies, self.engine, True)
        lnl = RateMatrixLikelihood.apply(q, pi_q, bls, rates, props, frequencies, self.engine, False)
        if torch.isinf(lnl).any():
            self.rescale = True
            lnl = RateMatrixLikelihood.apply(q, pi_q, bls, rates, props, frequencies, self.engine, True)
        return lnl

    def evaluate_eigen(self, lam, u, w, bls, rates, props, frequencies):
        if self.rescale:
            return EigenLikelihood.apply(lam, u, w, bls, rates, props, frequencies, self.engine, True)
        lnl = EigenLikelihood.apply(lam, u, w, bls, rates, props, frequencies, self.engine, False)
        if torch.isinf(lnl).any():
            self.rescale = True
            lnl = EigenLikelihood.apply(lam, u, w, bls, rates, props, frequencies, self.engine, True)
        return lnl

    def evaluate_general(self, q, bls, rates, props, frequencies):
        """lnL from a normalised rate matrix that need not be reversible
        (``q [b,S,S]``): P = exp(Q t r) on the device by the scaling-and-squaring
        Pade kernel; gradients reach ``q``, ``bls`` and ``rates`` through the
        Frechet derivative of the exponential (S <= 32 for gradients)."""
        def run(rescale):
            return GeneralRateMatrixLikelihood.apply(q, bls, rates, props, frequencies, self.engine, rescale)

        if self.rescale:
            return run(True)
        lnl = run(False)
        if torch.isinf(lnl).any():
            self.rescale = True
            lnl = run(True)
        return lnl

    def evaluate_matrices(self, mats, props, frequencies):
        if self.rescale:
            return MatrixLikelihood.apply(mats, props, frequencies, self.engine, True)
        lnl = MatrixLikelihood.apply(mats, props, frequencies, self.engine, False)
        if torch.isinf(lnl).any():
            self.rescale = True
            lnl = MatrixLikelihood.apply(mats, props, frequencies, self.engine, True)
        return lnl

    def site_log_likelihoods(self, lam, u, w, bls, rates, props, frequencies) -> torch.Tensor:
        """Per-pattern log site likelihoods ``[b, N]`` (no gradient)."""
        self.engine.set_eigen(lam, u, w, bls, rates)
        _, site = self.engine.log_likelihood(props, frequencies, rescale=True, site=True)
        return site


def batch_inputs(workload, device, dtype=torch.float64):
    """Torch inputs of a ``synthetic.DnaWorkload``: (bl, exch, pi, shape)."""
    t = lambda a: torch.as_tensor(np.asarray(a), dtype=dtype, device=device)  # noqa: E731
    return t(workload.branch_lengths), t(workload.exch), t(workload.pi), t(workload.shape)
