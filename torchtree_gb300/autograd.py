"""``torch.autograd.Function`` wrappers around a ``LikelihoodEngine``.

Forward runs the transition-matrix kernel and the post-order kernel; the
backward runs the pre-order adjoint kernel, reduces dlnL/dP per branch and
(in the eigen form) chains it through ``P = U diag(exp(lambda t r)) W``.
Torch autograd then carries the result through the small host-side graph
(eigh, rate matrix, site model, clock), as the reference's autograd does
(torchtree/evolution/tree_likelihood.py:313-356 is differentiated end to
end there).
"""
from __future__ import annotations

import torch

from .substitution import device_eigen, eigen_of_normalised


def _scale(g: torch.Tensor, x: torch.Tensor, like: torch.Tensor) -> torch.Tensor:
    shape = g.shape + (1,) * (x.dim() - 1)
    return (x * g.reshape(shape)).to(dtype=like.dtype, device=like.device)


class EigenLikelihood(torch.autograd.Function):
    """lnL ``[b]`` from ``(lam, U, W, branch_lengths, rates, props, freqs)``."""

    @staticmethod
    def forward(ctx, lam, u, w, bls, rates, props, freqs, engine, rescale):
        engine.set_eigen(lam, u, w, bls, rates)
        keep = any(ctx.needs_input_grad[:7])
        lnl = engine.log_likelihood(props, freqs, rescale=rescale, keep_partials=keep)
        ctx.engine = engine
        ctx.token = engine.token
        ctx.rescale = rescale
        ctx.save_for_backward(lam, u, w, bls, rates, props, freqs)
        return lnl.to(lam.dtype)

    @staticmethod
    def backward(ctx, g):
        lam, u, w, bls, rates, props, freqs = ctx.saved_tensors
        eng = ctx.engine
        if eng.token != ctx.token:  # a later forward overwrote the stored partials
            eng.set_eigen(lam, u, w, bls, rates)
            eng.log_likelihood(props, freqs, rescale=ctx.rescale, keep_partials=True)
        _, dpi, dc = eng.gradient(props, freqs)
        dlam, du, dw, dt, dr = eng.eigen_gradient(lam, u, w, bls, rates)
        g = g.to(torch.float64)
        return (_scale(g, dlam, lam), _scale(g, du, u), _scale(g, dw, w), _scale(g, dt, bls),
                _scale(g, dr, rates), _scale(g, dc, props), _scale(g, dpi, freqs), None, None)


class RateMatrixLikelihood(torch.autograd.Function):
    """lnL ``[b]`` from the normalised rate matrix ``q [b,S,S]`` (stationary
    distribution ``pi_q``), node branch lengths, category rates/weights and
    root frequencies.  The eigen system is formed here without autograd (on
    the device, by the engine's eigensolver, for CUDA tensors); the
    backward returns dlnL/dQ from the derivative of the matrix exponential in
    the eigenbasis (``tt_rate_matrix_gradient``), so no eigenvector
    derivative enters the chain to the rate-matrix parameters."""

    @staticmethod
    def forward(ctx, q, pi_q, bls, rates, props, freqs, engine, rescale):
        if q.is_cuda:
            lam, u, w = device_eigen(q, pi_q)
        else:
            lam, u, w = eigen_of_normalised(q.detach(), pi_q.detach())
        lam, u, w = (t.to(q.device).contiguous() for t in (lam, u, w))
        engine.set_eigen(lam, u, w, bls, rates)
        keep = any(ctx.needs_input_grad[:6])
        lnl = engine.log_likelihood(props, freqs, rescale=rescale, keep_partials=keep)
        ctx.engine = engine
        ctx.token = engine.token
        ctx.rescale = rescale
        ctx.q_like = q.new_empty(0)
        ctx.save_for_backward(lam, u, w, bls, rates, props, freqs)
        return lnl.to(q.dtype)

    @staticmethod
    def backward(ctx, g):
        lam, u, w, bls, rates, props, freqs = ctx.saved_tensors
        eng = ctx.engine
        if eng.token != ctx.token:
            eng.set_eigen(lam, u, w, bls, rates)
            eng.log_likelihood(props, freqs, rescale=ctx.rescale, keep_partials=True)
        _, dpi, dc = eng.gradient(props, freqs)
        dq, dt, dr = eng.rate_matrix_gradient(lam, u, w, bls, rates)
        g = g.to(torch.float64)
        return (_scale(g, dq, ctx.q_like), None, _scale(g, dt, bls), _scale(g, dr, rates),
                _scale(g, dc, props), _scale(g, dpi, freqs), None, None)


class MatrixLikelihood(torch.autograd.Function):
    """lnL ``[b]`` from transition matrices ``[b,B,K,S,S]``, ``props``, ``freqs``."""

    @staticmethod
    def forward(ctx, mats, props, freqs, engine, rescale):
        engine.set_matrices(mats)
        keep = any(ctx.needs_input_grad[:3])
        lnl = engine.log_likelihood(props, freqs, rescale=rescale, keep_partials=keep)
        ctx.engine = engine
        ctx.token = engine.token
        ctx.rescale = rescale
        ctx.save_for_backward(mats, props, freqs)
        return lnl.to(mats.dtype)

    @staticmethod
    def backward(ctx, g):
        mats, props, freqs = ctx.saved_tensors
        eng = ctx.engine
        if eng.token != ctx.token:
            eng.set_matrices(mats)
            eng.log_likelihood(props, freqs, rescale=ctx.rescale, keep_partials=True)
        dP, dpi, dc = eng.gradient(props, freqs, want_matrices=ctx.needs_input_grad[0])
        g = g.to(torch.float64)
        dmats = _scale(g, dP, mats) if dP is not None else None
        return dmats, _scale(g, dc, props), _scale(g, dpi, freqs), None, None


class GeneralRateMatrixLikelihood(torch.autograd.Function):
    """lnL ``[b]`` from a normalised rate matrix ``q [b,S,S]`` that need not
    be reversible (NonSymmetricSubstitutionModel.p_t, abstract.py:86-94):
    P = exp(Q t r) by the engine's scaling-and-squaring Pade kernel; the
    backward chains dlnL/dP through the Frechet derivative of the exponential
    to dlnL/dQ, branch lengths and category rates."""

    @staticmethod
    def forward(ctx, q, bls, rates, props, freqs, engine, rescale):
        mats = engine.expm_matrices(q.detach(), bls.detach(), rates.detach())
        engine.set_matrices(mats)
        keep = any(ctx.needs_input_grad[:5])
        lnl = engine.log_likelihood(props, freqs, rescale=rescale, keep_partials=keep)
        ctx.engine = engine
        ctx.token = engine.token
        ctx.rescale = rescale
        ctx.save_for_backward(q, bls, rates, props, freqs, mats)
        return lnl.to(q.dtype)

    @staticmethod
    def backward(ctx, g):
        q, bls, rates, props, freqs, mats = ctx.saved_tensors
        eng = ctx.engine
        if eng.token != ctx.token:
            eng.set_matrices(mats)
            eng.log_likelihood(props, freqs, rescale=ctx.rescale, keep_partials=True)
        dP, dpi, dc = eng.gradient(props, freqs, want_matrices=True)
        dq, dt, dr = eng.expm_gradient(q.detach(), bls.detach(), rates.detach(), dP)
        g = g.to(torch.float64)
        return (_scale(g, dq, q), _scale(g, dt, bls), _scale(g, dr, rates), _scale(g, dc, props),
                _scale(g, dpi, freqs), None, None)

