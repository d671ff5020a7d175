"""Discretised rate-heterogeneity models (host side, differentiable).

``weibull_rates`` follows torchtree's ``WeibullSiteModel``
(torchtree/evolution/site_model.py:173-195, 237-247).  ``gamma_rates`` is
the discretised Gamma(shape, rate=shape) model, which torchtree 1.0.2 does
not ship: it uses the same (2i+1)/(2K) quantiles and mean-one
normalisation.  The quantiles and their analytic shape derivative come from
the engine (``tt_gamma_quantiles``: on the device for CUDA tensors, so no
host round trip enters a step; the same code on the host for CPU tensors);
the tests check them against scipy's ``gammaincinv`` and finite differences.
"""
from __future__ import annotations

import torch


def _quantiles(k: int, dtype, device):
    return (2.0 * torch.arange(k, dtype=dtype, device=device) + 1.0) / (2.0 * k)


def _finish(rates, categories, invariant, mu):
    k = categories
    if invariant is not None:
        probs = torch.cat((invariant, ((1.0 - invariant) / k).expand(invariant.shape[:-1] + (k,))), -1)
        rates = torch.cat((torch.zeros_like(invariant), rates.expand(invariant.shape[:-1] + (k,))), -1)
    else:
        probs = torch.full(rates.shape[-1:], 1.0 / k, dtype=rates.dtype, device=rates.device)
    rates = rates / (rates * probs).sum(-1, keepdim=True)
    if mu is not None:
        rates = rates * mu
    return rates, probs.expand(rates.shape)


def weibull_rates(shape: torch.Tensor, categories: int, invariant=None, mu=None):
    """``shape [...,1]`` -> ``(rates [...,K'], probabilities [...,K'])``."""
    q = _quantiles(categories, shape.dtype, shape.device)
    rates = torch.pow(-torch.log(1.0 - q), 1.0 / shape)
    return _finish(rates, categories, invariant, mu)


class _GammaQuantile(torch.autograd.Function):
    """x(alpha) / alpha, x the Gamma(alpha, 1) quantile at each of the K
    quantile levels (2k+1)/(2K), with the analytic shape derivative.  Both
    come from the engine (``tt_gamma_quantiles`` on the device,
    ``tt_gamma_quantiles_host`` for CPU tensors): Halley's method on the
    regularised incomplete gamma series, dx/dalpha by differentiating the
    series term by term.  ``alpha [..., 1]`` -> ``[..., K]``."""

    @staticmethod
    def forward(ctx, alpha, categories):
        from . import _native

        lib = _native.load()
        a = alpha.detach().to(torch.float64).reshape(-1).contiguous()
        b = a.shape[0]
        x = torch.empty(b, categories, dtype=torch.float64, device=alpha.device)
        dx = torch.empty_like(x)
        if alpha.is_cuda:
            with torch.cuda.device(alpha.device):
                stream = torch.cuda.current_stream(alpha.device).cuda_stream
                _native.check(lib.tt_gamma_quantiles(b, categories, _native.ptr(a), _native.ptr(x), _native.ptr(dx),
                                                     _native.ptr_value(stream)))
        else:
            _native.check(lib.tt_gamma_quantiles_host(b, categories, _native.ptr(a), _native.ptr(x),
                                                      _native.ptr(dx)))
        a1 = a.unsqueeze(-1)
        shape = alpha.shape[:-1] + (categories,)
        drda = (dx / a1 - x / (a1 * a1)).reshape(shape).to(alpha.dtype)
        ctx.save_for_backward(drda)
        return (x / a1).reshape(shape).to(alpha.dtype)

    @staticmethod
    def backward(ctx, grad):
        (drda,) = ctx.saved_tensors
        return (grad * drda).sum(-1, keepdim=True), None


def gamma_rates(shape: torch.Tensor, categories: int, invariant=None, mu=None):
    """Discretised Gamma rates; ``shape [...,1]`` (not in the reference)."""
    rates = _GammaQuantile.apply(shape, categories)
    return _finish(rates, categories, invariant, mu)


def invariant_rates(invariant: torch.Tensor, mu=None):
    """Proportion-invariant model without rate heterogeneity, torchtree's
    InvariantSiteModel (site_model.py:77-110): probabilities ``[p, 1-p]``,
    rates ``[0, 1/(1-p)]`` (mean rate 1), times ``mu`` when given;
    ``invariant [...,1]``."""
    ones = torch.ones(invariant.shape[:-1] + (1,), dtype=invariant.dtype, device=invariant.device)
    return _finish(ones, 1, invariant, mu)


def constant_rates(dtype=torch.float64, device=None):
    one = torch.ones(1, dtype=dtype, device=device)
    return one, one.clone()
