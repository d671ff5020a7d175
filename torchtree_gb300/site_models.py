"""Discretised rate-heterogeneity models (host side, differentiable).

``weibull_rates`` follows torchtree's ``WeibullSiteModel``
(torchtree/evolution/site_model.py:173-195, 237-247).  ``gamma_rates`` is
the discretised Gamma(shape, rate=shape) model, which torchtree 1.0.2 does
not ship: it uses the same (2i+1)/(2K) quantiles and mean-one
normalisation, scipy's ``gammaincinv`` for the quantiles, and implicit
differentiation for the shape gradient (checked against central finite
differences in the tests).
"""
from __future__ import annotations

import numpy as np
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
    """x(alpha) / alpha with x = inverse regularised lower incomplete gamma."""

    @staticmethod
    def forward(ctx, alpha, q):
        from scipy.special import gammainc, gammaincinv, gammaln

        a = alpha.detach().cpu().double().numpy()
        qq = q.detach().cpu().double().numpy()
        x = gammaincinv(a, qq)
        h = 1e-6 * np.maximum(a, 1e-3)
        dpda = (gammainc(a + h, x) - gammainc(a - h, x)) / (2 * h)
        dpdx = np.exp((a - 1.0) * np.log(x) - x - gammaln(a))
        dxda = -dpda / dpdx
        drda = dxda / a - x / (a * a)
        ctx.save_for_backward(torch.as_tensor(drda, dtype=alpha.dtype, device=alpha.device))
        return torch.as_tensor(x / a, dtype=alpha.dtype, device=alpha.device)

    @staticmethod
    def backward(ctx, grad):
        (drda,) = ctx.saved_tensors
        return (grad * drda).sum(-1, keepdim=True), None


def gamma_rates(shape: torch.Tensor, categories: int, invariant=None, mu=None):
    """Discretised Gamma rates; ``shape [...,1]`` (not in the reference)."""
    q = _quantiles(categories, shape.dtype, shape.device)
    rates = _GammaQuantile.apply(shape, q)
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
