"""torchtree plug-in model: ``TreeLikelihoodModel`` on the GB300 engine.

Importing this module needs torchtree.  The class subclasses torchtree's
``TreeLikelihoodModel`` (torchtree/evolution/tree_likelihood.py:281-450),
keeps its constructor, JSON keys (``tree_model``, ``site_model``,
``substitution_model``, ``site_pattern``, optional ``branch_model``,
``use_ambiguities``, ``use_tip_states``) and cached-call behaviour, adds an
optional ``"precision": "f64" | "f32"`` key, and replaces ``_call`` with the
GPU path.  A JSON configuration selects it with
``"type": "torchtree_gb300.TreeLikelihoodModel"``.

Reversible models that inherit torchtree's eigen-based ``p_t`` use the
eigen route (the transition-matrix kernel forms every P on the device);
non-reversible models that inherit its matrix-exponential ``p_t`` use the
device Pade kernel; any other substitution model (JC69's closed form) hands
its ``p_t`` matrices to the engine directly.
"""
from __future__ import annotations

import math

import torch
from torchtree.core.utils import process_object, process_object_with_key, register_class
from torchtree.evolution.branch_model import BranchModel
from torchtree.evolution.site_model import SiteModel, UnivariateDiscretizedSiteModel
from torchtree.evolution.site_pattern import SitePattern
from torchtree.evolution.substitution_model.abstract import (
    NonSymmetricSubstitutionModel,
    SubstitutionModel,
    SymmetricSubstitutionModel,
)
from torchtree.evolution.tree_likelihood import TreeLikelihoodModel as _ReferenceModel
from torchtree.evolution.tree_model import TreeModel

from . import patterns
from .autograd import GeneralRateMatrixLikelihood, MatrixLikelihood, RateMatrixLikelihood
from .engine import LikelihoodEngine
from .site_models import _GammaQuantile
from .substitution import normalise


def _uses_eigen_form(subst_model) -> bool:
    return (isinstance(subst_model, SymmetricSubstitutionModel)
            and type(subst_model).p_t is SymmetricSubstitutionModel.p_t)


def _uses_matrix_exp(subst_model) -> bool:
    """torchtree's non-reversible p_t: torch.matrix_exp of the normalised Q
    (abstract.py:86-94)."""
    return (isinstance(subst_model, NonSymmetricSubstitutionModel)
            and type(subst_model).p_t is NonSymmetricSubstitutionModel.p_t)


@register_class
class TreeLikelihoodModel(_ReferenceModel):
    def __init__(self, id_, site_pattern, tree_model, subst_model, site_model, clock_model=None,
                 use_ambiguities=False, use_tip_states=False, precision="f64"):
        super().__init__(id_, site_pattern, tree_model, subst_model, site_model, clock_model,
                         use_ambiguities, use_tip_states)
        if precision not in ("f64", "f32"):
            raise ValueError("precision must be 'f64' or 'f32'")
        self.precision = precision
        tip_count = len(tree_model.taxa)
        tips = [t.detach().cpu().numpy() for t in self.partials[:tip_count]]
        w = self.weights.detach().cpu().numpy()
        if use_tip_states:
            state_count = int(subst_model.frequencies.shape[-1])
            self._alignment = patterns.from_tip_states(tips, state_count, w)
        else:
            self._alignment = patterns.from_tip_partials(tips, w)
        self._engines = {}
        if precision == "f32":
            self.rescale = True

    def _engine(self, batch, state_count, category_count):
        key = (batch, state_count, category_count)
        eng = self._engines.get(key)
        if eng is None:
            post = [list(t) for t in self.tree_model.postorder]
            eng = LikelihoodEngine(post, len(self.tree_model.taxa), state_count, category_count,
                                   self._alignment.codes, self._alignment.table,
                                   self._alignment.weights, batch=batch, precision=self.precision)
            self._engines[key] = eng
        return eng

    def engine_inputs(self, device):
        """The engine's inputs for the current parameters, on ``device``, as
        ``(route, tensors, sample_shape, (b, S, K))``, mirroring the inputs
        that ``_call`` gathers (tree_likelihood.py:313-349):

        * route ``"rate_matrix"`` (reversible models with the eigen-form
          ``p_t``): ``(Q normalised, frequencies, node lengths, rates,
          probabilities, frequencies)``;
        * route ``"general_rate_matrix"`` (non-reversible models with the
          matrix-exponential ``p_t``, up to 32 states): ``(Q normalised, node
          lengths, rates, probabilities, frequencies)``;
        * route ``"matrices"`` (any other ``p_t``): ``(P [b, 2T-2, K, S, S],
          probabilities, frequencies)``.

        Node lengths are the unrooted lengths with the zero branch appended,
        or clock rates times time lengths; every tensor is flattened to
        ``b = prod(sample_shape)`` samples.
        """
        sample_shape = self.sample_shape
        b = math.prod(sample_shape)
        branch_lengths = self.tree_model.branch_lengths()
        rates = self.site_model.rates()
        probs = self.site_model.probabilities()
        K = rates.shape[-1]
        rates = rates.expand(sample_shape + (K,)) if rates.dim() == 1 else rates.reshape(sample_shape + (K,))
        probs = probs.expand(sample_shape + (K,))
        if self.clock_model is None:
            if branch_lengths.dim() == 1:
                branch_lengths = branch_lengths.expand(sample_shape + (-1,))
            zero = torch.zeros(sample_shape + (1,), dtype=branch_lengths.dtype, device=branch_lengths.device)
            bls = torch.cat((branch_lengths, zero), -1)
        else:
            if branch_lengths.dim() == 1:
                bls = self.clock_model.rates * branch_lengths.expand(sample_shape + (1, -1))
            else:
                bls = self.clock_model.rates * branch_lengths
        bls = bls.reshape(sample_shape + (-1,))
        freqs = self.subst_model.frequencies
        S = freqs.shape[-1]
        freqs = freqs.expand(sample_shape + (S,))

        def flat(x, *tail):
            return x.to(device).reshape((b,) + tail)

        if _uses_eigen_form(self.subst_model):
            q = self.subst_model.q()
            q = q.expand(sample_shape + (S, S)) if q.dim() == 2 else q.reshape(sample_shape + (S, S))
            qn = normalise(flat(q, S, S), flat(freqs, S))  # abstract.py:49-50
            tensors = (qn, flat(freqs, S), flat(bls, bls.shape[-1]), flat(rates, K), flat(probs, K), flat(freqs, S))
            return "rate_matrix", tensors, sample_shape, (b, S, K)
        if _uses_matrix_exp(self.subst_model) and S <= 32:
            q = self.subst_model.q()
            q = q.expand(sample_shape + (S, S)) if q.dim() == 2 else q.reshape(sample_shape + (S, S))
            qn = normalise(flat(q, S, S), flat(freqs, S))  # abstract.py:88-94
            tensors = (qn, flat(bls, bls.shape[-1]), flat(rates, K), flat(probs, K), flat(freqs, S))
            return "general_rate_matrix", tensors, sample_shape, (b, S, K)
        mats = self.subst_model.p_t(bls.reshape(sample_shape + (-1, 1)) * rates.unsqueeze(-2))
        tensors = (flat(mats, mats.shape[-4], K, S, S), flat(probs, K), flat(freqs, S))
        return "matrices", tensors, sample_shape, (b, S, K)

    def _call(self, *args, **kwargs) -> torch.Tensor:
        dev = torch.device("cuda", torch.cuda.current_device())  # raises without CUDA: no CPU fallback
        route, tensors, sample_shape, (b, S, K) = self.engine_inputs(dev)
        eng = self._engine(b, S, K)
        # rate-matrix routes: gradients reach Q through dlnL/dQ (no eigenvector derivatives)
        fn = {"rate_matrix": RateMatrixLikelihood, "general_rate_matrix": GeneralRateMatrixLikelihood,
              "matrices": MatrixLikelihood}[route]

        def run(rescale):
            return fn.apply(*tensors, eng, rescale)

        if self.rescale:
            lnl = run(True)
        else:
            lnl = run(False)
            if torch.isinf(lnl).any():  # sticky switch (tree_likelihood.py:378-388)
                self.rescale = True
                lnl = run(True)
        device = self.tree_model.branch_lengths().device
        return lnl.to(device).reshape(sample_shape + (1,))

    @classmethod
    def from_json(cls, data, dic):
        tree_model = process_object(data[TreeModel.tag], dic)
        site_model = process_object(data[SiteModel.tag], dic)
        subst_model = process_object(data[SubstitutionModel.tag], dic)
        site_pattern = process_object(data[SitePattern.tag], dic)
        clock_model = process_object(data[BranchModel.tag], dic) if BranchModel.tag in data else None
        return cls(data["id"], site_pattern, tree_model, subst_model, site_model, clock_model,
                   data.get("use_ambiguities", False), data.get("use_tip_states", False),
                   data.get("precision", "f64"))


@register_class
class GammaSiteModel(UnivariateDiscretizedSiteModel):
    """Discretised Gamma(shape, rate = shape) rate heterogeneity.

    torchtree 1.0.2 ships only constant, proportion-invariant and discretised
    Weibull models (site_model.py:37-256).  This one is built exactly like
    ``WeibullSiteModel`` (categories at the quantiles (2i+1)/(2K), rates
    divided by their mean, optional invariant proportion and ``mu``;
    site_model.py:173-195, 223-256) with the Gamma quantile in place of the
    Weibull one.  The quantiles and their analytic shape derivative come from
    the engine (``tt_gamma_quantiles``).  JSON:
    ``{"type": "torchtree_gb300.GammaSiteModel", "shape": ..., "categories": K,
    ["invariant": ...], ["mu": ...]}``.
    """

    @property
    def shape(self) -> torch.Tensor:
        return self._parameter.tensor

    def inverse_cdf(self, parameter, quantile, invariant):
        x = _GammaQuantile.apply(parameter, quantile.shape[-1])
        if invariant is not None:
            return torch.cat((torch.zeros_like(invariant), x), dim=-1)
        return x

    @classmethod
    def from_json(cls, data, dic):
        shape = process_object(data["shape"], dic)
        invariant = process_object_with_key("invariant", data, dic)
        mu = process_object_with_key("mu", data, dic)
        return cls(data["id"], shape, data["categories"], invariant, mu)

