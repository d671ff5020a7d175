"""GB300 tree-likelihood engine and torchtree plug-in.

Core (no torchtree needed): ``LikelihoodEngine`` (C-ABI plan handle),
``PhyloLikelihood`` (standalone batched lnL + gradient), the drop-in
``functional`` counterparts of torchtree's ``calculate_treelikelihood*``,
and host utilities (``tree``, ``patterns``, ``datatype``, ``substitution``,
``site_models``, ``synthetic``).

With torchtree installed, ``torchtree_gb300.TreeLikelihoodModel`` is the
JSON-configurable plug-in class, ``torchtree_gb300.GammaSiteModel`` a
discretised Gamma site model for it, and ``__plugin__`` names the CLI plug-in.
"""
from __future__ import annotations

__version__ = "0.1.0"
__plugin__ = "plugin.GB300"

from . import datatype, patterns, site_models, substitution, synthetic, tree  # noqa: F401


def __getattr__(name):
    if name in ("TreeLikelihoodModel", "GammaSiteModel"):
        from . import model

        return getattr(model, name)
    if name in ("LikelihoodEngine",):
        from .engine import LikelihoodEngine

        return LikelihoodEngine
    if name in ("PhyloLikelihood",):
        from .likelihood import PhyloLikelihood

        return PhyloLikelihood
    if name == "functional":
        import importlib

        return importlib.import_module(".functional", __name__)
    raise AttributeError(name)
