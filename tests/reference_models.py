"""Helpers for the tests that run torchtree itself.

torchtree comes from ``TORCHTREE_REFERENCE`` (a source tree) or, failing
that, from the unmodified copy installed in ``baseline/_ref``
(``oracle/reference.py`` does the search; the installed copy has no
``data/``).  Tests that need it are skipped where neither is present.
torchtree imports dendropy at module load; ``oracle/_stub/dendropy.py``
stands in for it (trees are never parsed through dendropy: post-order
triples come from this package's Newick parser and are handed to
``fixed_tree_class()``).
"""
from __future__ import annotations

from pathlib import Path

import numpy as np
import torch

from oracle import reference as _reference

ROOT = Path(__file__).resolve().parents[1]
DATA = _reference.data_dir() or ROOT / "tests" / "_no_reference_data"


def import_torchtree() -> bool:
    """Put torchtree and the dendropy stub on the path; True when it imports."""
    return _reference.import_torchtree() is not None


fixed_tree_class = _reference.fixed_tree_class


def reference_objects(case, wl, b):
    """torchtree objects of one case over a synthetic DNA workload: (tree, site
    pattern, substitution model, site model, clock, tip_states, leaf tensors).

    ``case`` names the model: ``gtr_weibull``, ``jc69_constant``,
    ``hky_weibull_clock`` (rooted time lengths times a strict clock) or
    ``gtr_weibull_tipstates``; ``b`` samples."""
    from torchtree import Parameter
    from torchtree.evolution.alignment import Alignment, Sequence
    from torchtree.evolution.branch_model import StrictClockModel
    from torchtree.evolution.datatype import NucleotideDataType
    from torchtree.evolution.site_model import ConstantSiteModel, WeibullSiteModel
    from torchtree.evolution.site_pattern import SitePattern
    from torchtree.evolution.substitution_model import GTR, HKY, JC69
    from torchtree.evolution.taxa import Taxa, Taxon

    names = wl.topology.tip_names
    taxa = Taxa(None, [Taxon(n, {}) for n in names])
    aln = Alignment(None, [Sequence(n, s) for n, s in zip(names, wl.sequences)], taxa, NucleotideDataType(None))
    sp = SitePattern(None, aln)
    T = wl.topology.tip_count
    leaf = lambda a: torch.tensor(np.asarray(a), dtype=torch.float64, requires_grad=True)  # noqa: E731
    bl = torch.tensor(wl.branch_lengths[:b])
    clock = None
    if case == "hky_weibull_clock":  # rooted time lengths (2T-2) times a strict clock
        bl = leaf(torch.cat((bl, torch.full((b, 1), 0.02)), -1).numpy() * 10.0)
        rate = leaf(np.full((b, 1), 0.1))
        tree = fixed_tree_class()(wl.topology.postorder, names, Parameter(None, bl))
        clock = StrictClockModel(None, Parameter(None, rate), tree)
        leaves = [bl, rate]
    else:
        bl = leaf(bl.numpy())
        tree = fixed_tree_class()(wl.topology.postorder, names, Parameter(None, bl))
        leaves = [bl]
    pi_t = leaf(wl.pi[:b])
    pi = Parameter(None, pi_t)
    if case.startswith("gtr"):
        ex = leaf(wl.exch[:b])
        subst = GTR(None, Parameter(None, ex), pi)
        leaves += [ex, pi_t]
    elif case.startswith("hky"):
        kappa = leaf(wl.exch[:b, 1:2])
        subst = HKY(None, Parameter(None, kappa), pi)
        leaves += [kappa, pi_t]
    else:
        subst = JC69(None)
    if "weibull" in case:
        shape = leaf(wl.shape[:b])
        site = WeibullSiteModel(None, Parameter(None, shape), 4)
        leaves.append(shape)
    else:
        site = ConstantSiteModel(None)
    assert T == len(names)
    return tree, sp, subst, site, clock, case.endswith("tipstates"), leaves


def wide_reference_objects(kind, wl):
    """torchtree objects of a 20-state (``GeneralSymmetricSubstitutionModel``,
    190 free rates) or 61-state (``MG94`` with alpha = 1) workload with a
    Weibull site model: (tree, site pattern, substitution model, site model,
    leaf tensors)."""
    from torchtree import Parameter
    from torchtree.evolution.alignment import Alignment, Sequence
    from torchtree.evolution.datatype import AminoAcidDataType, CodonDataType
    from torchtree.evolution.site_model import WeibullSiteModel
    from torchtree.evolution.site_pattern import SitePattern
    from torchtree.evolution.substitution_model import MG94
    from torchtree.evolution.substitution_model.general import GeneralSymmetricSubstitutionModel
    from torchtree.evolution.taxa import Taxa, Taxon

    names = wl.topology.tip_names
    leaf = lambda a: torch.tensor(np.asarray(a, dtype=np.float64), requires_grad=True)  # noqa: E731
    bl, pi, shape, ex = leaf(wl.branch_lengths), leaf(wl.pi), leaf(wl.shape), leaf(wl.exch)
    if kind == "protein":
        dtype = AminoAcidDataType(None)
        subst = GeneralSymmetricSubstitutionModel(None, dtype, Parameter(None, torch.arange(190)),
                                                  Parameter(None, ex), Parameter(None, pi))
    else:
        dtype = CodonDataType(None, "Universal")
        subst = MG94(None, dtype, Parameter(None, torch.ones_like(ex[..., :1])), Parameter(None, ex[..., 1:2]),
                     Parameter(None, ex[..., 0:1]), Parameter(None, pi))
    taxa = Taxa(None, [Taxon(n, {}) for n in names])
    aln = Alignment(None, [Sequence(n, s) for n, s in zip(names, wl.sequences)], taxa, dtype)
    tree = fixed_tree_class()(wl.topology.postorder, names, Parameter(None, bl))
    site = WeibullSiteModel(None, Parameter(None, shape), 4)
    return tree, SitePattern(None, aln), subst, site, [bl, ex, pi, shape]
