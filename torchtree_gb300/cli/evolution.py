"""Engine hook for ``torchtree-cli ... --engine torchtree_gb300``.

torchtree's CLI imports ``<engine>.cli.evolution`` and calls
``process_tree_likelihood(arg, json)`` on every generated likelihood
(torchtree/cli/evolution.py:700-711, 1739-1754).  The hook retargets the
likelihood object to the GPU class and records the chosen precision.
"""
from __future__ import annotations


def process_tree_likelihood(arg, data) -> None:
    if data.get("type") == "JointDistributionModel":
        for d in data.get("distributions", []):
            process_tree_likelihood(arg, d)
        return
    data["type"] = "torchtree_gb300.TreeLikelihoodModel"
    data["precision"] = getattr(arg, "gb300_precision", None) or "f64"
