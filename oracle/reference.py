"""Locating and importing the reference torchtree (pure Python, CPU).

TEST/BENCH INFRASTRUCTURE ONLY: used by ``tests/`` and by ``bench.py``'s CPU
legs, never by the package.

Two places are searched, in order:

* ``TORCHTREE_REFERENCE``: a torchtree source tree (the directory holding
  ``torchtree/`` and, for the known-answer tests, ``data/``);
* ``baseline/_ref`` beside this repository: an unmodified copy of torchtree
  1.0.2 installed there with ``pip install --no-deps --target baseline/_ref``
  (git-ignored; it carries the package only, no ``data/``).

torchtree imports dendropy at module load; ``oracle/_stub`` provides the three
names it needs.
"""
from __future__ import annotations

import os
import sys
from pathlib import Path

REPO = Path(__file__).resolve().parents[1]
STUB = REPO / "oracle" / "_stub"
INSTALLED = REPO / "baseline" / "_ref"


def source_root() -> Path | None:
    """The torchtree source tree named by TORCHTREE_REFERENCE, if it exists."""
    env = os.environ.get("TORCHTREE_REFERENCE")
    if env and (Path(env) / "torchtree").is_dir():
        return Path(env)
    return None


def data_dir() -> Path | None:
    """The reference's ``data/`` folder (only a source tree has one)."""
    root = source_root()
    if root is not None and (root / "data").is_dir():
        return root / "data"
    return None


def torchtree_root() -> Path | None:
    root = source_root()
    if root is not None:
        return root
    if (INSTALLED / "torchtree").is_dir():
        return INSTALLED
    return None


def import_torchtree():
    """Import torchtree from its source tree or the installed copy; the module, or None."""
    root = torchtree_root()
    if root is None:
        return None
    for path in (str(STUB), str(root)):
        if path not in sys.path:
            sys.path.insert(0, path)
    try:
        import torchtree
    except ImportError:
        return None
    return torchtree


def describe() -> str:
    root = torchtree_root()
    if root is None:
        return "absent"
    return "source tree (TORCHTREE_REFERENCE)" if root == source_root() else "installed copy (baseline/_ref)"


def fixed_tree_class():
    """A minimal torchtree ``TreeModel``: fixed post-order, branch lengths from a Parameter."""
    from torchtree.evolution.tree_model import TreeModel

    class FixedTree(TreeModel):
        def __init__(self, post, names, bl):
            super().__init__(None)
            self._post = [list(map(int, t)) for t in post]
            self._names = list(names)
            self._bl = bl
            self.taxa_count = len(names)

        def branch_lengths(self):
            return self._bl.tensor

        @property
        def postorder(self):
            return self._post

        @property
        def taxa(self):
            return self._names

        def write_newick(self, stream, **kwargs):
            stream.write("();")

        def _sample_shape(self):
            return self._bl.tensor.shape[:-1]

        def handle_model_changed(self, model, obj, index):
            pass

        def handle_parameter_changed(self, variable, index, event):
            self.fire_model_changed()

        @classmethod
        def from_json(cls, data, dic):
            raise NotImplementedError

    return FixedTree


class PatternSource:
    """Stands in for torchtree's ``SitePattern`` where its pure-Python
    compression would take minutes (a 1,000 x 100,000 alignment): it hands
    ``TreeLikelihoodModel`` the tip partials and weights of the numpy
    compression in ``oracle/reference_arm.py`` (same pattern order and
    values as ``compress_alignment(..., use_ambiguities=False)``,
    site_pattern.py:100-124)."""

    def __init__(self, tips, weights):
        import torch

        self._tips = [torch.from_numpy(t) for t in tips]
        self._weights = torch.from_numpy(weights)

    def compute_tips_partials(self, use_ambiguities=False):
        return list(self._tips), self._weights
