"""Helpers for the tests that import torchtree from its source tree.

The source location is TORCHTREE_REFERENCE, else the default below; tests
that need it are skipped where it is absent.  torchtree imports dendropy at
module load; ``tests/golden/_stub/dendropy.py`` stands in for it (trees are
never parsed through dendropy: post-order triples come from this package's
Newick parser and are handed to ``fixed_tree_class()``).
"""
from __future__ import annotations

import os
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
REFERENCE = Path(os.environ.get("TORCHTREE_REFERENCE", "/root/reference"))
DATA = REFERENCE / "data"


def import_torchtree() -> bool:
    """Put torchtree's source and the dendropy stub on the path; True when it imports."""
    if not (REFERENCE / "torchtree").is_dir():
        return False
    for path in (str(ROOT / "tests" / "golden" / "_stub"), str(REFERENCE)):
        if path not in sys.path:
            sys.path.insert(0, path)
    try:
        import torchtree  # noqa: F401
    except ImportError:
        return False
    return True


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
