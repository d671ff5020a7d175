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

from oracle import reference as _reference

ROOT = Path(__file__).resolve().parents[1]
DATA = _reference.data_dir() or ROOT / "tests" / "_no_reference_data"


def import_torchtree() -> bool:
    """Put torchtree and the dendropy stub on the path; True when it imports."""
    return _reference.import_torchtree() is not None


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
