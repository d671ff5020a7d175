"""Import-only stand-in for dendropy.

TEST/BENCH INFRASTRUCTURE ONLY.  torchtree imports three dendropy names at
module load (evolution/tree_model.py:9, evolution/io.py:6-9).  Nothing here
parses a tree through dendropy: post-order triples come from this package's
Newick parser or Yule generator and are handed to a minimal ``TreeModel``.
Empty classes are therefore enough to import the likelihood modules, for the
golden-vector generator, the tests that run torchtree, and the timed CPU
baseline of the reference path.
"""


class TaxonNamespace:  # noqa: D101
    pass


class Tree:  # noqa: D101
    pass


class DnaCharacterMatrix:  # noqa: D101
    pass
