"""Import-only stand-in for dendropy, used by make_golden.py.

torchtree imports three dendropy names at module load. The golden-vector
script never parses a tree through dendropy (it builds post-order triples
itself), so empty classes are enough to import the likelihood modules.
"""


class TaxonNamespace:  # noqa: D101
    pass


class Tree:  # noqa: D101
    pass


class DnaCharacterMatrix:  # noqa: D101
    pass
