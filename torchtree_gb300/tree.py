"""Tree topologies: Newick parsing, node indexing and branch-length vectors.

The indexing follows torchtree's ``setup_indexes``
(torchtree/evolution/tree_model.py:37-53): tips 0..T-1 in taxa order,
internal nodes T..2T-2 in post-order, root 2T-2, and the branch above node i
has index i.  ``postorder`` lists ``(node, left, right)`` triples like
``AbstractTreeModel.update_traversals`` (tree_model.py:187-195).

A node with more than two children (e.g. an unrooted Newick string with a
trifurcating root) is resolved by joining its first two children under a
new zero-length node until it is binary; a zero-length branch has P = I, so
the likelihood is unchanged.
"""
from __future__ import annotations

import re
from dataclasses import dataclass, field

import numpy as np


@dataclass
class NewickNode:
    label: str | None = None
    length: float | None = None
    children: list = field(default_factory=list)
    index: int = -1

    def is_leaf(self) -> bool:
        return not self.children


_TOKEN = re.compile(r"\s*(\(|\)|,|;|:|\[[^\]]*\]|'(?:[^']|'')*'|[^\s(),;:\[\]']+)")


def parse_newick(text: str) -> NewickNode:
    """Parse one Newick tree (labels, quoted labels, lengths, comments)."""
    tokens = [m.group(1) for m in _TOKEN.finditer(text.strip())]
    tokens = [t for t in tokens if not t.startswith("[")]
    pos = 0

    def peek():
        return tokens[pos] if pos < len(tokens) else None

    def take():
        nonlocal pos
        t = tokens[pos]
        pos += 1
        return t

    def node() -> NewickNode:
        nd = NewickNode()
        if peek() == "(":
            take()
            nd.children.append(node())
            while peek() == ",":
                take()
                nd.children.append(node())
            if take() != ")":
                raise ValueError("malformed Newick: expected ')'")
        t = peek()
        if t is not None and t not in "(),;:":
            lab = take()
            if lab.startswith("'"):
                lab = lab[1:-1].replace("''", "'")
            nd.label = lab
        if peek() == ":":
            take()
            nd.length = float(take())
        return nd

    root = node()
    if peek() == ";":
        take()
    if pos != len(tokens):
        raise ValueError("malformed Newick: trailing tokens")
    return root


def _resolve(nd: NewickNode) -> None:
    for c in nd.children:
        _resolve(c)
    while len(nd.children) > 2:
        a, b = nd.children[0], nd.children[1]
        joined = NewickNode(length=0.0, children=[a, b])
        nd.children = [joined] + nd.children[2:]
    if len(nd.children) == 1:
        raise ValueError("unary nodes are not supported")


def _postorder(nd: NewickNode):
    out = []
    stack = [(nd, False)]
    while stack:
        v, seen = stack.pop()
        if v.is_leaf() or seen:
            out.append(v)
        else:
            stack.append((v, True))
            for c in reversed(v.children):
                stack.append((c, False))
    return out


class Topology:
    """A rooted binary tree with torchtree's node indexing.

    ``postorder``: int32 array ``[T-1, 3]`` of (node, left, right).
    ``parent``: int array ``[2T-1]`` (-1 for the root).
    ``edge_lengths``: float64 ``[2T-2]`` lengths read from the Newick string
    (NaN when absent), indexed by child node.
    """

    def __init__(self, postorder, tip_names, edge_lengths=None):
        self.postorder = np.asarray(postorder, dtype=np.int32).reshape(-1, 3)
        self.tip_names = list(tip_names)
        self.tip_count = len(self.tip_names)
        T = self.tip_count
        if self.postorder.shape[0] != T - 1:
            raise ValueError("a binary tree with T tips has T-1 internal nodes")
        self.parent = np.full(2 * T - 1, -1, dtype=np.int64)
        for v, l, r in self.postorder:
            self.parent[l] = v
            self.parent[r] = v
        self.edge_lengths = (np.full(2 * T - 2, np.nan) if edge_lengths is None
                             else np.asarray(edge_lengths, dtype=np.float64))

    @property
    def root(self) -> int:
        return int(self.postorder[-1, 0])

    @property
    def branch_count(self) -> int:
        return 2 * self.tip_count - 2

    def postorder_list(self):
        """Triples as a list of lists, the reference's ``tree_model.postorder``."""
        return [list(map(int, t)) for t in self.postorder]

    def root_children(self):
        v, l, r = self.postorder[-1]
        return int(l), int(r)

    def unrooted_branch_lengths(self) -> np.ndarray:
        """The ``2T-3`` free lengths of the unrooted tree (tree_model.py:328-344).

        The two root edges are merged onto each root child; node 2T-3 (a root
        child) then gets the padded zero branch and is dropped here.
        """
        bl = self.edge_lengths.copy()
        c1, c2 = self.root_children()
        e1, e2 = bl[c1], bl[c2]
        bl[c1] += e2
        bl[c2] += e1
        return bl[:-1]

    @classmethod
    def from_newick(cls, text: str, taxa=None) -> "Topology":
        root = parse_newick(text)
        _resolve(root)
        nodes = _postorder(root)
        leaves = [v for v in nodes if v.is_leaf()]
        names = [v.label for v in leaves]
        if taxa is None:
            taxa = names
        taxa = list(taxa)
        if sorted(taxa) != sorted(names):
            raise ValueError("taxon names in the tree do not match the taxa list")
        where = {name: i for i, name in enumerate(taxa)}
        T = len(taxa)
        nxt = T
        for v in nodes:
            if v.is_leaf():
                v.index = where[v.label]
            else:
                v.index = nxt
                nxt += 1
        post = [(v.index, v.children[0].index, v.children[1].index) for v in nodes if not v.is_leaf()]
        lengths = np.full(2 * T - 2, np.nan)
        for v in nodes:
            if v is not root and v.length is not None:
                lengths[v.index] = v.length
        return cls(post, taxa, lengths)

    def to_newick(self, branch_lengths=None) -> str:
        bl = self.edge_lengths if branch_lengths is None else np.asarray(branch_lengths)
        kids = {int(v): (int(l), int(r)) for v, l, r in self.postorder}

        def rec(v):
            if v < self.tip_count:
                s = self.tip_names[v]
            else:
                l, r = kids[v]
                s = f"({rec(l)},{rec(r)})"
            if v != self.root and v < len(bl):
                s += f":{bl[v]!r}"
            return s

        return rec(self.root) + ";"


def node_heights_from_lengths(topo: Topology, tip_heights=None, min_length: float = 0.0) -> np.ndarray:
    """Heights of all nodes when tips sit at ``tip_heights`` (default 0): a
    parent sits at the highest child plus its branch, each branch counted as
    at least ``min_length`` (torchtree's heights_from_branch_lengths,
    tree_model.py:110-122, uses 1e-6)."""
    T = topo.tip_count
    h = np.zeros(2 * T - 1)
    if tip_heights is not None:
        h[:T] = tip_heights
    for v, l, r in topo.postorder:
        h[v] = max(h[l] + max(min_length, topo.edge_lengths[l]), h[r] + max(min_length, topo.edge_lengths[r]))
    return h
