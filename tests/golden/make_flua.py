"""Generate ``flua.json``: the input of torchtree's influenza A known answer.

Usage (from the repository root, in a container where the reference source
is available):

    python tests/golden/make_flua.py /path/to/torchtree-source

test/test_tree_likelihood.py:268-342 in the reference evaluates its bundled
``data/fluA.fa`` / ``data/fluA.tree`` (69 taxa, 987 sites) and asserts
lnL = -4618.2062529058.  The GPU machine has no reference source, so this script
records what that test needs, computed by the reference's own code: the taxon
names (which carry the sampling dates), the Newick tree, and the alignment
compressed by torchtree's ``compress_alignment`` (site_pattern.py:100-124):
the unique site columns as per-taxon character strings in the reference's
pattern order, with their integer weights.  ``tests/test_reference_kat.py``
reads the data from the source tree where it exists and from this file
elsewhere.
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent


def main(ref_root: str) -> None:
    sys.path.insert(0, str(REPO / "oracle" / "_stub"))
    sys.path.insert(0, ref_root)
    import torch

    torch.set_default_dtype(torch.float64)
    from torchtree.evolution.alignment import Alignment, Sequence
    from torchtree.evolution.datatype import NucleotideDataType
    from torchtree.evolution.site_pattern import compress
    from torchtree.evolution.taxa import Taxa, Taxon

    data = Path(ref_root) / "data"
    names, seqs = [], []
    for line in (data / "fluA.fa").read_text().splitlines():
        line = line.strip()
        if line.startswith(">"):
            names.append(line[1:].strip())
            seqs.append([])
        elif line:
            seqs[-1].append(line)
    seqs = ["".join(s) for s in seqs]
    taxa = Taxa(None, [Taxon(n, {}) for n in names])
    aln = Alignment(None, [Sequence(n, s) for n, s in zip(names, seqs)], taxa, NucleotideDataType(None))
    patterns, weights = compress(aln)  # site_pattern.py:69-97
    out = {"names": names, "newick": (data / "fluA.tree").read_text().strip(),
           "patterns": ["".join(patterns[n]) for n in names], "weights": [int(w) for w in weights],
           "site_count": len(seqs[0]), "lnl": -4618.2062529058}
    (HERE / "flua.json").write_text(json.dumps(out))


if __name__ == "__main__":
    main(sys.argv[1])
