"""Restatement of torchtree's data types and site-pattern compression.

TEST INFRASTRUCTURE ONLY (the checker of the package's compression; never
imported by the package), pinned by the golden fixtures generated from the
reference.

Pure Python, written for small alignments.  Follows
evolution/datatype.py:57-335 (state codes and tip partial vectors) and
evolution/site_pattern.py:69-151 (column compression).  The code tables are
built here from the IUPAC rules they encode rather than written out; the
golden fixtures generated from the reference pin every ASCII code.
"""
from __future__ import annotations

from collections import Counter

# ---------------------------------------------------------------- nucleotides
# Row order of the ambiguity table (datatype.py:78-97): A C G T U R Y M W S K B D H V N ? -
_NUC_ROWS = "ACGTURYMWSKBDHVN?-"
_NUC_SETS = {
    "A": "A", "C": "C", "G": "G", "T": "T", "U": "T", "R": "AG", "Y": "CT", "M": "AC",
    "W": "AT", "S": "CG", "K": "GT", "B": "CGT", "D": "AGT", "H": "ACT", "V": "ACG",
    "N": "ACGT", "?": "ACGT", "-": "ACGT",
}


def nucleotide_code(ch: str) -> int:
    """ASCII -> row of the ambiguity table (datatype.py:61-75, 102-103).

    IUPAC letters (either case) map to their row, with U sharing T's row 3;
    other letters and '?' map to row 16 ('?'); every other character maps to
    row 17 ('-').
    """
    o = ord(ch)
    if o >= 128:
        raise IndexError("character outside ASCII")
    up = ch.upper() if ch.isalpha() and o < 128 else ch
    if up == "U":
        return 3
    if up in _NUC_ROWS[:4] or up in _NUC_ROWS[5:16]:
        return _NUC_ROWS.index(up)
    if ch.isalpha() or ch == "?":
        return 16
    return 17


def nucleotide_partial(ch: str, use_ambiguities: bool = True):
    """Tip partial vector of one character (datatype.py:105-110)."""
    if not use_ambiguities and ch not in "ACGTUacgtu":
        return (1.0,) * 4
    row = _NUC_ROWS[nucleotide_code(ch)]
    allowed = _NUC_SETS[row]
    return tuple(1.0 if s in allowed else 0.0 for s in "ACGT")


# ---------------------------------------------------------------- amino acids
_AA = "ACDEFGHIKLMNPQRSTVWY"
_AA_ROWS = _AA + "BZX*?-"


def amino_acid_code(ch: str) -> int:
    """ASCII -> amino-acid row (datatype.py:122-136, 164-165).

    The 20 residues and B, Z, X (either case) map to their position in
    ``ACDEFGHIKLMNPQRSTVWYBZX*?-``; '*' -> 23; the letters J, O, U and '?'
    -> 24; every other character -> 25.
    """
    if ord(ch) >= 128:
        raise IndexError("character outside ASCII")
    up = ch.upper() if ch.isalpha() else ch
    if up in _AA_ROWS[:23]:
        return _AA_ROWS.index(up)
    if up == "*":
        return 23
    if ch.isalpha() or ch == "?":
        return 24
    return 25


def amino_acid_partial(ch: str, use_ambiguities: bool = True):
    """Tip partial vector (datatype.py:139-157, 167-175)."""
    if not use_ambiguities and ch not in _AA + _AA.lower():
        return (1.0,) * 20
    code = amino_acid_code(ch)
    if code < 20:
        return tuple(1.0 if i == code else 0.0 for i in range(20))
    if code == 20:  # B = D or N
        allowed = "DN"
    elif code == 21:  # Z = E or Q
        allowed = "EQ"
    else:
        return (1.0,) * 20
    return tuple(1.0 if a in allowed else 0.0 for a in _AA)


# ---------------------------------------------------------------- codons
GENETIC_CODES = {
    "universal": "KNKNTTTTRSRSIIMIQHQHPPPPRRRRLLLLEDEDAAAAGGGGVVVV*Y*YSSSS*CWCLFLF",
    "vertebrate mitochondrial": "KNKNTTTT*S*SMIMIQHQHPPPPRRRRLLLLEDEDAAAAGGGGVVVV*Y*YSSSSWCWCLFLF",
}


class CodonCode:
    """Codon encoding of one genetic code (datatype.py:180-297).

    Codon index = 16*n1 + 4*n2 + n3 over the nucleotide rows (A,C,G,T = 0..3);
    the state code subtracts the number of stop codons at or before that
    index.  A codon with any non-ACGTU character has code 65.
    """

    def __init__(self, table: str):
        self.table = table
        self.state_count = sum(1 for a in table if a != "*")
        acc = 0
        self.stops_upto = []
        for a in table:
            acc += a == "*"
            self.stops_upto.append(acc)

    def code(self, codon) -> int:
        n = [nucleotide_code(c) for c in codon]
        if all(v <= 3 for v in n):
            idx = n[0] * 16 + n[1] * 4 + n[2]
            return idx - self.stops_upto[idx]
        return 65

    def partial(self, codon, use_ambiguities: bool = True):
        c = self.code(codon)
        if c == 65:
            return (1.0,) * self.state_count
        return tuple(1.0 if i == c else 0.0 for i in range(self.state_count))


# ---------------------------------------------------------------- general
class GeneralCode:
    """User-defined alphabet (datatype.py:300-335)."""

    def __init__(self, codes, ambiguities=None):
        self.codes = tuple(codes)
        self.state_count = len(self.codes)
        self.index = {c: i for i, c in enumerate(self.codes)}
        self.sets = {c: [i] for i, c in enumerate(self.codes)}
        self.alias = dict(self.index)
        for amb, members in (ambiguities or {}).items():
            self.sets[amb] = [self.index[m] for m in members]
            if not isinstance(members, list) or len(members) == 1:
                self.alias[amb] = self.index[members] if isinstance(members, str) else self.index[members[0]]

    def code(self, s) -> int:
        return self.alias.get(s, self.state_count)

    def partial(self, s, use_ambiguities: bool = True):
        if s in self.sets:
            allowed = set(self.sets[s])
            return tuple(1.0 if i in allowed else 0.0 for i in range(self.state_count))
        return (1.0,) * self.state_count


# ---------------------------------------------------------------- compression
def _columns(sequences, size, indices):
    if size > 1:
        seqs = [list(zip(*[s[i::size] for i in range(size)])) for s in sequences]
    else:
        seqs = list(sequences)
    if indices is not None:
        picked = [""] * len(seqs)
        for index in indices:
            for t, s in enumerate(seqs):
                picked[t] += s[index]
        seqs = picked
    return list(zip(*seqs))


def compress(sequences, size=1, indices=None):
    """Unique columns in sorted order with their counts (site_pattern.py:69-97).

    ``sequences``: per-taxon strings in taxa order.  Returns
    ``(patterns, weights)`` where ``patterns[t]`` is the tuple of characters
    (or codon tuples) of taxon t over the sorted unique columns.
    """
    counts = Counter(_columns(sequences, size, indices))
    order = sorted(counts)
    weights = [counts[c] for c in order]
    patterns = [tuple(col[t] for col in order) for t in range(len(sequences))]
    return patterns, weights


def compress_partials(sequences, partial_fn, size=1, indices=None):
    """Tip partial vectors ``[T][S][N]`` and int weights (site_pattern.py:100-124)."""
    patterns, weights = compress(sequences, size, indices)
    tips = []
    for pat in patterns:
        cols = [partial_fn(c) for c in pat]
        tips.append([[col[s] for col in cols] for s in range(len(cols[0]))])
    return tips, weights


def compress_states(sequences, code_fn, state_count, size=1, indices=None):
    """Tip state codes ``[T][N]`` clamped to ``state_count`` (site_pattern.py:127-151)."""
    patterns, weights = compress(sequences, size, indices)
    tips = [[min(code_fn(c), state_count) for c in pat] for pat in patterns]
    return tips, weights
