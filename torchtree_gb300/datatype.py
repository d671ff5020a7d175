"""Tip encodings: byte -> tip partial vector lookup tables.

Vectorised counterparts of torchtree's data types
(torchtree/evolution/datatype.py:57-335).  Every tip partial torchtree can
produce is a 0/1 vector, so a compressed alignment is stored on the device
as one uint8 code per tip and pattern plus a small table of the distinct
vectors (``codes``, ``table``).  The byte rules below reproduce the
reference's ASCII tables exactly (pinned by the golden fixtures):

* nucleotides: IUPAC letters in either case; U/u behave as T; any other
  letter and '?' are "unknown" (all states); every other byte is a gap
  (all states).  Without ambiguities, anything but ACGTU is all states.
* amino acids: the 20 residues, B = D|N, Z = E|Q; X, '*', J, O, U, '?' and
  every other byte are all states.  Without ambiguities, anything but the 20
  residues is all states.
* tip states (``compute_tips_states``): the state index for an unambiguous
  character, otherwise the extra code S whose row is all ones.
"""
from __future__ import annotations

import numpy as np

_NUC_SETS = {
    "A": "A", "C": "C", "G": "G", "T": "T", "U": "T", "R": "AG", "Y": "CT", "M": "AC", "W": "AT",
    "S": "CG", "K": "GT", "B": "CGT", "D": "AGT", "H": "ACT", "V": "ACG", "N": "ACGT",
}
_AA = "ACDEFGHIKLMNPQRSTVWY"


class DataType:
    """Byte-level encoding of one alphabet."""

    name = "abstract"
    state_count = 0
    size = 1  # characters per site (3 for codons)

    def partial_vector(self, byte: int, use_ambiguities: bool) -> tuple:
        raise NotImplementedError

    def state_code(self, byte: int) -> int:
        """State index, or ``state_count`` for anything ambiguous."""
        raise NotImplementedError

    def byte_luts(self, use_ambiguities: bool, tip_states: bool = False):
        """(table [C,S] float64, lut [256] uint8) mapping bytes to codes.

        Tip-state mode uses the table [I_S; ones]; partial mode numbers the
        distinct vectors in order of first appearance over bytes 0..255,
        after the S one-hot vectors and the all-ones vector.
        """
        S = self.state_count
        rows = [tuple(1.0 if j == i else 0.0 for j in range(S)) for i in range(S)]
        rows.append((1.0,) * S)
        index = {r: i for i, r in enumerate(rows)}
        lut = np.zeros(256, dtype=np.uint8)
        for byte in range(256):
            if tip_states:
                lut[byte] = min(self.state_code(byte), S)
                continue
            vec = self.partial_vector(byte, use_ambiguities)
            if vec not in index:
                index[vec] = len(rows)
                rows.append(vec)
            lut[byte] = index[vec]
        return np.asarray(rows, dtype=np.float64), lut


class Nucleotide(DataType):
    name = "nucleotide"
    state_count = 4

    def partial_vector(self, byte, use_ambiguities=True):
        ch = chr(byte).upper() if byte < 128 else "\0"
        if not use_ambiguities and ch not in "ACGTU":
            return (1.0,) * 4
        allowed = _NUC_SETS.get(ch, "ACGT")
        return tuple(1.0 if s in allowed else 0.0 for s in "ACGT")

    def state_code(self, byte):
        ch = chr(byte).upper() if byte < 128 else "\0"
        return {"A": 0, "C": 1, "G": 2, "T": 3, "U": 3}.get(ch, 4)


class AminoAcid(DataType):
    name = "amino_acid"
    state_count = 20

    def partial_vector(self, byte, use_ambiguities=True):
        ch = chr(byte).upper() if byte < 128 else "\0"
        if ch in _AA:
            return tuple(1.0 if a == ch else 0.0 for a in _AA)
        if not use_ambiguities:
            return (1.0,) * 20
        allowed = {"B": "DN", "Z": "EQ"}.get(ch)
        if allowed is None:
            return (1.0,) * 20
        return tuple(1.0 if a in allowed else 0.0 for a in _AA)

    def state_code(self, byte):
        ch = chr(byte).upper() if byte < 128 else "\0"
        return _AA.index(ch) if ch in _AA else 20


class General(DataType):
    """User alphabet (datatype.py:300-335): single characters and ambiguity sets."""

    name = "general"

    def __init__(self, codes, ambiguities=None):
        self.codes = tuple(codes)
        self.state_count = len(self.codes)
        self.sets = {c: [i] for i, c in enumerate(self.codes)}
        self.alias = {c: i for i, c in enumerate(self.codes)}
        for amb, members in (ambiguities or {}).items():
            self.sets[amb] = [self.codes.index(m) for m in members]
            if isinstance(members, str) and len(members) == 1:
                self.alias[amb] = self.codes.index(members)

    def partial_vector(self, byte, use_ambiguities=True):
        ch = chr(byte)
        allowed = self.sets.get(ch)
        if allowed is None:
            return (1.0,) * self.state_count
        return tuple(1.0 if i in allowed else 0.0 for i in range(self.state_count))

    def state_code(self, byte):
        return self.alias.get(chr(byte), self.state_count)


class Codon(DataType):
    """Codons of one genetic code (datatype.py:180-297): a site is three
    bytes; the state is 16*n1 + 4*n2 + n3 over A,C,G,T(U) minus the stop
    codons before it; any other byte in the triplet makes the codon unknown
    (all states, tip-state code ``state_count``).  Ambiguity flags are ignored,
    as in the reference, and a stop codon takes the code of the sense codon
    before it (the reference subtracts the stop count including itself)."""

    name = "codon"
    size = 3
    UNIVERSAL = "KNKNTTTTRSRSIIMIQHQHPPPPRRRRLLLLEDEDAAAAGGGGVVVV*Y*YSSSS*CWCLFLF"

    def __init__(self, table: str = UNIVERSAL):
        self.table = table
        stops = np.array([c == "*" for c in table[:64]], dtype=np.int64)
        self.state_count = int(64 - stops.sum())
        self._shift = np.cumsum(stops)
        nuc = np.full(256, 4, dtype=np.int64)
        for ch, v in (("A", 0), ("C", 1), ("G", 2), ("T", 3), ("U", 3)):
            nuc[ord(ch)] = nuc[ord(ch.lower())] = v
        self._nuc = nuc

    def triplet_codes(self, b1: np.ndarray, b2: np.ndarray, b3: np.ndarray) -> np.ndarray:
        """Codes (0..S-1, or S for unknown/stop) of byte triplets."""
        n1, n2, n3 = self._nuc[b1], self._nuc[b2], self._nuc[b3]
        ok = (n1 < 4) & (n2 < 4) & (n3 < 4)
        idx = np.where(ok, n1 * 16 + n2 * 4 + n3, 0)
        code = idx - self._shift[idx]  # a stop codon lands on the sense codon before it, as in the reference
        return np.where(ok, code, self.state_count)

    def table_rows(self) -> np.ndarray:
        S = self.state_count
        return np.vstack([np.eye(S), np.ones((1, S))])


def get(name: str) -> DataType:
    if name in ("nucleotide", "dna"):
        return Nucleotide()
    if name in ("amino_acid", "protein", "aa"):
        return AminoAcid()
    if name in ("codon", "codon_universal"):
        return Codon()
    raise ValueError(f"unknown data type {name!r}")
