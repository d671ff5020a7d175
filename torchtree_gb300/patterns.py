"""Site-pattern compression (vectorised; bit-exact with torchtree).

torchtree's ``compress`` (torchtree/evolution/site_pattern.py:69-97) counts
alignment columns with a ``Counter`` and sorts the distinct columns as
tuples of characters in taxa order.  Comparing such tuples is comparing the
columns' bytes lexicographically, which is exactly the order
``numpy.unique(axis=1)`` produces on a ``[T, L]`` uint8 matrix, with the
counts as the int64 weights (site_pattern.py:94).
"""
from __future__ import annotations

from dataclasses import dataclass

import ctypes

import numpy as np

from .datatype import DataType, Nucleotide


@dataclass
class CompressedAlignment:
    """Device-ready compressed alignment.

    ``codes``: uint8 ``[T, N]`` indexing ``table`` ``[C, S]`` (float64);
    ``weights``: int64 ``[N]``; ``columns``: uint8 ``[T, N]`` raw bytes of
    the distinct columns.
    """

    codes: np.ndarray
    table: np.ndarray
    weights: np.ndarray
    columns: np.ndarray

    @property
    def pattern_count(self) -> int:
        return int(self.weights.shape[0])

    def tip_partials(self) -> np.ndarray:
        """Partials ``[T, S, N]`` (the reference's per-tip ``[S, N]`` tensors)."""
        return np.transpose(self.table[self.codes], (0, 2, 1))


def as_byte_matrix(sequences) -> np.ndarray:
    """Stack equal-length sequences (str or bytes) into a uint8 ``[T, L]``."""
    rows = [np.frombuffer(s.encode("latin-1") if isinstance(s, str) else bytes(s), dtype=np.uint8)
            for s in sequences]
    length = {len(r) for r in rows}
    if len(length) != 1:
        raise ValueError("sequences must all have the same length")
    return np.stack(rows)


def select_sites(matrix: np.ndarray, indices) -> np.ndarray:
    """Columns picked by a list of ints / slices, in the given order (site_pattern.py:85-89)."""
    if indices is None:
        return matrix
    picks = []
    L = matrix.shape[1]
    for idx in indices:
        if isinstance(idx, slice):
            picks.extend(range(L)[idx])
        else:
            picks.append(int(idx))
    return matrix[:, picks]


def unique_columns(matrix: np.ndarray, native: bool | None = None):
    """Distinct columns in lexicographic (taxa-order) byte order and counts.

    ``native`` (default: when the engine library is built) runs the C++
    hash-and-sort compressor (``tt_compress_columns``); otherwise numpy's
    ``unique(axis=1)``.  Both give the reference's order exactly."""
    if matrix.shape[1] == 0:
        return matrix, np.zeros(0, dtype=np.int64)
    from . import _native

    if native is None:
        native = _native.LIB_PATH.exists()
    if native:
        m = np.ascontiguousarray(matrix, dtype=np.uint8)
        T, L = m.shape
        n = ctypes.c_int64()
        first = np.empty(L, dtype=np.int64)
        counts = np.empty(L, dtype=np.int64)
        lib = _native.load()
        _native.check(lib.tt_compress_columns(_native.ptr(m), T, L, ctypes.byref(n), _native.ptr(first),
                                              _native.ptr(counts), None))
        k = int(n.value)
        return np.ascontiguousarray(m[:, first[:k]]), counts[:k].copy()
    cols, counts = np.unique(matrix, axis=1, return_counts=True)
    return cols, counts.astype(np.int64)


def compress(sequences, data_type: DataType | None = None, use_ambiguities: bool = False,
             tip_states: bool = False, indices=None) -> CompressedAlignment:
    """Compress an alignment given as per-tip sequences in taxa order.

    ``use_ambiguities`` / ``tip_states`` select torchtree's
    ``compute_tips_partials(use_ambiguities)`` or ``compute_tips_states()``
    encodings.  Only single-character alphabets are handled here.
    """
    data_type = data_type or Nucleotide()
    if data_type.size == 3:
        return _compress_codons(sequences, data_type, indices)
    if data_type.size != 1:
        raise ValueError("only single-character and codon data types are supported")
    matrix = select_sites(as_byte_matrix(sequences), indices)
    cols, weights = unique_columns(matrix)
    table, lut = data_type.byte_luts(use_ambiguities, tip_states)
    codes = lut[cols]
    # keep only the table rows in use, preserving order
    used = np.unique(codes)
    remap = np.zeros(table.shape[0], dtype=np.uint8)
    remap[used] = np.arange(used.size, dtype=np.uint8)
    if not tip_states:
        table = table[used]
        codes = remap[codes]
    return CompressedAlignment(codes=np.ascontiguousarray(codes), table=table, weights=weights,
                               columns=cols)


def _compress_codons(sequences, data_type, indices=None) -> CompressedAlignment:
    """Codon sites (site_pattern.py:77-82): a column is the per-taxon tuple of
    triplets, ordered lexicographically like the reference's sorted tuples,
    i.e. by the interleaved bytes (taxon 0 positions 1-3, taxon 1, ...)."""
    raw = as_byte_matrix(sequences)
    T, L = raw.shape
    if L % 3:
        raise ValueError("codon sequences must have a multiple of 3 characters")
    trip = raw.reshape(T, L // 3, 3)
    trip = select_sites(np.ascontiguousarray(np.transpose(trip, (0, 2, 1)).reshape(T * 3, L // 3)), indices)
    cols, weights = unique_columns(trip)
    c3 = cols.reshape(T, 3, -1)
    codes = data_type.triplet_codes(c3[:, 0], c3[:, 1], c3[:, 2]).astype(np.uint8)
    return CompressedAlignment(codes=np.ascontiguousarray(codes), table=data_type.table_rows(), weights=weights,
                               columns=cols)


_FP_MULT = np.array([0x9E3779B97F4A7C15, 0xC2B2AE3D27D4EB4F, 0x165667B19E3779F9, 0xD6E8FEB86659FD93],
                    dtype=np.uint64)


def _fingerprints(rows: np.ndarray) -> np.ndarray:
    """64-bit fingerprint of each row's bytes (``rows [n, S]`` float64)."""
    words = np.ascontiguousarray(rows).view(np.uint64)
    h = np.full(rows.shape[0], 0x84222325CBF29CE4, dtype=np.uint64)
    for j in range(words.shape[1]):
        w = words[:, j]
        h = (h ^ (w ^ (w >> np.uint64(31)))) * _FP_MULT[j % 4]
        h ^= h >> np.uint64(29)
    return h


def _from_tip_partials_exact(arrs, weights) -> CompressedAlignment:
    arr = np.stack(arrs)  # [T,S,N]
    T, S, N = arr.shape
    cols = np.ascontiguousarray(np.transpose(arr, (0, 2, 1)).reshape(T * N, S))
    table, inverse = np.unique(cols, axis=0, return_inverse=True)
    if table.shape[0] > 256:
        raise ValueError(f"{table.shape[0]} distinct tip partial vectors; at most 256 are supported")
    codes = inverse.reshape(T, N).astype(np.uint8)
    return CompressedAlignment(codes=codes, table=table, weights=np.asarray(weights),
                               columns=np.zeros((T, 0), dtype=np.uint8))


def from_tip_partials(tips, weights) -> CompressedAlignment:
    """Codes and table from arbitrary tip partial tensors ``T x [S, N]``.

    The distinct tip columns become the table (at most 256), in order of
    first appearance.  Tips are taken one at a time: each column gets a
    64-bit fingerprint of its bytes, a table row per new fingerprint, and the
    decoded tip is compared with the original exactly; a fingerprint shared
    by two different columns (or a NaN) falls back to one lexicographic
    ``np.unique`` over all columns.
    """
    arrs = [np.asarray(t, dtype=np.float64) for t in tips]
    T = len(arrs)
    S, N = arrs[0].shape
    codes = np.empty((T, N), dtype=np.uint8)
    index: dict = {}  # fingerprint -> code
    rows_of: list = []  # code -> table row
    for t, a in enumerate(arrs):
        if a.shape != (S, N):
            raise ValueError("every tip partial must have shape [S, N]")
        rows = np.ascontiguousarray(a.T)  # [N, S]
        uniq, first, inverse = np.unique(_fingerprints(rows), return_index=True, return_inverse=True)
        local = np.empty(uniq.size, dtype=np.int64)
        for i, (key, f) in enumerate(zip(uniq.tolist(), first.tolist())):
            c = index.get(key)
            if c is None:  # distinct fingerprints are distinct columns
                c = len(rows_of)
                if c >= 256:
                    raise ValueError("more than 256 distinct tip partial vectors; at most 256 are supported")
                index[key] = c
                rows_of.append(rows[f].copy())
            local[i] = c
        code = local[inverse.reshape(-1)]
        if not np.array_equal(np.stack(rows_of)[code], rows):
            return _from_tip_partials_exact(arrs, weights)
        codes[t] = code
    return CompressedAlignment(codes=codes, table=np.stack(rows_of), weights=np.asarray(weights),
                               columns=np.zeros((T, 0), dtype=np.uint8))


def from_tip_states(tips, state_count: int, weights) -> CompressedAlignment:
    """Codes from tip state tensors ``T x [N]`` with values in ``[0, S]``."""
    codes = np.stack([np.asarray(t, dtype=np.int64) for t in tips])
    if codes.min() < 0 or codes.max() > state_count:
        raise ValueError("tip states must lie in [0, state_count]")
    table = np.vstack([np.eye(state_count), np.ones((1, state_count))])
    return CompressedAlignment(codes=codes.astype(np.uint8), table=table, weights=np.asarray(weights),
                               columns=np.zeros((codes.shape[0], 0), dtype=np.uint8))
