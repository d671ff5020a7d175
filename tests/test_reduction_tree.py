"""Host emulation of the DNA adjoint's pattern-reduction tree
(``csrc/tt_prune_ta.cuh``), in FP32 numpy.

UR lanes each hold a 4 x 4 block of category pairs (32 floats); recursive
halving across the lanes leaves each lane 32 / UR of the block's sums.  The
kernel's tree loads rows i ^ a (and, for an internal child, jj ^ b; for a
tip child only the jj1 half swap) so that every lane keeps the lower half of
its registers at the permuted levels.  These tests run that tree and the
plain select-based halving on the same per-lane partial sums and check that
they write the same block bit for bit: the same lanes add the same operands
at every level.
"""
import numpy as np
import pytest


def _plain_tree(blocks: np.ndarray) -> np.ndarray:
    """Select-based recursive halving over the block index
    (k << 4) | (i << 2) | jj, top bit first; lane s keeps NV = 32 / UR
    consecutive floats starting at NV * s."""
    UR = blocks.shape[0]
    f = [blocks[s].transpose(2, 0, 1).reshape(32).copy() for s in range(UR)]  # [k][i][jj]
    o, h = UR // 2, 16
    while o >= 1:
        new = []
        for s in range(UR):
            p = s ^ o
            up = (s & o) != 0
            keep = f[s][h:2 * h] if up else f[s][:h]
            recv = f[p][h:2 * h] if up else f[p][:h]  # the partner sends the half it does not keep
            new.append((keep + recv).astype(np.float32))
        f = new
        o, h = o // 2, h // 2
    out = np.zeros(32, np.float32)
    nv = 32 // UR
    for s in range(UR):
        out[nv * s: nv * s + nv] = f[s][:nv]
    return out


def _permuted_tree(blocks: np.ndarray, tip: bool) -> np.ndarray:
    """The kernel's tree: slot (i', jj') of lane s holds element
    (i' ^ a, jj' ^ b) as a category pair; select-free levels for i1, i0,
    jj1 and (internal child) jj0; selects for a tip's jj0 and the category
    level (32 lanes)."""
    UR = blocks.shape[0]
    LV = int(np.log2(UR))
    g = []
    for s in range(UR):
        bits = s << (5 - LV)
        a, b = bits >> 3, (bits >> 1) & (2 if tip else 3)
        g.append(np.array([[blocks[s][i ^ a][j ^ b] for j in range(4)] for i in range(4)],
                          np.float32).reshape(16, 2))
    o, h = UR // 2, 8
    while o >= 1 and h >= 1:
        new = []
        for s in range(UR):
            p = s ^ o
            if h >= 2 or not tip:
                new.append((g[s][:h] + g[p][h:2 * h]).astype(np.float32))
            else:  # a tip's jj0 level: plain halving
                up = (s & o) != 0
                keep = g[s][h:2 * h] if up else g[s][:h]
                recv = g[p][h:2 * h] if up else g[p][:h]
                new.append((keep + recv).astype(np.float32))
        g = new
        o, h = o // 2, h // 2
    out = np.zeros(32, np.float32)
    if LV == 5:  # the category level
        for s in range(UR):
            up = s & 1
            keep, recv = g[s][0][up], g[s ^ 1][0][up]  # both lanes' category `up`
            k = s & 1
            out[k * 16 + (s >> 1)] = np.float32(keep + recv)
        return out
    ng = 16 >> LV
    for s in range(UR):
        for slot in range(ng):
            el = (s << (4 - LV)) | slot
            out[el] = g[s][slot][0]
            out[16 + el] = g[s][slot][1]
    return out


@pytest.mark.parametrize("UR", [8, 16, 32])
@pytest.mark.parametrize("tip", [False, True])
def test_permuted_tree_writes_the_plain_trees_block(UR, tip):
    rng = np.random.default_rng(UR + 7 * tip)
    for _ in range(20):
        # per-lane partial sums of one (child, category pair) block: [lane][i][jj][k]
        blocks = (rng.standard_normal((UR, 4, 4, 2)) * rng.uniform(1e-3, 1e3)).astype(np.float32)
        want = _plain_tree(blocks)
        got = _permuted_tree(blocks, tip)
        np.testing.assert_array_equal(got, want)
        exact = blocks.astype(np.float64).sum(0).transpose(2, 0, 1).reshape(32)
        np.testing.assert_allclose(got, exact, rtol=1e-5, atol=1e-5 * np.abs(exact).max())
