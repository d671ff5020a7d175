"""CPU restatement of the time-tree operations around the likelihood.

TEST INFRASTRUCTURE ONLY: imported by ``tests/`` as the checker of the GPU
kernels in ``torchtree_gb300/csrc/tt_timetree.cu``; pinned against
``tests/golden/timetree.json`` (outputs of the reference itself).

* ``ratio_transform`` follows torchtree/evolution/tree_height_transform.py:
  38-60 (lower bounds), 62-70 (pre-order heights) and 92-95 (log|det J|),
  with branch lengths as in tree_model.py:23-40;
* ``constant_coalescent`` follows coalescent.py:112-134.
"""
from __future__ import annotations

import torch


def lower_bounds(postorder, times):
    T = len(times)
    lb = [0.0] * (T - 1)
    for v, l, r in postorder:
        hl = times[l] if l < T else lb[l - T]
        hr = times[r] if r < T else lb[r - T]
        lb[v - T] = max(hl, hr)
    return lb


def ratio_transform(postorder, times, ratios: torch.Tensor):
    """``ratios [..., T-1]`` (non-root internal nodes by index - T, root height
    last) -> (internal heights, branch lengths [..., 2T-2], log|J|)."""
    T = len(times)
    lb = lower_bounds(postorder, times)
    parent = {}
    for v, l, r in postorder:
        parent[int(l)] = int(v)
        parent[int(r)] = int(v)
    h = [None] * (T - 1)
    h[T - 2] = ratios[..., T - 2]
    logdet = torch.zeros_like(ratios[..., 0])
    for v, _, _ in reversed(postorder[:-1]):  # pre-order of the non-root internal nodes
        v = int(v)
        span = h[parent[v] - T] - lb[v - T]
        h[v - T] = lb[v - T] + ratios[..., v - T] * span
        logdet = logdet + torch.log(span)
    heights = torch.stack(h, -1)
    bl = []
    for n in range(2 * T - 2):
        hn = torch.full_like(heights[..., 0], float(times[n])) if n < T else heights[..., n - T]
        bl.append(heights[..., parent[n] - T] - hn)
    return heights, torch.stack(bl, -1), logdet


def constant_coalescent(times, internal: torch.Tensor, theta: torch.Tensor):
    """log p of node heights (tips' sampling times + ``internal``) under theta."""
    T = len(times)
    t = torch.tensor(times, dtype=internal.dtype).expand(internal.shape[:-1] + (T,))
    heights = torch.cat((t, internal), -1)
    mask = torch.cat((torch.ones(T), -torch.ones(T - 1))).to(internal.dtype)
    order = torch.argsort(heights, -1)
    hs = torch.gather(heights, -1, order)
    ms = mask[order]
    lineages = ms.cumsum(-1)[..., :-1]
    dur = hs[..., 1:] - hs[..., :-1]
    c = lineages * (lineages - 1) / 2.0
    return torch.sum(-c * dur / theta[..., None], -1) - (T - 1) * torch.log(theta)
