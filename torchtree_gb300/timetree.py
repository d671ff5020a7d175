"""Time-tree operations on the GPU: node-height ratio transform and the
constant-size coalescent, batched over samples, as autograd functions.

``RatioTransform`` maps the reference's ``GeneralNodeHeightTransform``
parameters (ratios of the non-root internal nodes, root height last;
torchtree/evolution/tree_height_transform.py:7-99) to internal node heights,
branch lengths (tree_model.py:23-40) and log|det J|; ``constant_coalescent``
is ``ConstantCoalescent.log_prob`` (torchtree/evolution/coalescent.py:86-134).
Both run the C-ABI kernels of ``csrc/tt_timetree.cu`` on the current stream.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _native
from ._native import check, ptr


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class TimeTree:
    """A rooted time tree: topology (post-order triples, root 2T-2 last) and
    the tips' sampling times, resident on the current CUDA device."""

    def __init__(self, postorder, sampling_times):
        if not torch.cuda.is_available():
            raise RuntimeError("torchtree_gb300 needs a CUDA device; there is no CPU fallback")
        self.lib = _native.load()
        post = np.ascontiguousarray(np.asarray(postorder, dtype=np.int32).reshape(-1, 3))
        times = np.ascontiguousarray(np.asarray(sampling_times, dtype=np.float64))
        self.tip_count = int(times.shape[0])
        self.device = torch.device("cuda", torch.cuda.current_device())
        h = ctypes.c_void_p()
        check(self.lib.tt_time_tree_create(ctypes.byref(h), self.tip_count,
                                           post.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), ptr(times)))
        self._tree = h

    def __del__(self):
        try:
            if getattr(self, "_tree", None):
                self.lib.tt_time_tree_destroy(self._tree)
                self._tree = None
        except Exception:
            pass

    def ratio_transform(self, ratios: torch.Tensor):
        """``(heights [b,T-1], branch_lengths [b,2T-2], log|J| [b])``, differentiable."""
        return _RatioTransform.apply(ratios, self)

    def constant_coalescent(self, heights: torch.Tensor, theta: torch.Tensor) -> torch.Tensor:
        """Log-density ``[b]`` of internal heights ``[b,T-1]`` under population size ``theta [b]``."""
        return _ConstantCoalescent.apply(heights, theta, self)


def _dev(x, device):
    return x.detach().to(device=device, dtype=torch.float64).contiguous()


class _RatioTransform(torch.autograd.Function):
    @staticmethod
    def forward(ctx, ratios, tree):
        x = _dev(ratios, tree.device)
        b, T = x.shape[0], tree.tip_count
        kw = dict(dtype=torch.float64, device=tree.device)
        h, bl, ld = torch.empty(b, T - 1, **kw), torch.empty(b, 2 * T - 2, **kw), torch.empty(b, **kw)
        check(tree.lib.tt_ratio_transform(tree._tree, b, ptr(x), ptr(h), ptr(bl), ptr(ld), _stream()))
        ctx.tree = tree
        ctx.save_for_backward(x, h)
        return h.to(ratios.dtype), bl.to(ratios.dtype), ld.to(ratios.dtype)

    @staticmethod
    def backward(ctx, gh, gbl, gld):
        x, h = ctx.saved_tensors
        tree = ctx.tree
        b = x.shape[0]
        args = [None if g is None else _dev(g, tree.device) for g in (gh, gbl, gld)]
        gx = torch.empty_like(x)
        check(tree.lib.tt_ratio_transform_backward(tree._tree, b, ptr(x), ptr(h), *map(ptr, args), ptr(gx),
                                                   _stream()))
        return gx, None


class _ConstantCoalescent(torch.autograd.Function):
    @staticmethod
    def forward(ctx, heights, theta, tree):
        h = _dev(heights, tree.device)
        b = h.shape[0]
        th = _dev(theta, tree.device).reshape(-1).expand(b).contiguous()
        kw = dict(dtype=torch.float64, device=tree.device)
        lp, gh, gth = torch.empty(b, **kw), torch.empty_like(h), torch.empty(b, **kw)
        check(tree.lib.tt_constant_coalescent(tree._tree, b, ptr(h), ptr(th), ptr(lp), ptr(gh), ptr(gth),
                                              _stream()))
        ctx.save_for_backward(gh, gth)
        ctx.theta_shape = theta.shape
        return lp.to(heights.dtype)

    @staticmethod
    def backward(ctx, g):
        gh, gth = ctx.saved_tensors
        g = g.to(torch.float64)
        dth = (gth * g)
        if dth.numel() != int(np.prod(ctx.theta_shape)):
            dth = dth.sum().reshape(ctx.theta_shape)
        return gh * g[:, None], dth.reshape(ctx.theta_shape), None
