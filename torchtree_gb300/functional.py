"""Drop-in counterparts of torchtree's pruning functions.

Same names, arguments and return shapes as
``torchtree.evolution.tree_likelihood.calculate_treelikelihood*``
(torchtree/evolution/tree_likelihood.py:14-278), computed by the GPU engine
and differentiable with respect to ``mats``, ``freqs`` and ``props``:

* ``partials``: list of T tip tensors ``[S, N]`` (or int codes ``[N]`` for
  the ``tip_states`` variants) followed by T-1 placeholders;
* ``weights [N]``; ``post_indexing``: ``(node, left, right)`` triples;
* ``mats [..., B, K, S, S]`` (``[..., B, S, S]`` for the single-category
  function); ``freqs [..., 1, S]``; ``props [..., K, 1, 1]``;
* result: lnL ``[..., 1]``.

The unscaled functions run the kernels without rescaling, exactly like the
reference.  ``*_rescaled`` and ``*_safe`` rescale every node by a power of
two; the reference's ``_safe`` rescales only nodes below ``threshold`` after
an underflow, and both give the same lnL up to rounding.  ``precision``
selects FP64 (default, the drop-in) or rescaled FP32 partials.  The tip
data stay resident on the device between calls with the same, unmodified
tensors (an in-place change to a tip or weight tensor makes a new engine).
"""
from __future__ import annotations

import math

import numpy as np
import torch

from . import patterns
from .autograd import MatrixLikelihood
from .engine import LikelihoodEngine

_ENGINES: "OrderedDict" = None
# Resident engines are kept for repeated calls on the same tip data, at most
# _MAX_ENGINES of them and at most _MAX_CACHED_BYTES of device workspace in
# total (least recently used first out).  An engine that alone exceeds the
# byte budget is not cached at all.
_MAX_ENGINES = 4
_MAX_CACHED_BYTES = 8 << 30


def _identity(t: torch.Tensor):
    """Identity of a tensor's current contents: the object, its storage and
    its version counter (bumped by every in-place change)."""
    return (id(t), t.data_ptr(), t._version, tuple(t.shape), t.dtype)


def _engine(tips, weights, post_indexing, S, K, batch, precision, tip_states):
    global _ENGINES
    from collections import OrderedDict

    if _ENGINES is None:
        _ENGINES = OrderedDict()
    key = (tuple(map(tuple, post_indexing)), tuple(_identity(t) for t in tips), _identity(weights), S, K,
           batch, precision, tip_states)
    hit = _ENGINES.get(key)
    if hit is not None:
        _ENGINES.move_to_end(key)
        return hit[0]
    w = weights.detach().cpu().numpy()
    if tip_states:
        ca = patterns.from_tip_states([t.detach().cpu().numpy() for t in tips], S, w)
    else:
        ca = patterns.from_tip_partials([t.detach().cpu().numpy() for t in tips], w)
    device = None
    eng = LikelihoodEngine(np.asarray(post_indexing, dtype=np.int32), len(tips), S, K, ca.codes, ca.table,
                           w, batch=batch, precision=precision, device=device)
    size = eng.workspace_bytes
    if size <= _MAX_CACHED_BYTES:
        while _ENGINES and (len(_ENGINES) >= _MAX_ENGINES or
                            sum(v[0].workspace_bytes for v in _ENGINES.values()) + size > _MAX_CACHED_BYTES):
            _ENGINES.popitem(last=False)  # freed once no autograd graph holds it
        _ENGINES[key] = (eng, tips, weights)  # keep the tensors alive so that ids stay unique
    return eng


def clear_cache() -> None:
    if _ENGINES is not None:
        _ENGINES.clear()


def _run(partials, weights, post_indexing, mats, freqs, props, rescale, precision, tip_states):
    tip_count = len(post_indexing) + 1
    tips = partials[:tip_count]
    S = mats.shape[-1]
    K = mats.shape[-3]
    B = mats.shape[-4]
    batch_shape = torch.broadcast_shapes(mats.shape[:-4], freqs.shape[:-2], props.shape[:-3])
    b = math.prod(batch_shape)
    dev = torch.device("cuda", torch.cuda.current_device())
    m = mats.to(dev).expand(batch_shape + mats.shape[-4:]).reshape(b, B, K, S, S)
    f = freqs.to(dev).expand(batch_shape + freqs.shape[-2:]).reshape(b, S)
    p = props.to(dev).expand(batch_shape + props.shape[-3:]).reshape(b, K)
    eng = _engine(tips, weights, post_indexing, S, K, b, precision, tip_states)
    lnl = MatrixLikelihood.apply(m, p, f, eng, rescale)
    return lnl.reshape(batch_shape + (1,)).to(mats.device)


def calculate_treelikelihood(partials, weights, post_indexing, mats, freqs, precision="f64"):
    """Single-category pruning (tree_likelihood.py:14-37)."""
    ones = torch.ones(mats.shape[:-3] + (1, 1, 1), dtype=mats.dtype, device=mats.device)
    return _run(partials, weights, post_indexing, mats.unsqueeze(-3), freqs, ones, False, precision,
                False)


def calculate_treelikelihood_discrete(partials, weights, post_indexing, mats, freqs, props,
                                      precision="f64"):
    """K-category pruning without rescaling (tree_likelihood.py:40-75)."""
    return _run(partials, weights, post_indexing, mats, freqs, props, False, precision, False)


def calculate_treelikelihood_tip_states_discrete(partials, weights, post_indexing, mats, freqs,
                                                 props, precision="f64"):
    """Tip-state-code pruning without rescaling (tree_likelihood.py:78-131)."""
    return _run(partials, weights, post_indexing, mats, freqs, props, False, precision, True)


def calculate_treelikelihood_discrete_safe(partials, weights, post_indexing, mats, freqs, props,
                                           threshold, precision="f64"):
    """Rescaled pruning (the result of tree_likelihood.py:134-183)."""
    del threshold
    return _run(partials, weights, post_indexing, mats, freqs, props, True, precision, False)


def calculate_treelikelihood_discrete_rescaled(partials, weights, post_indexing, mats, freqs, props,
                                               precision="f64"):
    """Pruning with rescaling (tree_likelihood.py:186-221)."""
    return _run(partials, weights, post_indexing, mats, freqs, props, True, precision, False)


def calculate_treelikelihood_tip_states_discrete_rescaled(partials, weights, post_indexing, mats,
                                                          freqs, props, precision="f64"):
    """Tip-state-code pruning with rescaling (tree_likelihood.py:224-278)."""
    return _run(partials, weights, post_indexing, mats, freqs, props, True, precision, True)
