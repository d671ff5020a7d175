"""Kernel-shape autotuner.

A plan's kernel shapes (staging-ring depths of the FP32 4-state kernels,
the in-place or shared-memory-stack adjoint, pair-thread kernels, tensor-core
or CUDA-core codon post-order) do not change results, only speed.  ``tune`` times one full step under each candidate option set with
CUDA events and leaves the fastest set on the plan.  Choices are cached per
problem shape (tips, patterns, states, categories, batch, precision), so a
serving process tunes each shape once.
"""
from __future__ import annotations

import statistics

import torch

from . import _native
from ._native import EngineError

_CACHE: dict = {}


def candidates(engine) -> list:
    """Option sets worth timing for this plan."""
    if engine.precision == "f32" and engine.state_count == 4:
        F, B, Q = _native.TT_OPT_FWD_STAGES, _native.TT_OPT_BWD_STAGES, _native.TT_OPT_PAIR_THREADS
        W, P = _native.TT_OPT_PRODUCER_WARP, _native.TT_OPT_INPLACE_ADJOINT
        return [{Q: 0, W: 1, P: 1, F: 6, B: 2}, {Q: 0, W: 1, P: 1, F: 4, B: 3}, {Q: 0, W: 1, P: 0, F: 6, B: 2},
                {Q: 1, W: 0, P: 0, F: 6, B: 3}]
    if engine.precision == "f32" and engine.state_count > 20:
        return [{_native.TT_OPT_TENSOR_CORES: 1}, {_native.TT_OPT_TENSOR_CORES: 0}]
    return [{}]


def shape_key(engine) -> tuple:
    return (engine.tip_count, engine.pattern_count, engine.state_count, engine.category_count, engine.batch,
            engine.precision)


def _apply(engine, opts: dict) -> bool:
    try:
        for k, v in opts.items():
            engine.set_option(k, v)
        return True
    except EngineError:
        return False


def tune(engine, step, repeats: int = 3, cache: dict | None = None) -> dict:
    """Time ``step()`` (one full lnL + gradient evaluation on the current
    stream) under each candidate; apply and return the fastest option set."""
    cache = _CACHE if cache is None else cache
    key = shape_key(engine)
    if key in cache:
        _apply(engine, cache[key])
        return cache[key]
    cands = candidates(engine)
    best, best_ms = {}, float("inf")
    if len(cands) > 1:
        stream = torch.cuda.current_stream()
        for opts in cands:
            if not _apply(engine, opts):
                continue
            step()  # warm-up
            times = []
            for _ in range(repeats):
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                step()
                b.record(stream)
                b.synchronize()
                times.append(a.elapsed_time(b))
            ms = statistics.median(times)
            if ms < best_ms:
                best, best_ms = opts, ms
        _apply(engine, best)
    cache[key] = best
    return best
