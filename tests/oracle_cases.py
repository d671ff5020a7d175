"""Helpers that turn a golden likelihood record into oracle / engine inputs.

Shared by the CPU oracle tests and the GPU parity tests.  Only the oracle
(CPU) path needs torch autograd; the GPU path reuses ``record_inputs``.
"""
from __future__ import annotations

import numpy as np
import torch

from oracle import likelihood as OL
from oracle import patterns as OP


def record_encoding(rec):
    """(code_fn, partial_fn(use_ambiguities), state_count, characters per site) of a record's data type."""
    kind = rec.get("data_type", "nucleotide")
    if kind == "amino_acid":
        return OP.amino_acid_code, OP.amino_acid_partial, 20, 1
    if kind == "codon":
        cc = OP.CodonCode(OL.UNIVERSAL_CODE)
        return cc.code, cc.partial, cc.state_count, 3
    return OP.nucleotide_code, OP.nucleotide_partial, 4, 1


def state_count_of(rec) -> int:
    return record_encoding(rec)[2]


def tips_from_record(rec, dtype=torch.float64):
    seqs = rec["sequences"]
    code_fn, partial_fn, S, size = record_encoding(rec)
    if rec.get("tip_states"):
        tips, w = OP.compress_states(seqs, code_fn, S, size=size)
        return [torch.tensor(t, dtype=torch.long) for t in tips], torch.tensor(w)
    amb = rec.get("use_ambiguities", False)
    tips, w = OP.compress_partials(seqs, lambda c: partial_fn(c, amb), size=size)
    return [torch.tensor(t, dtype=dtype) for t in tips], torch.tensor(w)


def record_inputs(rec, requires_grad=True):
    """Leaf tensors (bl, exch, pi, shape, invariant) of a record."""
    t = lambda x: torch.tensor(x, dtype=torch.float64, requires_grad=requires_grad)  # noqa: E731
    out = {"bl": t(rec["branch_lengths"])}
    if rec["model"] != "jc69":
        out["exch"] = t(rec["exch"])
        out["pi"] = t(rec["pi"])
    if rec["site_model"] == "weibull":
        out["shape"] = t(rec["shape"])
    if "invariant" in rec:
        out["invariant"] = t(rec["invariant"])
    return out


def model_pieces(rec, x):
    """(q_unnorm or None, pi, rates, probs, node branch lengths) for a record."""
    bls = OL.model_branch_lengths(x["bl"])
    if rec["model"] == "jc69":
        pi = torch.full((4,), 0.25, dtype=torch.float64)
        q = None
    elif rec["model"] == "gtr":
        pi = x["pi"]
        q = OL.q_gtr(x["exch"], pi)
    elif rec["model"] == "general":
        pi = x["pi"]
        q = OL.q_general_symmetric(x["exch"], pi, pi.shape[-1])
    elif rec["model"] == "mg94":  # exch = (kappa, omega), alpha = 1
        pi = x["pi"]
        kappa, omega = x["exch"][..., 0:1], x["exch"][..., 1:2]
        q = OL.q_mg94(torch.ones_like(kappa), omega, kappa, pi)
    else:
        pi = x["pi"]
        q = OL.q_hky(x["exch"], pi)
    if rec["site_model"] == "weibull":
        rates, probs = OL.weibull_rates(x["shape"], rec["categories"], x.get("invariant"))
    elif rec["site_model"] == "constant":
        rates = torch.ones(1, dtype=torch.float64)
        probs = torch.ones(1, dtype=torch.float64)
    else:
        rates = torch.tensor(rec["category_rates"], dtype=torch.float64)
        probs = torch.full((rec["categories"],), 1.0 / rec["categories"], dtype=torch.float64)
    return q, pi, rates, probs, bls


def oracle_lnl(rec, x):
    tips, w = tips_from_record(rec)
    q, pi, rates, probs, bls = model_pieces(rec, x)
    times = bls.unsqueeze(-1) * rates.unsqueeze(-2)
    mats = OL.p_t_jc69(times) if q is None else OL.p_t_symmetric(q, pi, times)
    freqs = pi.unsqueeze(-2)
    props = probs.unsqueeze(-1).unsqueeze(-1)
    post = rec["postorder"]
    parts = list(tips) + [None] * (len(tips) - 1)
    if rec.get("tip_states"):
        fn = (OL.treelikelihood_tip_states_discrete_rescaled if rec.get("rescale", False)
              else OL.treelikelihood_tip_states_discrete)
        lnl = fn(parts, w, post, mats, freqs, props)
        if not rec.get("rescale", False) and torch.isinf(lnl).any():
            lnl = OL.treelikelihood_tip_states_discrete_rescaled(parts, w, post, mats, freqs, props)
        return lnl
    if rec.get("rescale", False):
        return OL.treelikelihood_discrete_rescaled(parts, w, post, mats, freqs, props)
    lnl, _ = OL.unscaled_then_safe(parts, w, post, mats, freqs, props, 1e-40)
    return lnl


GRAD_KEYS = (("bl", "grad_branch_lengths"), ("exch", "grad_exch"), ("pi", "grad_pi"),
             ("shape", "grad_shape"), ("invariant", "grad_invariant"))


def as_np(x):
    return np.asarray(x, dtype=np.float64)
