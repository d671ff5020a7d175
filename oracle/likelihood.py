"""FP64 CPU restatement of torchtree's likelihood path.

TEST INFRASTRUCTURE ONLY: the checker of the GPU kernels in ``tests/`` and
``__graft_entry__.smoke()``, and the timed CPU baseline of ``bench.py``;
never imported by the package.  Pinned against the reference's golden
vectors (``tests/golden/``) and, where its source is present, against the
reference's own functions on random problems.

Every function states the reference code it restates (paths inside the
torchtree 1.0.2 project).  Tensors are torch CPU tensors; gradients come from
torch autograd, which is how the reference obtains them (it has no hand-written
gradient).  Shapes follow the reference: tips ``[S,N]`` (or ``[N]`` state
codes), internal partials ``[*b,K,S,N]``, transition matrices
``[*b,B,K,S,S]``, frequencies ``[*b,1,S]``, proportions ``[*b,K,1,1]``.
"""
from __future__ import annotations

import itertools
import math

import numpy as np
import torch

# --------------------------------------------------------------------------
# Rate matrices
# --------------------------------------------------------------------------


def q_jc69(dtype=torch.float64) -> torch.Tensor:
    """JC69 rate matrix (evolution/substitution_model/nucleotide.py:115-126)."""
    q = torch.full((4, 4), 1.0 / 3.0, dtype=dtype)
    q.fill_diagonal_(-1.0)
    return q


def p_t_jc69(branch_lengths: torch.Tensor) -> torch.Tensor:
    """JC69 closed form P(t) (evolution/substitution_model/nucleotide.py:102-113).

    ``branch_lengths [...]`` -> ``[..., 4, 4]``.
    """
    e = torch.exp(-4.0 / 3.0 * branch_lengths)
    same = 0.25 + 0.75 * e
    diff = 0.25 - 0.25 * e
    eye = torch.eye(4, dtype=branch_lengths.dtype)
    return diff[..., None, None] * (1 - eye) + same[..., None, None] * eye


def _assemble_q(exch: torch.Tensor, pi: torch.Tensor) -> torch.Tensor:
    """Q_ij = R_ij * pi_j off the diagonal, rows summing to zero.

    ``exch [...,S,S]`` symmetric with zero diagonal, ``pi [...,S]``.
    """
    q = exch * pi.unsqueeze(-2)
    diag = -q.sum(-1)
    return q + torch.diag_embed(diag)


def q_hky(kappa: torch.Tensor, pi: torch.Tensor) -> torch.Tensor:
    """HKY rate matrix (evolution/substitution_model/nucleotide.py:238-264).

    ``kappa [...,1]``, ``pi [...,4]`` (order A,C,G,T); transitions are A<->G
    and C<->T.
    """
    kappa, pi = _broadcast_params(kappa, pi)
    one = torch.ones_like(kappa[..., 0])
    k = kappa[..., 0]
    z = torch.zeros_like(k)
    rows = [
        [z, one, k, one],
        [one, z, one, k],
        [k, one, z, one],
        [one, k, one, z],
    ]
    exch = torch.stack([torch.stack(r, -1) for r in rows], -2)
    return _assemble_q(exch, pi)


def q_gtr(rates: torch.Tensor, pi: torch.Tensor) -> torch.Tensor:
    """GTR rate matrix (evolution/substitution_model/nucleotide.py:328-374).

    ``rates [...,6]`` in the order AC, AG, AT, CG, CT, GT (upper triangle,
    row-major); ``pi [...,4]``.
    """
    rates, pi = _broadcast_params(rates, pi)
    return q_general_symmetric(rates, pi, 4)


def q_general_symmetric(rates: torch.Tensor, pi: torch.Tensor, state_count: int,
                        mapping: torch.Tensor | None = None) -> torch.Tensor:
    """Symmetric M-state rate matrix (evolution/substitution_model/general.py:267-281).

    The upper triangle (row-major) takes ``rates[mapping[:M(M-1)/2]]`` and the
    lower triangle, visited in the same row-major order of the transposed
    indices, takes ``rates[mapping[M(M-1)/2:]]``.  With ``mapping=None`` both
    halves use ``arange(M(M-1)/2)``, i.e. a symmetric exchangeability matrix.
    """
    m = state_count
    iu = torch.triu_indices(m, m, 1)
    half = iu.shape[1]
    if mapping is None:
        up = torch.arange(half)
        lo = up
    else:
        up = mapping[:half]
        lo = mapping[half:]
    exch = torch.zeros(rates.shape[:-1] + (m, m), dtype=rates.dtype)
    exch[..., iu[0], iu[1]] = rates[..., up]
    exch[..., iu[1], iu[0]] = rates[..., lo]
    pi = pi.expand(rates.shape[:-1] + (m,))
    return _assemble_q(exch, pi)


def _stop_codon_free_triplets(table: str):
    bases = "ACGT"
    trip = ["".join(t) for t in itertools.product(bases, repeat=3)]
    coding = [i for i, aa in enumerate(table[:64]) if aa != "*"]
    return [trip[i] for i in coding], [table[i] for i in coding]


def mg94_masks(table: str):
    """Masks of MG94 over the upper-triangle codon pairs (codon.py:33-55).

    Returns float64 arrays (transitions, synonymous, non_synonymous) of length
    M(M-1)/2 over ``itertools.combinations`` order of the sense codons.  Pairs
    that differ at more than one position set no mask.
    """
    trip, aa = _stop_codon_free_triplets(table)
    m = len(trip)
    n = m * (m - 1) // 2
    ts = np.zeros(n)
    syn = np.zeros(n)
    nonsyn = np.zeros(n)
    for idx, (i, j) in enumerate(itertools.combinations(range(m), 2)):
        c1, c2 = trip[i], trip[j]
        diffs = [p for p in range(3) if c1[p] != c2[p]]
        if len(diffs) != 1:
            continue
        p = diffs[0]
        if {c1[p], c2[p]} in ({"A", "G"}, {"C", "T"}):
            ts[idx] = 1.0
        if aa[i] == aa[j]:
            syn[idx] = 1.0
        else:
            nonsyn[idx] = 1.0
    return ts, syn, nonsyn


UNIVERSAL_CODE = "KNKNTTTTRSRSIIMIQHQHPPPPRRRRLLLLEDEDAAAAGGGGVVVV*Y*YSSSS*CWCLFLF"


def q_mg94(alpha, beta, kappa, pi, table: str = UNIVERSAL_CODE) -> torch.Tensor:
    """MG94 codon rate matrix as torchtree computes it (codon.py:57-77).

    Off-diagonal exchangeability = kappa^ts * alpha^syn * beta^nonsyn over the
    pair masks; a pair differing at two or three positions sets no mask and
    therefore gets exchangeability 1 (this is what the reference computes).
    """
    ts, syn, nonsyn = (torch.tensor(a) for a in mg94_masks(table))
    kappa, alpha, beta = torch.broadcast_tensors(kappa, alpha, beta)
    one = torch.ones_like(kappa)
    off = (torch.where(ts == 1.0, kappa, one) * torch.where(syn == 1.0, alpha, one)
           * torch.where(nonsyn == 1.0, beta, one))
    m = pi.shape[-1]
    return q_general_symmetric(off, pi, m)


def _broadcast_params(a: torch.Tensor, pi: torch.Tensor):
    batch = torch.broadcast_shapes(a.shape[:-1], pi.shape[:-1])
    return a.expand(batch + a.shape[-1:]), pi.expand(batch + pi.shape[-1:])


# --------------------------------------------------------------------------
# Transition matrices
# --------------------------------------------------------------------------


def normalise_q(q: torch.Tensor, pi: torch.Tensor) -> torch.Tensor:
    """Q / (-sum_i pi_i Q_ii) (evolution/substitution_model/abstract.py:49-50, 59)."""
    mu = -(torch.diagonal(q, dim1=-2, dim2=-1) * pi).sum(-1)
    return q / mu[..., None, None]


def eigen_symmetric(q_unnorm: torch.Tensor, pi: torch.Tensor):
    """Eigen system of the normalised Q via its symmetrised form.

    Restates evolution/substitution_model/abstract.py:57-66: with
    A = Pi^1/2 Q Pi^-1/2 = V diag(lambda) V^T,
    Q = (Pi^-1/2 V) diag(lambda) (V^-1 Pi^1/2).
    Returns ``(lambda [...,S], U = Pi^-1/2 V, U_inv = V^-1 Pi^1/2)``.
    The reference inverts V with ``inverse()``; this restatement does the same.
    """
    q = normalise_q(q_unnorm, pi)
    sp = pi.sqrt()
    a = sp[..., :, None] * q / sp[..., None, :]
    lam, v = torch.linalg.eigh(a)
    u = v / sp[..., :, None]
    u_inv = torch.linalg.inv(v) * sp[..., None, :]
    return lam, u, u_inv


def p_t_from_eigen(lam, u, u_inv, times: torch.Tensor) -> torch.Tensor:
    """P(t) = U diag(exp(lambda t)) U^-1 for every entry of ``times``.

    ``lam [*b,S]``, ``u``/``u_inv`` ``[*b,S,S]``, ``times [*b,...]`` ->
    ``[*b,...,S,S]`` (abstract.py:67-76).
    """
    extra = times.dim() - lam.dim() + 1
    shape_l = lam.shape[:-1] + (1,) * extra + lam.shape[-1:]
    shape_m = u.shape[:-2] + (1,) * extra + u.shape[-2:]
    e = torch.exp(lam.reshape(shape_l) * times.unsqueeze(-1))
    return (u.reshape(shape_m) * e.unsqueeze(-2)) @ u_inv.reshape(shape_m)


def p_t_symmetric(q_unnorm, pi, times):
    """Reversible-model P(t) (abstract.py:57-76)."""
    lam, u, u_inv = eigen_symmetric(q_unnorm, pi)
    return p_t_from_eigen(lam, u, u_inv, times)


# --------------------------------------------------------------------------
# Site models
# --------------------------------------------------------------------------


def _discretised(inverse_cdf, param, categories, invariant=None, mu=None):
    """Mean-one discretisation (evolution/site_model.py:173-195).

    Quantiles (2i+1)/(2K); with a proportion of invariant sites an extra
    zero-rate category is prepended with probability ``invariant``.
    """
    k = categories
    q = (2.0 * torch.arange(k, dtype=param.dtype) + 1.0) / (2.0 * k)
    rates = inverse_cdf(param, q)
    if invariant is not None:
        probs = torch.cat((invariant, ((1.0 - invariant) / k).expand(invariant.shape[:-1] + (k,))), -1)
        rates = torch.cat((torch.zeros_like(invariant), rates.expand(invariant.shape[:-1] + (k,))), -1)
    else:
        probs = torch.full((k,), 1.0 / k, dtype=param.dtype)
    rates = rates / (rates * probs).sum(-1, keepdim=True)
    if mu is not None:
        rates = rates * mu
    return rates, probs


def weibull_rates(shape, categories, invariant=None, mu=None):
    """Discretised Weibull rates (site_model.py:237-247, 173-195).

    ``shape [...,1]`` -> ``(rates [...,K'], probabilities [...,K'])``.
    """
    return _discretised(lambda s, q: torch.pow(-torch.log(1.0 - q), 1.0 / s),
                        shape, categories, invariant, mu)


def gamma_rates(shape, categories, invariant=None, mu=None):
    """Discretised Gamma(shape, rate=shape) quantile rates.

    NOT IN THE REFERENCE (torchtree 1.0.2 has no Gamma site model): same
    quantiles and mean-one normalisation as ``weibull_rates``; the quantile
    function is scipy's ``gammaincinv``.  Values only (no autograd).
    """
    from scipy.special import gammaincinv

    def icdf(s, q):
        s_np = s.detach().numpy()
        out = gammaincinv(s_np, q.numpy()) / s_np
        return torch.tensor(out, dtype=s.dtype)

    return _discretised(icdf, shape, categories, invariant, mu)


# --------------------------------------------------------------------------
# Pruning (evolution/tree_likelihood.py)
# --------------------------------------------------------------------------


def _root_site_likelihood(root_partial, freqs, props):
    """freqs @ sum_k props_k * partial_k  ->  [*b,1,N]  (tree_likelihood.py:72-75)."""
    mixed = (props * root_partial).sum(-3)
    return freqs @ mixed


def treelikelihood(partials, weights, post_indexing, mats, freqs):
    """Single-category pruning (tree_likelihood.py:14-37).

    ``partials``: list of T tip tensors ``[S,N]`` followed by T-1 slots;
    ``mats [...,B,S,S]``; ``freqs [...,1,S]`` -> lnL ``[...,1]``.
    """
    parts = list(partials)
    for node, left, right in post_indexing:
        a = mats[..., left, :, :] @ parts[left]
        b = mats[..., right, :, :] @ parts[right]
        parts[node] = a * b
    root = parts[post_indexing[-1][0]]
    return (torch.log(freqs @ root) * weights).sum(-1)


def treelikelihood_discrete(partials, weights, post_indexing, mats, freqs, props):
    """K-category pruning without rescaling (tree_likelihood.py:40-75)."""
    parts = list(partials)
    for node, left, right in post_indexing:
        parts[node] = (mats[..., left, :, :, :] @ parts[left]) * (
            mats[..., right, :, :, :] @ parts[right])
    site = _root_site_likelihood(parts[post_indexing[-1][0]], freqs, props)
    return (torch.log(site) * weights).sum(-1)


def _tip_state_columns(mats, tip_count):
    """P columns for tip codes plus an all-ones column for code S (tree_likelihood.py:103-112)."""
    tips = mats[..., :tip_count, :, :, :]
    ones = torch.ones(tips.shape[:-1] + (1,), dtype=mats.dtype)
    return torch.cat((tips, ones), -1)


def _child_term(mats, mat_tips, partials, idx, tip_count):
    if idx < tip_count:
        return mat_tips[..., idx, :, :, partials[idx]]
    return mats[..., idx, :, :, :] @ partials[idx]


def treelikelihood_tip_states_discrete(partials, weights, post_indexing, mats, freqs, props):
    """Tip-state-code pruning without rescaling (tree_likelihood.py:78-131).

    Tip entries of ``partials`` are int64 codes ``[N]`` in ``[0, S]``.
    """
    tip_count = len(post_indexing) + 1
    mat_tips = _tip_state_columns(mats, tip_count)
    parts = list(partials)
    for node, left, right in post_indexing:
        parts[node] = (_child_term(mats, mat_tips, parts, left, tip_count)
                       * _child_term(mats, mat_tips, parts, right, tip_count))
    site = _root_site_likelihood(parts[post_indexing[-1][0]], freqs, props)
    return (torch.log(site) * weights).sum(-1)


def _scale(partial):
    """Per-pattern max over the K*S entries (tree_likelihood.py:209-212)."""
    flat = partial.reshape(partial.shape[:-3] + (-1,) + partial.shape[-1:])
    scaler = flat.max(-2, keepdim=True)[0]
    return partial / scaler.unsqueeze(-2), scaler


def _rescaled_total(root, scalers, freqs, props, weights):
    site = _root_site_likelihood(root, freqs, props)
    log_scale = torch.cat(scalers, -2).log().sum(-2).unsqueeze(-2)
    return ((torch.log(site) + log_scale) * weights).sum(-1)


def treelikelihood_discrete_rescaled(partials, weights, post_indexing, mats, freqs, props):
    """Pruning with per-node rescaling (tree_likelihood.py:186-221)."""
    parts = list(partials)
    scalers = []
    for node, left, right in post_indexing:
        prod = (mats[..., left, :, :, :] @ parts[left]) * (
            mats[..., right, :, :, :] @ parts[right])
        parts[node], s = _scale(prod)
        scalers.append(s)
    return _rescaled_total(parts[post_indexing[-1][0]], scalers, freqs, props, weights)


def treelikelihood_tip_states_discrete_rescaled(partials, weights, post_indexing, mats, freqs, props):
    """Tip-state-code pruning with rescaling (tree_likelihood.py:224-278)."""
    tip_count = len(post_indexing) + 1
    mat_tips = _tip_state_columns(mats, tip_count)
    parts = list(partials)
    scalers = []
    for node, left, right in post_indexing:
        prod = (_child_term(mats, mat_tips, parts, left, tip_count)
                * _child_term(mats, mat_tips, parts, right, tip_count))
        parts[node], s = _scale(prod)
        scalers.append(s)
    return _rescaled_total(parts[post_indexing[-1][0]], scalers, freqs, props, weights)


def treelikelihood_discrete_safe(partials, weights, post_indexing, mats, freqs, props, threshold):
    """Selective rescaling after a first underflow (tree_likelihood.py:134-183).

    A node is recomputed and rescaled when a child was rescaled or when its
    stored partial (from the failed unscaled pass) has a per-pattern max over
    states below ``threshold`` in some category/pattern.  ``partials`` must
    hold the previous (unscaled) pass's internal partials.
    """
    parts = list(partials)
    scalers = []
    rescaled = [False] * (post_indexing[-1][0] + 1)
    for node, left, right in post_indexing:
        below = torch.any(parts[node].max(-2, keepdim=True)[0] < threshold)
        if rescaled[left] or rescaled[right] or below:
            prod = (mats[..., left, :, :, :] @ parts[left]) * (
                mats[..., right, :, :, :] @ parts[right])
            parts[node], s = _scale(prod)
            scalers.append(s)
            rescaled[node] = True
    return _rescaled_total(parts[post_indexing[-1][0]], scalers, freqs, props, weights)


def unscaled_then_safe(partials, weights, post_indexing, mats, freqs, props, threshold):
    """The model-level switch (tree_likelihood.py:358-389).

    Runs the unscaled recursion; when any lnL is -inf, runs the selective
    rescaling on the partials the failed pass left behind.  Returns
    ``(lnL, rescaled_flag)``.
    """
    parts = list(partials)
    for node, left, right in post_indexing:
        parts[node] = (mats[..., left, :, :, :] @ parts[left]) * (
            mats[..., right, :, :, :] @ parts[right])
    site = _root_site_likelihood(parts[post_indexing[-1][0]], freqs, props)
    lnl = (torch.log(site) * weights).sum(-1)
    if torch.any(torch.isinf(lnl)):
        return treelikelihood_discrete_safe(parts, weights, post_indexing, mats, freqs, props,
                                            threshold), True
    return lnl, False


# --------------------------------------------------------------------------
# Model-level glue (TreeLikelihoodModel._call, tree_likelihood.py:313-356)
# --------------------------------------------------------------------------


def model_branch_lengths(branch_lengths, clock_rates=None):
    """Per-node branch lengths fed to P(t) (tree_likelihood.py:323-344).

    Without a clock model an unrooted tree's ``[*b, 2T-3]`` parameter gets a
    trailing zero (node 2T-3 hangs from the root by a zero-length branch).
    With a clock the ``[*b, 2T-2]`` time lengths are multiplied by the
    per-branch rates.
    """
    if clock_rates is None:
        zero = torch.zeros(branch_lengths.shape[:-1] + (1,), dtype=branch_lengths.dtype)
        return torch.cat((branch_lengths, zero), -1)
    return clock_rates * branch_lengths


def model_loglik(tips, weights, post_indexing, bls, lam, u, u_inv, rates, props, freqs,
                 rescale=False, tip_states=False):
    """lnL ``[b,1]`` from per-node branch lengths and an eigen system.

    ``bls [b,B]``, ``lam [b,S]``, ``u``/``u_inv`` ``[b,S,S]``, ``rates [b,K]``,
    ``props [b,K]``, ``freqs [b,S]``; mirrors ``_call`` from the P(t) call on
    (tree_likelihood.py:346-356).
    """
    mats = p_t_from_eigen(lam, u, u_inv, bls.unsqueeze(-1) * rates.unsqueeze(-2))
    f = freqs.unsqueeze(-2)
    p = props.unsqueeze(-1).unsqueeze(-1)
    parts = list(tips) + [None] * (len(tips) - 1)
    if tip_states:
        fn = (treelikelihood_tip_states_discrete_rescaled if rescale
              else treelikelihood_tip_states_discrete)
    else:
        fn = treelikelihood_discrete_rescaled if rescale else treelikelihood_discrete
    return fn(parts, weights, post_indexing, mats, f, p)


def site_log_likelihoods(tips, post_indexing, mats, freqs, props):
    """Per-pattern log site likelihood ``[*b,N]`` with rescaling (oracle helper)."""
    parts = list(tips) + [None] * (len(tips) - 1)
    scalers = []
    for node, left, right in post_indexing:
        prod = (mats[..., left, :, :, :] @ parts[left]) * (
            mats[..., right, :, :, :] @ parts[right])
        parts[node], s = _scale(prod)
        scalers.append(s)
    site = _root_site_likelihood(parts[post_indexing[-1][0]], freqs, props)
    log_scale = torch.cat(scalers, -2).log().sum(-2).unsqueeze(-2)
    return (torch.log(site) + log_scale).squeeze(-2)


def finite_difference(fn, x: torch.Tensor, h: float = 1e-6) -> torch.Tensor:
    """Central differences of a scalar ``fn`` at every entry of ``x`` (FP64)."""
    x = x.detach().clone()
    g = torch.empty_like(x)
    flat = x.view(-1)
    gf = g.view(-1)
    for i in range(flat.numel()):
        old = flat[i].item()
        step = h * max(1.0, abs(old))
        flat[i] = old + step
        fp = float(fn(x))
        flat[i] = old - step
        fm = float(fn(x))
        flat[i] = old
        gf[i] = (fp - fm) / (2 * step)
    return g


__all__ = [name for name in dir() if not name.startswith("_") and name not in ("math", "np", "torch", "itertools")]
