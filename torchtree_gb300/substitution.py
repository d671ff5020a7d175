"""Rate matrices and their eigen systems (host side, FP64, differentiable).

The pruning engine consumes ``(lambda, U, W)`` with
``Q = U diag(lambda) W`` for the normalised rate matrix, exactly the
factorisation of torchtree's ``SymmetricSubstitutionModel.p_t``
(torchtree/evolution/substitution_model/abstract.py:57-76): symmetrise with
Pi^1/2, ``eigh``, ``U = Pi^-1/2 V``, ``W = V^-1 Pi^1/2``.  The rate-matrix
builders stay in torch so that autograd carries the engine's gradients back
to exchangeabilities and frequencies.  The eigendecomposition of device
tensors runs in the engine's eigensolver (``tt_reversible_eigen``)
whenever no gradient has to flow through it, as in the rate-matrix route,
whose backward needs no eigenvector derivative; otherwise ``torch.linalg.eigh``
keeps the autograd graph.
"""
from __future__ import annotations

import itertools

import torch


def normalise(q: torch.Tensor, pi: torch.Tensor) -> torch.Tensor:
    """Q / (-sum_i pi_i Q_ii)  (abstract.py:49-50)."""
    mu = -(torch.diagonal(q, dim1=-2, dim2=-1) * pi).sum(-1)
    return q / mu[..., None, None]


def eigen_system(q_unnorm: torch.Tensor, pi: torch.Tensor):
    """``(lambda [...,S], U [...,S,S], W [...,S,S])`` of the normalised Q."""
    return eigen_of_normalised(normalise(q_unnorm, pi), pi)


def device_eigen(q: torch.Tensor, pi: torch.Tensor):
    """``(lambda, U, W)`` of normalised reversible ``q [b,S,S]`` (CUDA, FP64)
    by the engine's eigensolver (``tt_reversible_eigen``: FP32 Jacobi, FP64
    refinement of the eigenvectors); no autograd graph."""
    from . import _native

    lib = _native.load()
    q = q.detach().to(torch.float64).contiguous()
    pi = pi.detach().to(torch.float64).expand(q.shape[:-1]).contiguous()
    b, S = q.shape[0], q.shape[-1]
    lam = torch.empty(b, S, dtype=torch.float64, device=q.device)
    u = torch.empty(b, S, S, dtype=torch.float64, device=q.device)
    w = torch.empty_like(u)
    status = torch.zeros(1, dtype=torch.int32, device=q.device)
    with torch.cuda.device(q.device):
        stream = torch.cuda.current_stream(q.device).cuda_stream
        _native.check(lib.tt_reversible_eigen(b, S, _native.ptr(q), _native.ptr(pi), _native.ptr(lam),
                                              _native.ptr(u), _native.ptr(w), _native.ptr(status),
                                              _native.ptr_value(stream)))
    return lam, u, w


def eigen_of_normalised(q: torch.Tensor, pi: torch.Tensor):
    """Eigen system of an already normalised reversible Q with stationary ``pi``."""
    needs_graph = torch.is_grad_enabled() and (q.requires_grad or pi.requires_grad)
    if q.is_cuda and not needs_graph:
        lead = q.shape[:-2]
        S = q.shape[-1]
        lam, u, w = device_eigen(q.reshape(-1, S, S), pi.expand(lead + (S,)).reshape(-1, S))
        return lam.reshape(lead + (S,)), u.reshape(lead + (S, S)), w.reshape(lead + (S, S))
    sp = pi.sqrt()
    a = sp.unsqueeze(-1) * q / sp.unsqueeze(-2)
    lam, v = torch.linalg.eigh(a)
    u = v / sp.unsqueeze(-1)
    w = torch.linalg.inv(v) * sp.unsqueeze(-2)
    return lam, u, w


def exchangeability_q(exch: torch.Tensor, pi: torch.Tensor) -> torch.Tensor:
    """Q_ij = R_ij pi_j, rows summing to zero; ``exch`` symmetric, zero diagonal."""
    q = exch * pi.unsqueeze(-2)
    return q - torch.diag_embed(q.sum(-1))


def symmetric_from_upper(rates: torch.Tensor, state_count: int) -> torch.Tensor:
    """Symmetric matrix from its upper triangle in row-major order."""
    iu = torch.triu_indices(state_count, state_count, 1, device=rates.device)
    r = torch.zeros(rates.shape[:-1] + (state_count, state_count), dtype=rates.dtype, device=rates.device)
    r[..., iu[0], iu[1]] = rates
    return r + r.transpose(-1, -2)


def gtr_q(rates: torch.Tensor, pi: torch.Tensor) -> torch.Tensor:
    """GTR (torchtree/evolution/substitution_model/nucleotide.py:328-374).

    ``rates [...,6]`` ordered AC, AG, AT, CG, CT, GT; ``pi [...,4]``.
    """
    batch = torch.broadcast_shapes(rates.shape[:-1], pi.shape[:-1])
    rates = rates.expand(batch + (6,))
    pi = pi.expand(batch + (4,))
    return exchangeability_q(symmetric_from_upper(rates, 4), pi)


def hky_q(kappa: torch.Tensor, pi: torch.Tensor) -> torch.Tensor:
    """HKY (nucleotide.py:238-264): transitions A<->G, C<->T scaled by kappa."""
    batch = torch.broadcast_shapes(kappa.shape[:-1], pi.shape[:-1])
    kappa = kappa.expand(batch + (1,))
    one = torch.ones_like(kappa)
    # upper triangle AC, AG, AT, CG, CT, GT
    rates = torch.cat([one, kappa, one, one, kappa, one], -1)
    return gtr_q(rates, pi)


def general_symmetric_q(rates: torch.Tensor, pi: torch.Tensor, state_count: int) -> torch.Tensor:
    """M-state symmetric model from its M(M-1)/2 exchangeabilities (general.py:267-281)."""
    batch = torch.broadcast_shapes(rates.shape[:-1], pi.shape[:-1])
    rates = rates.expand(batch + rates.shape[-1:])
    pi = pi.expand(batch + (state_count,))
    return exchangeability_q(symmetric_from_upper(rates, state_count), pi)


UNIVERSAL_CODE = "KNKNTTTTRSRSIIMIQHQHPPPPRRRRLLLLEDEDAAAAGGGGVVVV*Y*YSSSS*CWCLFLF"


def codon_pair_masks(table: str = UNIVERSAL_CODE):
    """MG94 pair classes over sense-codon pairs in combinations order (codon.py:33-55)."""
    trip = ["".join(t) for t in itertools.product("ACGT", repeat=3)]
    sense = [i for i, a in enumerate(table[:64]) if a != "*"]
    m = len(sense)
    ts, syn, nonsyn = [], [], []
    for i, j in itertools.combinations(range(m), 2):
        c1, c2 = trip[sense[i]], trip[sense[j]]
        d = [p for p in range(3) if c1[p] != c2[p]]
        single = len(d) == 1
        p = d[0] if single else 0
        ts.append(single and {c1[p], c2[p]} in ({"A", "G"}, {"C", "T"}))
        same = table[sense[i]] == table[sense[j]]
        syn.append(single and same)
        nonsyn.append(single and not same)
    f = lambda x: torch.tensor(x, dtype=torch.bool)  # noqa: E731
    return f(ts), f(syn), f(nonsyn), m


def mg94_q(alpha, beta, kappa, pi, table: str = UNIVERSAL_CODE) -> torch.Tensor:
    """MG94 as torchtree computes it (codon.py:57-77): exchangeability
    kappa^ts alpha^syn beta^nonsyn; pairs differing at 2-3 positions get 1."""
    ts, syn, nonsyn, m = codon_pair_masks(table)
    dev = pi.device
    ts, syn, nonsyn = ts.to(dev), syn.to(dev), nonsyn.to(dev)
    kappa, alpha, beta = torch.broadcast_tensors(kappa, alpha, beta)
    one = torch.ones_like(kappa)
    off = torch.where(ts, kappa, one) * torch.where(syn, alpha, one) * torch.where(nonsyn, beta, one)
    return general_symmetric_q(off, pi, m)
