"""Seeded synthetic phylogenetic workloads (inputs only).

Yule topologies, branch lengths, model parameters, and alignments simulated
along the tree.  Every draw comes from one ``numpy.random.Generator`` seeded
by the caller; parameterisations are stated in each docstring.  These
stand in for the influenza datasets of the published torchtree benchmark,
which are not available.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import scipy.linalg

from .tree import Topology


def yule_topology(tip_count: int, rng: np.random.Generator) -> Topology:
    """Random Yule (pure-birth) rooted binary topology.

    Starting from a root with two lineages, a uniformly chosen lineage
    splits until there are ``tip_count``; tips get taxa ``t0..t{T-1}`` in a
    random order, internal nodes are numbered in post-order from T.
    """
    T = tip_count
    if T < 2:
        raise ValueError("need at least 2 tips")
    children = {0: [1, 2]}
    leaves = [1, 2]
    nxt = 3
    while len(leaves) < T:
        i = int(rng.integers(len(leaves)))
        v = leaves[i]
        children[v] = [nxt, nxt + 1]
        leaves[i] = nxt
        leaves.append(nxt + 1)
        nxt += 2
    perm = rng.permutation(T)
    tip_index = {leaf: int(perm[j]) for j, leaf in enumerate(leaves)}
    post = []
    index = {}
    counter = T
    stack = [(0, False)]
    while stack:
        v, seen = stack.pop()
        if v not in children:
            index[v] = tip_index[v]
            continue
        if seen:
            index[v] = counter
            counter += 1
            post.append((index[v], index[children[v][0]], index[children[v][1]]))
        else:
            stack.append((v, True))
            stack.append((children[v][1], False))
            stack.append((children[v][0], False))
    return Topology(post, [f"t{i}" for i in range(T)])


def exp_branch_lengths(count: int, mean: float, rng: np.random.Generator) -> np.ndarray:
    """``count`` i.i.d. Exponential lengths with the given mean."""
    return rng.exponential(mean, size=count)


def transition_matrices(q: np.ndarray, lengths: np.ndarray) -> np.ndarray:
    """``expm(Q t)`` for every length (simulation helper, FP64)."""
    return np.stack([scipy.linalg.expm(q * t) for t in lengths])


def simulate_alignment(topo: Topology, node_lengths: np.ndarray, q: np.ndarray, pi: np.ndarray,
                       rates: np.ndarray, probs: np.ndarray, site_count: int,
                       rng: np.random.Generator, alphabet: str = "ACGT") -> list:
    """Evolve ``site_count`` sites down the tree.

    ``node_lengths [2T-2]`` indexed by child node (zero allowed); each site
    draws a rate category from ``probs``; the root state is drawn from
    ``pi``.  Returns the tip sequences in taxa order.
    """
    T = topo.tip_count
    S = q.shape[0]
    cat = rng.choice(len(rates), size=site_count, p=probs)
    states = np.empty((2 * T - 1, site_count), dtype=np.int64)
    states[topo.root] = rng.choice(S, size=site_count, p=pi)
    kids = {int(v): (int(l), int(r)) for v, l, r in topo.postorder}
    order = [int(v) for v in topo.postorder[::-1, 0]]  # pre-order over internal nodes
    for v in order:
        for c in kids[v]:
            t = node_lengths[c]
            cum = np.cumsum(transition_matrices(q, rates * t), axis=-1)  # [K,S,S]
            rows = cum[cat, states[v]]  # [L, S]
            u = rng.random(site_count)[:, None]
            states[c] = np.minimum((u > rows).sum(-1), S - 1)
    letters = np.frombuffer(alphabet.encode(), dtype=np.uint8)
    return [letters[states[t]].tobytes().decode() for t in range(T)]


def normalised_q_np(q: np.ndarray, pi: np.ndarray) -> np.ndarray:
    return q / -(np.diag(q) * pi).sum()


def gtr_q_np(exch6: np.ndarray, pi: np.ndarray) -> np.ndarray:
    r = np.zeros((4, 4))
    r[np.triu_indices(4, 1)] = exch6
    r = r + r.T
    q = r * pi[None, :]
    np.fill_diagonal(q, -q.sum(1))
    return q


def general_q_np(exch: np.ndarray, pi: np.ndarray) -> np.ndarray:
    S = pi.shape[0]
    r = np.zeros((S, S))
    r[np.triu_indices(S, 1)] = exch
    r = r + r.T
    q = r * pi[None, :]
    np.fill_diagonal(q, -q.sum(1))
    return q


def discrete_gamma_np(shape: float, k: int) -> np.ndarray:
    from scipy.special import gammaincinv

    q = (2.0 * np.arange(k) + 1.0) / (2.0 * k)
    r = gammaincinv(shape, q) / shape
    return r / r.mean()


def discrete_weibull_np(shape: float, k: int) -> np.ndarray:
    q = (2.0 * np.arange(k) + 1.0) / (2.0 * k)
    r = np.power(-np.log(1.0 - q), 1.0 / shape)
    return r / r.mean()


@dataclass
class DnaWorkload:
    """A simulated data set plus per-sample likelihood inputs.

    ``branch_lengths [b, 2T-3]`` are the unrooted tree's free lengths
    (the engine appends the zero branch of node 2T-3); ``pi [b,S]``,
    ``shape [b,1]``; ``exch`` holds the model's rate parameters: GTR
    ``[b,6]`` exchangeabilities, HKY ``[b,6]`` with kappa at the transitions,
    general ``[b,S(S-1)/2]`` upper-triangle exchangeabilities, MG94 ``[b,2]``
    = (kappa, omega) with alpha = 1.
    """

    name: str
    seed: int
    topology: Topology
    sequences: list
    branch_lengths: np.ndarray
    exch: np.ndarray
    pi: np.ndarray
    shape: np.ndarray
    categories: int
    site_model: str  # "weibull" | "gamma"
    model: str       # "gtr" | "hky" | "general" | "mg94"
    data_type: str = "nucleotide"  # "nucleotide" | "amino_acid" | "codon"

    @property
    def state_count(self) -> int:
        return self.pi.shape[-1]


def dna_workload(name: str, tip_count: int, site_count: int, batch: int, seed: int,
                 model: str = "gtr", site_model: str = "weibull", shape: float = 0.5,
                 categories: int = 4, branch_mean: float = 0.01, kappa_lognormal=(1.0, 0.5),
                 branch_jitter: float = 0.1) -> DnaWorkload:
    """Simulate one DNA workload.

    Topology: Yule.  Branches: Exponential(mean ``branch_mean``) for the
    2T-3 unrooted lengths.  GTR: exchangeabilities ~ Dirichlet(1^6),
    frequencies ~ Dirichlet(1^4).  HKY: kappa ~ LogNormal(mu, sigma) (log
    scale), frequencies ~ Dirichlet(1^4).  The alignment is simulated with
    sample 0's parameters; samples 1..b-1 multiply every branch by
    LogNormal(0, ``branch_jitter``).
    """
    rng = np.random.default_rng(seed)
    topo = yule_topology(tip_count, rng)
    B = 2 * tip_count - 2
    bl0 = exp_branch_lengths(B - 1, branch_mean, rng)
    pi = rng.dirichlet(np.ones(4))
    if model == "gtr":
        exch = rng.dirichlet(np.ones(6))
    elif model == "hky":
        kappa = rng.lognormal(kappa_lognormal[0], kappa_lognormal[1])
        exch = np.array([1.0, kappa, 1.0, 1.0, kappa, 1.0])
    else:
        raise ValueError(model)
    rates = discrete_weibull_np(shape, categories) if site_model == "weibull" else \
        discrete_gamma_np(shape, categories)
    probs = np.full(categories, 1.0 / categories)
    q = normalised_q_np(gtr_q_np(exch, pi), pi)
    node_lengths = np.concatenate([bl0, [0.0]])
    seqs = simulate_alignment(topo, node_lengths, q, pi, rates, probs, site_count, rng)
    jitter = np.ones((batch, B - 1))
    if batch > 1:
        jitter[1:] = rng.lognormal(0.0, branch_jitter, size=(batch - 1, B - 1))
    return DnaWorkload(name=name, seed=seed, topology=topo, sequences=seqs,
                       branch_lengths=bl0[None, :] * jitter,
                       exch=np.repeat(exch[None, :], batch, 0), pi=np.repeat(pi[None, :], batch, 0),
                       shape=np.full((batch, 1), shape), categories=categories,
                       site_model=site_model, model=model)


AMINO_ACIDS = "ACDEFGHIKLMNPQRSTVWY"


def protein_workload(name: str, tip_count: int, site_count: int, batch: int, seed: int,
                     site_model: str = "gamma", shape: float = 0.5, categories: int = 4,
                     branch_mean: float = 0.05, branch_jitter: float = 0.1) -> DnaWorkload:
    """20-state amino-acid workload: exchangeabilities ~ Gamma(shape 1, scale 1)
    (190, upper triangle row-major), frequencies ~ Dirichlet(1^20), Yule tree,
    Exponential(mean ``branch_mean``) branches."""
    rng = np.random.default_rng(seed)
    topo = yule_topology(tip_count, rng)
    B = 2 * tip_count - 2
    bl0 = exp_branch_lengths(B - 1, branch_mean, rng)
    exch = rng.gamma(1.0, 1.0, 190)
    pi = rng.dirichlet(np.ones(20))
    rates = discrete_weibull_np(shape, categories) if site_model == "weibull" else \
        discrete_gamma_np(shape, categories)
    q = normalised_q_np(general_q_np(exch, pi), pi)
    seqs = simulate_alignment(topo, np.concatenate([bl0, [0.0]]), q, pi, rates, np.full(categories, 1.0 / categories),
                              site_count, rng, alphabet=AMINO_ACIDS)
    jitter = np.ones((batch, B - 1))
    if batch > 1:
        jitter[1:] = rng.lognormal(0.0, branch_jitter, size=(batch - 1, B - 1))
    return DnaWorkload(name=name, seed=seed, topology=topo, sequences=seqs, branch_lengths=bl0[None, :] * jitter,
                       exch=np.repeat(exch[None, :], batch, 0), pi=np.repeat(pi[None, :], batch, 0),
                       shape=np.full((batch, 1), shape), categories=categories, site_model=site_model,
                       model="general", data_type="amino_acid")


def sense_codons(table: str = "KNKNTTTTRSRSIIMIQHQHPPPPRRRRLLLLEDEDAAAAGGGGVVVV*Y*YSSSS*CWCLFLF"):
    trip = ["".join(t) for t in __import__("itertools").product("ACGT", repeat=3)]
    return [t for t, a in zip(trip, table) if a != "*"]


def f3x4_np(pos_freqs: np.ndarray) -> np.ndarray:
    """Codon frequencies from per-position nucleotide frequencies [3,4] (sense codons, normalised)."""
    idx = {"A": 0, "C": 1, "G": 2, "T": 3}
    f = np.array([np.prod([pos_freqs[p, idx[c[p]]] for p in range(3)]) for c in sense_codons()])
    return f / f.sum()


def mg94_q_np(kappa: float, omega: float, pi: np.ndarray) -> np.ndarray:
    import torch

    from .substitution import mg94_q

    q = mg94_q(torch.tensor(1.0, dtype=torch.float64), torch.tensor(omega, dtype=torch.float64),
               torch.tensor(kappa, dtype=torch.float64), torch.tensor(pi, dtype=torch.float64))
    return q.numpy()


def codon_workload(name: str, tip_count: int, site_count: int, batch: int, seed: int,
                   site_model: str = "gamma", shape: float = 0.5, categories: int = 4,
                   branch_mean: float = 0.05, branch_jitter: float = 0.1) -> DnaWorkload:
    """61-state codon workload (MG94 with alpha = 1, beta = omega): omega ~
    Gamma(shape 2, scale 0.25), kappa ~ LogNormal(1, 0.5) (log scale), F3x4
    frequencies from per-position Dirichlet(1^4); ``site_count`` codons."""
    rng = np.random.default_rng(seed)
    topo = yule_topology(tip_count, rng)
    B = 2 * tip_count - 2
    bl0 = exp_branch_lengths(B - 1, branch_mean, rng)
    omega = rng.gamma(2.0, 0.25)
    kappa = rng.lognormal(1.0, 0.5)
    pi = f3x4_np(rng.dirichlet(np.ones(4), size=3))
    rates = discrete_weibull_np(shape, categories) if site_model == "weibull" else \
        discrete_gamma_np(shape, categories)
    q = normalised_q_np(mg94_q_np(kappa, omega, pi), pi)
    letters = "".join(chr(48 + i) for i in range(61))
    states = simulate_alignment(topo, np.concatenate([bl0, [0.0]]), q, pi, rates,
                                np.full(categories, 1.0 / categories), site_count, rng, alphabet=letters)
    codons = sense_codons()
    seqs = ["".join(codons[ord(ch) - 48] for ch in s) for s in states]
    jitter = np.ones((batch, B - 1))
    if batch > 1:
        jitter[1:] = rng.lognormal(0.0, branch_jitter, size=(batch - 1, B - 1))
    return DnaWorkload(name=name, seed=seed, topology=topo, sequences=seqs, branch_lengths=bl0[None, :] * jitter,
                       exch=np.repeat(np.array([[kappa, omega]]), batch, 0), pi=np.repeat(pi[None, :], batch, 0),
                       shape=np.full((batch, 1), shape), categories=categories, site_model=site_model,
                       model="mg94", data_type="codon")


# The workloads of the benchmark configurations (sizes and distributions
# as stated there).
CONFIGS = {
    "gtr_w4_t69": dict(tip_count=69, site_count=1701, batch=1, seed=1, model="gtr",
                       site_model="weibull", shape=0.5),
    "hky_g4_t500_b64": dict(tip_count=500, site_count=10000, batch=64, seed=2, model="hky",
                            site_model="gamma", shape=0.3),
    "gtr_g4_t1000_b8": dict(tip_count=1000, site_count=100000, batch=8, seed=3, model="gtr",
                            site_model="gamma", shape=0.5),
}


WIDE_CONFIGS = {
    "codon_g4_t200_b16": (codon_workload, dict(tip_count=200, site_count=3000, batch=16, seed=4,
                                               site_model="gamma", shape=0.5)),
    "protein_g4_t200_b4": (protein_workload, dict(tip_count=200, site_count=5000, batch=4, seed=5,
                                                  site_model="gamma", shape=0.5)),
}


def named_workload(name: str, **overrides) -> DnaWorkload:
    if name in WIDE_CONFIGS:
        fn, kw = WIDE_CONFIGS[name]
        kw = dict(kw)
        kw.update(overrides)
        return fn(name, **kw)
    kw = dict(CONFIGS[name])
    kw.update(overrides)
    return dna_workload(name, **kw)
