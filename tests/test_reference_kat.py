"""torchtree's own known answer on its bundled influenza A data, where the
reference source tree is present (it is not copied into this repository).

test/test_tree_likelihood.py:268-342 builds a time tree from fluA.tree with
tip dates parsed from the taxon names and internal heights from the Newick
branch lengths (keep_branch_lengths: the ratios are the inverse
GeneralNodeHeightTransform of those heights), a strict clock of 0.001, JC69
and a 4-category Weibull site model of shape 0.1, and asserts
lnL = -4618.2062529058 with and without rescaling.  Here the same chain runs
through this package's Newick parser, tip-date heights and pattern
compression and the oracle's ratio transform and pruning, which pins the
oracle's time-tree, clock and Weibull chain to the reference's own number.
The data come from the reference source tree where it is present
(``tests/reference_models.py``) and otherwise from ``tests/golden/flua.json``,
which ``tests/golden/make_flua.py`` wrote from that source tree: the names,
the Newick tree and the alignment as compressed by torchtree's own
``compress_alignment``; its columns, each repeated by its weight, make an
alignment with the same site patterns and weights.
"""
import numpy as np
import pytest
import torch

from tests.conftest import GOLDEN
from tests.reference_models import DATA, fixed_tree_class, import_torchtree

KAT = -4618.2062529058


def _fasta(path):
    names, seqs = [], []
    for line in path.read_text().splitlines():
        line = line.strip()
        if line.startswith(">"):
            names.append(line[1:].strip())
            seqs.append([])
        elif line:
            seqs[-1].append(line)
    return names, ["".join(s) for s in seqs]


def _flua():
    """(taxon names, sequences, Newick) of the reference's influenza A data."""
    if (DATA / "fluA.fa").exists():
        names, seqs = _fasta(DATA / "fluA.fa")
        return names, seqs, (DATA / "fluA.tree").read_text().strip()
    import json

    d = json.loads((GOLDEN / "flua.json").read_text())
    reps = np.asarray(d["weights"])
    seqs = ["".join(np.repeat(np.array(list(p)), reps)) for p in d["patterns"]]
    return d["names"], seqs, d["newick"]


def _sampling_times(names):
    """Leaf heights from the dates that end the taxon names (tree_model.py:363-378)."""
    dates = np.array([float(n.split("_")[-1]) for n in names])
    return dates if dates.min() == 0.0 else dates.max() - dates


def test_flu_a_time_tree_weibull_strict_clock_known_answer():
    from oracle import likelihood as OL
    from oracle import timetree as OT
    from torchtree_gb300 import patterns
    from torchtree_gb300.tree import Topology

    names, seqs, newick = _flua()
    topo = Topology.from_newick(newick, names)
    T = topo.tip_count
    assert T == 69
    times = _sampling_times(names)
    # keep_branch_lengths: the ratios given in the test are replaced by the
    # inverse transform of the heights that the Newick lengths imply
    # (tree_model.py:700-705, 110-122); the forward transform returns them
    ratios, heights = _ratios_from_newick(topo, times)
    internal, time_lengths, _ = OT.ratio_transform(topo.postorder_list(), times.tolist(), ratios)
    np.testing.assert_allclose(internal.numpy(), heights, rtol=1e-12)
    bls = OL.model_branch_lengths(time_lengths, torch.tensor(0.001, dtype=torch.float64))
    ca = patterns.compress(seqs)
    tips = [torch.tensor(t) for t in ca.tip_partials()]
    weights = torch.tensor(ca.weights, dtype=torch.float64)
    rates, props = OL.weibull_rates(torch.tensor([0.1], dtype=torch.float64), 4)
    mats = OL.p_t_jc69(bls.unsqueeze(-1) * rates)  # [B, K, 4, 4]
    freqs = torch.full((1, 4), 0.25, dtype=torch.float64)
    p = props.reshape(4, 1, 1)
    parts = tips + [None] * (T - 1)
    post = topo.postorder_list()
    plain = OL.treelikelihood_discrete(parts, weights, post, mats, freqs, p)
    scaled = OL.treelikelihood_discrete_rescaled(parts, weights, post, mats, freqs, p)
    # the reference asserts torch.allclose (rtol 1e-5); the value it prints has
    # 10 decimals, and the oracle lands 4e-11 from it
    assert abs(float(plain) - KAT) < 1e-9
    assert abs(float(scaled) - KAT) < 1e-9


def _ratios_from_newick(topo, times):
    """Ratios whose transform gives the Newick heights (tree_model.py:700-705)."""
    from oracle import timetree as OT
    from torchtree_gb300.tree import node_heights_from_lengths

    T = topo.tip_count
    heights = node_heights_from_lengths(topo, times, min_length=1e-6)
    lb = OT.lower_bounds(topo.postorder_list(), times.tolist())
    ratios = torch.zeros(T - 1, dtype=torch.float64)
    ratios[T - 2] = heights[2 * T - 2]
    for v in range(T, 2 * T - 2):
        ratios[v - T] = (heights[v] - lb[v - T]) / (heights[topo.parent[v]] - lb[v - T])
    return ratios, heights[T:]


@pytest.mark.gpu
def test_flu_a_known_answer_through_the_gpu_path():
    """The same known answer through the product path on the GPU: the ratio
    transform kernel gives the time lengths, the pruning kernels the lnL.
    FP64 unscaled and rescaled within 1e-12 relative; FP32 within 1e-6."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from torchtree_gb300 import patterns, site_models, substitution
    from torchtree_gb300.likelihood import PhyloLikelihood
    from torchtree_gb300.timetree import TimeTree
    from torchtree_gb300.tree import Topology

    names, seqs, newick = _flua()
    topo = Topology.from_newick(newick, names)
    times = _sampling_times(names)
    ratios, heights = _ratios_from_newick(topo, times)
    dev = torch.device("cuda")
    h, time_lengths, _ = TimeTree(topo.postorder, times).ratio_transform(ratios[None].to(dev))
    np.testing.assert_allclose(h[0].cpu().numpy(), heights, rtol=1e-12)
    ca = patterns.compress(seqs)
    pi = torch.full((1, 4), 0.25, dtype=torch.float64, device=dev)
    q = substitution.gtr_q(torch.ones(1, 6, dtype=torch.float64, device=dev), pi)  # JC69
    rates, props = site_models.weibull_rates(torch.tensor([[0.1]], dtype=torch.float64, device=dev), 4)
    clock = torch.tensor([[0.001]], dtype=torch.float64, device=dev)
    for precision, rescale, tol in (("f64", False, 1e-12), ("f64", True, 1e-12), ("f32", True, 1e-6)):
        lik = PhyloLikelihood(topo, ca, 4, 4, batch=1, precision=precision)
        lik.rescale = rescale
        lnl = float(lik(time_lengths, q, pi, rates, props.expand(1, 4), clock_rates=clock)[0])
        assert abs(lnl - KAT) < tol * abs(KAT), (precision, rescale, lnl)
    # batched x 3 (test_tree_likelihood.py:334-342): every member equals the single evaluation
    for rescale in (False, True):
        lik = PhyloLikelihood(topo, ca, 4, 4, batch=3, precision="f64")
        lik.rescale = rescale
        x3 = lambda t: t.expand(3, *t.shape[1:]).contiguous()  # noqa: E731
        lnl3 = lik(x3(time_lengths), x3(q), x3(pi), x3(rates), props.expand(3, 4).contiguous(),
                   clock_rates=x3(clock)).cpu().numpy()
        assert np.all(np.abs(lnl3 - KAT) < 1e-12 * abs(KAT)), (rescale, lnl3)
        assert lnl3[0] == lnl3[1] == lnl3[2]


def test_flu_a_gradients_of_the_oracle_chain_match_torchtree():
    """On the same influenza A data, torchtree's own TreeLikelihoodModel
    (strict clock, JC69, Weibull) and the oracle's pruning agree on lnL and on
    the autograd gradients with respect to the time lengths, the clock rate
    and the Weibull shape (1e-9)."""
    if not import_torchtree():
        pytest.skip("torchtree source not present")
    from torchtree import Parameter
    from torchtree.evolution.alignment import Alignment, Sequence
    from torchtree.evolution.branch_model import StrictClockModel
    from torchtree.evolution.datatype import NucleotideDataType
    from torchtree.evolution.site_model import WeibullSiteModel
    from torchtree.evolution.site_pattern import SitePattern
    from torchtree.evolution.substitution_model import JC69
    from torchtree.evolution.taxa import Taxa, Taxon
    from torchtree.evolution.tree_likelihood import TreeLikelihoodModel

    from oracle import likelihood as OL
    from oracle import timetree as OT
    from torchtree_gb300 import patterns
    from torchtree_gb300.tree import Topology

    names, seqs, newick = _flua()
    topo = Topology.from_newick(newick, names)
    times = _sampling_times(names)
    ratios, _ = _ratios_from_newick(topo, times)
    _, lengths, _ = OT.ratio_transform(topo.postorder_list(), times.tolist(), ratios)

    def leaves():
        return (lengths.detach().clone().requires_grad_(), torch.tensor([0.001], dtype=torch.float64,
                requires_grad=True), torch.tensor([0.1], dtype=torch.float64, requires_grad=True))

    t_ref, c_ref, s_ref = leaves()
    dtype = torch.get_default_dtype()
    torch.set_default_dtype(torch.float64)  # the reference builds its tip partials in the default dtype
    try:
        taxa = Taxa(None, [Taxon(n, {}) for n in names])
        aln = Alignment(None, [Sequence(n, s) for n, s in zip(names, seqs)], taxa, NucleotideDataType(None))
        tree = fixed_tree_class()(topo.postorder, names, Parameter(None, t_ref))
        like = TreeLikelihoodModel(None, SitePattern(None, aln), tree, JC69(None),
                                   WeibullSiteModel(None, Parameter(None, s_ref), 4),
                                   StrictClockModel(None, Parameter(None, c_ref), tree))
        want = like().reshape(-1)
    finally:
        torch.set_default_dtype(dtype)
    assert abs(float(want.detach()[0]) - KAT) < 1e-9 * abs(KAT)
    g_want = torch.autograd.grad(want.sum(), [t_ref, c_ref, s_ref])

    t, c, s = leaves()
    ca = patterns.compress(seqs)
    tips = [torch.tensor(x) for x in ca.tip_partials()]
    rates, props = OL.weibull_rates(s, 4)
    mats = OL.p_t_jc69(OL.model_branch_lengths(t, c).unsqueeze(-1) * rates)
    got = OL.treelikelihood_discrete(tips + [None] * (len(tips) - 1), torch.tensor(ca.weights, dtype=torch.float64),
                                     topo.postorder_list(), mats, torch.full((1, 4), 0.25, dtype=torch.float64),
                                     props.reshape(4, 1, 1)).reshape(-1)
    np.testing.assert_allclose(got.detach().numpy(), want.detach().numpy(), rtol=1e-12)
    for g, w in zip(torch.autograd.grad(got.sum(), [t, c, s]), g_want):
        np.testing.assert_allclose(g.numpy(), w.numpy(), rtol=1e-9, atol=1e-9 * float(w.abs().max()))
