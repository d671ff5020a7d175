"""The plug-in layer above the engine: the CLI hooks that retarget a
generated configuration, and ``model.TreeLikelihoodModel``'s gathering of
engine inputs checked against torchtree's own ``TreeLikelihoodModel``.

The model tests import torchtree from its source tree
(``tests/reference_models.py``); they are skipped where it is absent.  They run
on the CPU: the inputs that ``_call`` would hand to the engine are gathered
on the CPU and evaluated by the oracle, and the result must equal the
reference model's own lnL (1e-12 relative).  Without CUDA, ``_call`` itself
must raise (no CPU fallback).
"""
import argparse

import numpy as np
import pytest
import torch

from tests.reference_models import fixed_tree_class, import_torchtree, reference_objects as _models



def test_cli_hook_retargets_every_likelihood():
    from torchtree_gb300.cli.evolution import process_tree_likelihood

    data = {"type": "JointDistributionModel", "distributions": [
        {"id": "like", "type": "TreeLikelihoodModel"},
        {"type": "JointDistributionModel", "distributions": [{"id": "like2", "type": "TreeLikelihoodModel"}]},
    ]}
    process_tree_likelihood(argparse.Namespace(gb300_precision="f32"), data)
    inner = [data["distributions"][0], data["distributions"][1]["distributions"][0]]
    for d in inner:
        assert d["type"] == "torchtree_gb300.TreeLikelihoodModel" and d["precision"] == "f32"
    single = {"id": "like", "type": "TreeLikelihoodModel"}
    process_tree_likelihood(argparse.Namespace(), single)
    assert single["precision"] == "f64"


@pytest.fixture(scope="module")
def torchtree_ref():
    if not import_torchtree():
        pytest.skip("torchtree source not present")
    torch.set_default_dtype(torch.float64)
    yield
    torch.set_default_dtype(torch.float32)


def test_plugin_flag_adds_arguments_and_retargets(torchtree_ref):
    from torchtree_gb300.plugin import GB300

    parser = argparse.ArgumentParser()
    sub = parser.add_subparsers()
    sub.add_parser("advi")
    sub.add_parser("map")
    plugin = GB300()
    plugin.load_arguments(sub)
    arg = parser.parse_args(["advi", "--gb300", "--gb300-precision", "f32"])
    data = {"id": "like", "type": "TreeLikelihoodModel"}
    plugin.process_tree_likelihood(arg, data)
    assert data["type"] == "torchtree_gb300.TreeLikelihoodModel" and data["precision"] == "f32"
    data = {"id": "like", "type": "TreeLikelihoodModel"}
    plugin.process_tree_likelihood(parser.parse_args(["map"]), data)
    assert data["type"] == "TreeLikelihoodModel"


def _oracle_lnl(route, tensors, topo, alignment, rescale):
    """lnL from the gathered engine inputs, by the oracle on the CPU."""
    from oracle import likelihood as OL

    if route == "rate_matrix":
        qn, _, bls, rates, probs, freqs = tensors
        times = bls.unsqueeze(-1) * rates.unsqueeze(-2)  # [b, B, K]
        mats = torch.linalg.matrix_exp(qn[:, None, None] * times[..., None, None])
    elif route == "general_rate_matrix":
        qn, bls, rates, probs, freqs = tensors
        times = bls.unsqueeze(-1) * rates.unsqueeze(-2)
        mats = torch.linalg.matrix_exp(qn[:, None, None] * times[..., None, None])
    else:
        mats, probs, freqs = tensors
    tips = [torch.tensor(alignment.table[c].T) for c in alignment.codes]  # [S, N] per tip
    parts = tips + [None] * (len(tips) - 1)
    fn = OL.treelikelihood_discrete_rescaled if rescale else OL.treelikelihood_discrete
    return fn(parts, torch.tensor(alignment.weights, dtype=torch.float64), topo.postorder_list(), mats,
              freqs.unsqueeze(-2), probs[..., None, None]).reshape(-1)


@pytest.mark.parametrize("case,b", [("gtr_weibull", 1), ("gtr_weibull", 2), ("jc69_constant", 1),
                                    ("hky_weibull_clock", 2), ("gtr_weibull_tipstates", 2)])
def test_model_gathers_the_reference_inputs(torchtree_ref, case, b):
    """The plug-in's engine inputs, evaluated by the oracle, give the
    reference model's own lnL (unscaled and rescaled) and, through autograd,
    its gradients with respect to every parameter (1e-9); the route follows
    the substitution model (eigen-form p_t: rate matrix; JC69's closed form:
    matrices)."""
    from torchtree.evolution.tree_likelihood import TreeLikelihoodModel as Reference

    from torchtree_gb300 import synthetic
    from torchtree_gb300.model import TreeLikelihoodModel

    wl = synthetic.dna_workload("plugin", tip_count=12, site_count=300, batch=2, seed=91, shape=0.5,
                                site_model="weibull")
    for rescale in (False, True):
        tree, sp, subst, site, clock, tip_states, leaves = _models(case, wl, b)
        ref = Reference(None, sp, tree, subst, site, clock, False, tip_states)
        ref.rescale = rescale
        want = ref().reshape(-1)
        gwant = torch.autograd.grad(want.sum(), leaves)
        tree, sp, subst, site, clock, tip_states, leaves = _models(case, wl, b)
        ours = TreeLikelihoodModel(None, sp, tree, subst, site, clock, False, tip_states, precision="f64")
        route, tensors, sample_shape, (nb, S, K) = ours.engine_inputs(torch.device("cpu"))
        assert route == ("matrices" if case.startswith("jc69") else "rate_matrix")
        assert (nb, S) == (b, 4) and tuple(sample_shape) == tuple(ref.sample_shape)
        got = _oracle_lnl(route, tensors, wl.topology, ours._alignment, rescale)
        np.testing.assert_allclose(got.detach().numpy(), want.detach().numpy(), rtol=1e-12)
        for g, w in zip(torch.autograd.grad(got.sum(), leaves), gwant):
            np.testing.assert_allclose(g.numpy(), w.numpy(), rtol=1e-9, atol=1e-9 * float(w.abs().max()))


def test_model_call_fails_loudly_without_cuda(torchtree_ref):
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    from torchtree_gb300 import synthetic
    from torchtree_gb300.model import TreeLikelihoodModel

    wl = synthetic.dna_workload("plugin", tip_count=6, site_count=50, batch=1, seed=92)
    tree, sp, subst, site, clock, tip_states, _ = _models("gtr_weibull", wl, 1)
    ours = TreeLikelihoodModel(None, sp, tree, subst, site, clock, False, tip_states)
    with pytest.raises((RuntimeError, AssertionError)):
        ours()


def test_json_route_selects_the_plugin_class(torchtree_ref):
    """A configuration names the class by its dotted path (core/utils.py:116-125)
    and may add "precision"; the other keys are the reference's."""
    from torchtree.core.utils import get_class, process_object

    from torchtree_gb300 import synthetic
    from torchtree_gb300.model import TreeLikelihoodModel

    assert get_class("torchtree_gb300.TreeLikelihoodModel") is TreeLikelihoodModel
    wl = synthetic.dna_workload("plugin", tip_count=8, site_count=100, batch=1, seed=93, site_model="weibull")
    tree, sp, subst, site, clock, _, _ = _models("hky_weibull_clock", wl, 1)
    dic = {"tree": tree, "sp": sp, "subst": subst, "site": site, "clock": clock}
    like = process_object({"id": "like", "type": "torchtree_gb300.TreeLikelihoodModel", "tree_model": "tree",
                           "site_model": "site", "substitution_model": "subst", "site_pattern": "sp",
                           "branch_model": "clock", "precision": "f32"}, dic)
    assert isinstance(like, TreeLikelihoodModel) and like.precision == "f32" and like.rescale
    assert like.clock_model is clock and dic["like"] is like
    assert like._alignment.codes.shape == (8, like.weights.shape[0])


@pytest.mark.parametrize("seed", range(12))
def test_compression_matches_torchtree_on_random_alignments(torchtree_ref, seed):
    """Randomized parity of the compression path (C++ column sort behind
    ``patterns.compress``) against torchtree's own ``compress_alignment`` /
    ``compress_alignment_states``: same pattern order and weights, and tip
    partials / states bit-exact, with IUPAC ambiguity codes, gaps, unknowns and
    lower case, in unsorted taxon order, with and without ambiguities.  Amino
    acids and codons (gaps, stop codons) too."""
    from torchtree.evolution.alignment import Alignment, Sequence
    from torchtree.evolution.datatype import AminoAcidDataType, NucleotideDataType
    from torchtree.evolution.site_pattern import compress_alignment, compress_alignment_states
    from torchtree.evolution.taxa import Taxa, Taxon

    from torchtree_gb300 import datatype, patterns

    rng = np.random.default_rng(100 + seed)
    T, L = int(rng.integers(2, 12)), int(rng.integers(1, 400))
    if seed % 4 == 3:
        _codon_case(rng, T, L)
        return
    amino = seed % 4 == 2
    alphabet = list("ACDEFGHIKLMNPQRSTVWYXBZ-?acd") if amino else list("ACGTACGTACGTRYKMSWBDHVN-?acgtu")
    repeats = rng.integers(1, 4)  # repeated columns make weights > 1
    base = rng.choice(alphabet, size=(T, max(1, L // repeats)))
    cols = np.tile(base, (1, repeats))[:, rng.permutation(base.shape[1] * repeats)]
    seqs = ["".join(r) for r in cols]
    names = [f"t{i}" for i in rng.permutation(T)]
    dt_ref = AminoAcidDataType(None) if amino else NucleotideDataType(None)
    dt = datatype.AminoAcid() if amino else datatype.Nucleotide()
    aln = Alignment(None, [Sequence(n, s) for n, s in zip(names, seqs)], Taxa(None, [Taxon(n, {}) for n in names]),
                    dt_ref)
    for amb in (False, True):
        parts, w = compress_alignment(aln, None, amb)
        ca = patterns.compress(seqs, dt, use_ambiguities=amb)
        assert ca.weights.tolist() == w.tolist()
        np.testing.assert_array_equal(ca.tip_partials(), np.stack([p.numpy() for p in parts]))
    states, w = compress_alignment_states(aln)
    st = patterns.compress(seqs, dt, tip_states=True)
    assert st.weights.tolist() == w.tolist()
    assert st.codes.tolist() == [s.tolist() for s in states]


def _codon_case(rng, T, L):
    from torchtree.evolution.alignment import Alignment, Sequence
    from torchtree.evolution.datatype import CodonDataType
    from torchtree.evolution.site_pattern import compress_alignment, compress_alignment_states
    from torchtree.evolution.taxa import Taxa, Taxon

    from torchtree_gb300 import datatype, patterns

    sense = [a + b + c for a in "ACGT" for b in "ACGT" for c in "ACGT"]
    pool = sense + ["---", "TAA", "TGA", "TAG"]  # gaps and stop codons
    n = max(1, L // 3)
    seqs = ["".join(rng.choice(pool, size=n)) for _ in range(T)]
    names = [f"c{i}" for i in rng.permutation(T)]
    aln = Alignment(None, [Sequence(m, s) for m, s in zip(names, seqs)], Taxa(None, [Taxon(m, {}) for m in names]),
                    CodonDataType(None, "Universal"))
    parts, w = compress_alignment(aln, None, False)
    ca = patterns.compress(seqs, datatype.Codon())
    assert ca.weights.tolist() == w.tolist()
    np.testing.assert_array_equal(ca.tip_partials(), np.stack([p.numpy() for p in parts]))
    states, w = compress_alignment_states(aln)
    assert ca.codes.tolist() == [s.tolist() for s in states]


@pytest.mark.parametrize("seed", range(10))
def test_model_inputs_on_random_problems(torchtree_ref, seed):
    """Randomized form of the input-gathering check: tree size, model (GTR, HKY,
    JC69), site model (Weibull, Weibull + invariant, constant), clock or not,
    tip states or partials, rescaling and batch drawn at random; the oracle's
    lnL and gradients from the plug-in's inputs equal torchtree's own."""
    from torchtree import Parameter
    from torchtree.evolution.alignment import Alignment, Sequence
    from torchtree.evolution.branch_model import StrictClockModel
    from torchtree.evolution.datatype import NucleotideDataType
    from torchtree.evolution.site_model import ConstantSiteModel, WeibullSiteModel
    from torchtree.evolution.site_pattern import SitePattern
    from torchtree.evolution.substitution_model import GTR, HKY, JC69
    from torchtree.evolution.taxa import Taxa, Taxon
    from torchtree.evolution.tree_likelihood import TreeLikelihoodModel as Reference

    from torchtree_gb300 import synthetic
    from torchtree_gb300.model import TreeLikelihoodModel

    rng = np.random.default_rng(500 + seed)
    T, b = int(rng.integers(3, 25)), int(rng.integers(1, 3))
    subst_kind = ["gtr", "hky", "jc69"][seed % 3]
    site_kind = ["weibull", "weibull_inv", "constant"][(seed // 3) % 3]
    clock_on, tip_states, rescale = bool(rng.integers(2)), bool(rng.integers(2)), bool(rng.integers(2))
    wl = synthetic.dna_workload("r", tip_count=T, site_count=int(rng.integers(20, 300)), batch=b,
                                seed=600 + seed, shape=float(rng.uniform(0.2, 2.0)), site_model="weibull")
    names = wl.topology.tip_names
    B = 2 * T - 2

    def build():
        leaf = lambda a: torch.tensor(np.asarray(a, dtype=np.float64), requires_grad=True)  # noqa: E731
        leaves = []
        taxa = Taxa(None, [Taxon(n, {}) for n in names])
        aln = Alignment(None, [Sequence(n, s) for n, s in zip(names, wl.sequences)], taxa,
                        NucleotideDataType(None))
        if clock_on:
            bl = leaf(np.random.default_rng(seed).uniform(0.5, 5.0, (b, B)))
            tree = fixed_tree_class()(wl.topology.postorder, names, Parameter(None, bl))
            rate = leaf(np.full((b, 1), 0.02))
            clock = StrictClockModel(None, Parameter(None, rate), tree)
            leaves += [bl, rate]
        else:
            bl = leaf(wl.branch_lengths)
            tree = fixed_tree_class()(wl.topology.postorder, names, Parameter(None, bl))
            clock = None
            leaves.append(bl)
        if subst_kind == "jc69":
            subst = JC69(None)
        else:
            pi = leaf(wl.pi)
            if subst_kind == "gtr":
                ex = leaf(wl.exch)
                subst = GTR(None, Parameter(None, ex), Parameter(None, pi))
            else:
                ex = leaf(wl.exch[:, 1:2])
                subst = HKY(None, Parameter(None, ex), Parameter(None, pi))
            leaves += [ex, pi]
        if site_kind == "constant":
            site = ConstantSiteModel(None)
        else:
            shape = leaf(wl.shape)
            inv = leaf(np.full((b, 1), 0.15)) if site_kind == "weibull_inv" else None
            site = WeibullSiteModel(None, Parameter(None, shape), 4,
                                    invariant=Parameter(None, inv) if inv is not None else None)
            leaves += [shape] + ([inv] if inv is not None else [])
        return tree, SitePattern(None, aln), subst, site, clock, leaves

    tree, sp, subst, site, clock, leaves = build()
    ref = Reference(None, sp, tree, subst, site, clock, False, tip_states)
    ref.rescale = rescale
    want = ref().reshape(-1)
    gwant = torch.autograd.grad(want.sum(), leaves)
    tree, sp, subst, site, clock, leaves = build()
    ours = TreeLikelihoodModel(None, sp, tree, subst, site, clock, False, tip_states)
    route, tensors, _, _ = ours.engine_inputs(torch.device("cpu"))
    got = _oracle_lnl(route, tensors, wl.topology, ours._alignment, rescale)
    np.testing.assert_allclose(got.detach().numpy(), want.detach().numpy(), rtol=1e-12)
    for g, w in zip(torch.autograd.grad(got.sum(), leaves), gwant):
        np.testing.assert_allclose(g.numpy(), w.numpy(), rtol=1e-9, atol=1e-9 * float(w.abs().max()))


@pytest.mark.parametrize("kind,seed", [("protein", 0), ("codon", 1), ("protein", 2), ("codon", 3)])
def test_model_inputs_for_amino_acids_and_codons(torchtree_ref, kind, seed):
    """The plug-in on 20- and 61-state models (GeneralSymmetricSubstitutionModel
    with 190 free rates, MG94 with alpha = 1), against torchtree's own lnL and
    gradients (1e-10 / 1e-8: 61 x 61 matrix exponentials)."""
    from torchtree import Parameter
    from torchtree.evolution.alignment import Alignment, Sequence
    from torchtree.evolution.datatype import AminoAcidDataType, CodonDataType
    from torchtree.evolution.site_model import WeibullSiteModel
    from torchtree.evolution.site_pattern import SitePattern
    from torchtree.evolution.substitution_model import MG94
    from torchtree.evolution.substitution_model.general import GeneralSymmetricSubstitutionModel
    from torchtree.evolution.taxa import Taxa, Taxon
    from torchtree.evolution.tree_likelihood import TreeLikelihoodModel as Reference

    from torchtree_gb300 import synthetic
    from torchtree_gb300.model import TreeLikelihoodModel

    if kind == "protein":
        wl = synthetic.protein_workload("p", tip_count=9, site_count=80, batch=1, seed=700 + seed, shape=0.7,
                                        site_model="weibull", branch_mean=0.1)
    else:
        wl = synthetic.codon_workload("c", tip_count=6, site_count=40, batch=1, seed=700 + seed, shape=0.7,
                                      site_model="weibull", branch_mean=0.1)
    names = wl.topology.tip_names

    def build():
        leaf = lambda a: torch.tensor(np.asarray(a, dtype=np.float64), requires_grad=True)  # noqa: E731
        bl, pi, shape, ex = leaf(wl.branch_lengths), leaf(wl.pi), leaf(wl.shape), leaf(wl.exch)
        if kind == "protein":
            dtype = AminoAcidDataType(None)
            subst = GeneralSymmetricSubstitutionModel(None, dtype, Parameter(None, torch.arange(190)),
                                                      Parameter(None, ex), Parameter(None, pi))
        else:
            dtype = CodonDataType(None, "Universal")
            subst = MG94(None, dtype, Parameter(None, torch.ones_like(ex[..., :1])), Parameter(None, ex[..., 1:2]),
                         Parameter(None, ex[..., 0:1]), Parameter(None, pi))
        taxa = Taxa(None, [Taxon(n, {}) for n in names])
        aln = Alignment(None, [Sequence(n, s) for n, s in zip(names, wl.sequences)], taxa, dtype)
        tree = fixed_tree_class()(wl.topology.postorder, names, Parameter(None, bl))
        site = WeibullSiteModel(None, Parameter(None, shape), 4)
        return tree, SitePattern(None, aln), subst, site, [bl, ex, pi, shape]

    tree, sp, subst, site, leaves = build()
    want = Reference(None, sp, tree, subst, site)().reshape(-1)
    gwant = torch.autograd.grad(want.sum(), leaves)
    tree, sp, subst, site, leaves = build()
    ours = TreeLikelihoodModel(None, sp, tree, subst, site)
    route, tensors, _, (_, S, _) = ours.engine_inputs(torch.device("cpu"))
    assert route == "rate_matrix" and S == (20 if kind == "protein" else 61)
    got = _oracle_lnl(route, tensors, wl.topology, ours._alignment, False)
    np.testing.assert_allclose(got.detach().numpy(), want.detach().numpy(), rtol=1e-10)
    for g, w in zip(torch.autograd.grad(got.sum(), leaves), gwant):
        np.testing.assert_allclose(g.numpy(), w.numpy(), rtol=1e-8, atol=1e-8 * float(w.abs().max()))


@pytest.mark.parametrize("seed", range(8))
def test_time_tree_oracle_matches_torchtree_on_random_trees(torchtree_ref, seed):
    """The oracle behind the time-tree kernels against torchtree's own
    GeneralNodeHeightTransform (heights, branch lengths, log|J|) and
    ConstantCoalescent, values and autograd gradients, on random trees with
    isochronous, heterochronous and tied sampling times."""
    from types import SimpleNamespace

    from torchtree.evolution.coalescent import ConstantCoalescent
    from torchtree.evolution.tree_height_transform import GeneralNodeHeightTransform
    from torchtree.evolution.tree_model import heights_to_branch_lengths

    from oracle import timetree as OT
    from torchtree_gb300 import synthetic

    rng = np.random.default_rng(800 + seed)
    T = int(rng.integers(2, 60))
    topo = synthetic.yule_topology(T, rng)
    kind = seed % 3
    times = np.zeros(T) if kind == 0 else (rng.uniform(0, 2, T) if kind == 1 else np.round(rng.uniform(0, 1, T), 1))
    times[int(rng.integers(T))] = 0.0
    kids = {int(v): (int(l), int(r)) for v, l, r in topo.postorder}
    pre, stack = [], [2 * T - 2]
    while stack:  # parent before child
        v = stack.pop()
        if v >= T:
            for c in kids[v]:
                pre.append((v, c))
                stack.append(c)
    fake = SimpleNamespace(taxa_count=T, postorder=[list(map(int, t)) for t in topo.postorder],
                           preorder=torch.tensor(pre), sampling_times=torch.tensor(times))
    tr = GeneralNodeHeightTransform(fake)
    x = np.concatenate([rng.uniform(0.05, 0.95, T - 2), [float(times.max()) + rng.uniform(0.5, 3.0)]])
    w_h, w_b = rng.normal(size=T - 1), rng.normal(size=2 * T - 2)
    theta_v = float(rng.uniform(0.3, 3.0))

    def objective(heights, bl, logdet):
        return (heights * torch.tensor(w_h)).sum() + 0.7 * logdet.sum() + (bl * torch.tensor(w_b)).sum()

    xr = torch.tensor(x, requires_grad=True)
    hr = tr(xr)
    ldr = tr.log_abs_det_jacobian(xr, hr)
    blr = heights_to_branch_lengths(hr, tr._bounds, fake.preorder)
    (gr,) = torch.autograd.grad(objective(hr, blr, ldr), xr)
    xo = torch.tensor(x, requires_grad=True)
    ho, blo, ldo = OT.ratio_transform(topo.postorder.tolist(), times.tolist(), xo)
    (go,) = torch.autograd.grad(objective(ho, blo, ldo), xo)
    np.testing.assert_allclose(ho.detach().numpy(), hr.detach().numpy(), rtol=1e-13)
    np.testing.assert_allclose(blo.detach().numpy(), blr.detach().numpy(), rtol=1e-12, atol=1e-13)
    np.testing.assert_allclose(float(ldo.detach()), float(ldr.detach()), rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(go.numpy(), gr.numpy(), rtol=1e-10, atol=1e-10 * float(gr.abs().max()))

    h_int = hr.detach().clone()
    hh_r, th_r = h_int.clone().requires_grad_(), torch.tensor([theta_v], requires_grad=True)
    lp_r = ConstantCoalescent(th_r).log_prob(torch.cat((torch.tensor(times), hh_r)))
    g_r = torch.autograd.grad(lp_r.sum(), [hh_r, th_r])
    hh_o, th_o = h_int.clone().requires_grad_(), torch.tensor([theta_v], requires_grad=True)
    lp_o = OT.constant_coalescent(times.tolist(), hh_o, th_o)
    g_o = torch.autograd.grad(lp_o.sum(), [hh_o, th_o])
    np.testing.assert_allclose(float(lp_o.detach().reshape(-1)[0]), float(lp_r.detach().reshape(-1)[0]), rtol=1e-12)
    for a, b in zip(g_o, g_r):
        np.testing.assert_allclose(a.numpy(), b.numpy(), rtol=1e-10, atol=1e-10 * float(b.abs().max()))


@pytest.mark.parametrize("seed", range(8))
def test_oracle_pruning_functions_match_torchtree(torchtree_ref, seed):
    """Each oracle pruning function against the reference function it restates
    (tree_likelihood.py:14-278), on random trees, partials, matrices and
    batches: the unscaled, rescaled and tip-state variants, and the selective
    rescaling after an underflow."""
    from torchtree.evolution import tree_likelihood as TL

    from oracle import likelihood as OL
    from torchtree_gb300 import synthetic

    rng = np.random.default_rng(900 + seed)
    T, S, K, N = int(rng.integers(2, 30)), [4, 20][seed % 2], int(rng.integers(1, 5)), int(rng.integers(1, 60))
    bshape = [(), (2,), (3,)][seed % 3]
    post = synthetic.yule_topology(T, rng).postorder.tolist()
    B = 2 * T - 2
    q = rng.random(bshape + (B, K, S, S))
    mats = torch.tensor(q / q.sum(-1, keepdims=True))
    f = rng.random(bshape + (1, S))
    freqs = torch.tensor(f / f.sum(-1, keepdims=True))
    p = rng.random(bshape + (K, 1, 1))
    props = torch.tensor(p / p.sum(-3, keepdims=True))
    weights = torch.tensor(rng.integers(1, 5, N), dtype=torch.float64)
    tips = [torch.tensor(rng.random((S, N))) for _ in range(T)]
    states = [torch.tensor(rng.integers(0, S + 1, N)) for _ in range(T)]
    blank = [None] * (T - 1)

    def close(a, b):
        np.testing.assert_allclose(a.numpy(), b.numpy(), rtol=1e-12)

    close(OL.treelikelihood_discrete(tips + blank, weights, post, mats, freqs, props),
          TL.calculate_treelikelihood_discrete(tips + blank, weights, post, mats, freqs, props))
    close(OL.treelikelihood_discrete_rescaled(tips + blank, weights, post, mats, freqs, props),
          TL.calculate_treelikelihood_discrete_rescaled(tips + blank, weights, post, mats, freqs, props))
    close(OL.treelikelihood_tip_states_discrete(states + blank, weights, post, mats, freqs, props),
          TL.calculate_treelikelihood_tip_states_discrete(states + blank, weights, post, mats, freqs, props))
    close(OL.treelikelihood_tip_states_discrete_rescaled(states + blank, weights, post, mats, freqs, props),
          TL.calculate_treelikelihood_tip_states_discrete_rescaled(states + blank, weights, post, mats, freqs,
                                                                   props))
    one = mats[..., 0, :, :]  # single category
    close(OL.treelikelihood(tips + blank, weights, post, one, freqs),
          TL.calculate_treelikelihood(tips + blank, weights, post, one, freqs))
    # selective rescaling on the partials an unscaled pass left behind (tiny values underflow)
    small = [t * 1e-30 for t in tips]
    failed = small + list(blank)
    TL.calculate_treelikelihood_discrete(failed, weights, post, mats, freqs, props)  # fills the internals
    close(OL.treelikelihood_discrete_safe(list(failed), weights, post, mats, freqs, props, 1e-20),
          TL.calculate_treelikelihood_discrete_safe(list(failed), weights, post, mats, freqs, props, 1e-20))
    lnl, flag = OL.unscaled_then_safe(small + list(blank), weights, post, mats, freqs, props, 1e-20)
    close(lnl, TL.calculate_treelikelihood_discrete_safe(list(failed), weights, post, mats, freqs, props, 1e-20)
          if flag else TL.calculate_treelikelihood_discrete(small + list(blank), weights, post, mats, freqs, props))


@pytest.mark.parametrize("seed", range(6))
def test_rate_matrices_and_eigen_form_match_torchtree(torchtree_ref, seed):
    """The package's host-side Q builders (GTR, HKY, general symmetric 20-state,
    MG94) and its eigen form P = U diag(exp(lambda t)) W against the reference
    models' q() and p_t() on random parameters (batched)."""
    from torchtree import Parameter
    from torchtree.evolution.datatype import AminoAcidDataType, CodonDataType
    from torchtree.evolution.substitution_model import GTR, HKY, MG94
    from torchtree.evolution.substitution_model.general import GeneralSymmetricSubstitutionModel

    from torchtree_gb300 import substitution

    rng = np.random.default_rng(1000 + seed)
    b = int(rng.integers(1, 4))
    kind = ["gtr", "hky", "general", "mg94"][seed % 4]
    t = torch.tensor(rng.uniform(0.001, 2.0, (b, 5)))
    if kind in ("gtr", "hky"):
        S = 4
    elif kind == "general":
        S = 20
    else:
        S = 61
    pi = torch.tensor(rng.dirichlet(np.ones(S), size=b))
    if kind == "gtr":
        ex = torch.tensor(rng.gamma(1.0, 1.0, (b, 6)))
        ref, ours = GTR(None, Parameter(None, ex), Parameter(None, pi)), substitution.gtr_q(ex, pi)
    elif kind == "hky":
        kappa = torch.tensor(rng.lognormal(1.0, 0.5, (b, 1)))
        ref, ours = HKY(None, Parameter(None, kappa), Parameter(None, pi)), substitution.hky_q(kappa, pi)
    elif kind == "general":
        ex = torch.tensor(rng.gamma(1.0, 1.0, (b, 190)))
        ref = GeneralSymmetricSubstitutionModel(None, AminoAcidDataType(None), Parameter(None, torch.arange(190)),
                                                Parameter(None, ex), Parameter(None, pi))
        ours = substitution.general_symmetric_q(ex, pi, 20)
    else:
        omega = torch.tensor(rng.gamma(2.0, 0.25, (b, 1)))
        kappa = torch.tensor(rng.lognormal(1.0, 0.5, (b, 1)))
        ref = MG94(None, CodonDataType(None, "Universal"), Parameter(None, torch.ones_like(omega)),
                   Parameter(None, omega), Parameter(None, kappa), Parameter(None, pi))
        ours = substitution.mg94_q(torch.ones_like(omega), omega, kappa, pi)
    q_ref = ref.q()
    q_ref = q_ref / ref.norm(q_ref)[..., None, None]
    np.testing.assert_allclose(substitution.normalise(ours, pi).numpy(), q_ref.expand(b, S, S).numpy(),
                               rtol=1e-12, atol=1e-14)
    lam, u, w = substitution.eigen_system(ours, pi)
    mine = u[:, None] @ torch.diag_embed(torch.exp(lam[:, None] * t[..., None])) @ w[:, None]
    np.testing.assert_allclose(mine.numpy(), ref.p_t(t).expand(b, 5, S, S).numpy(), rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize("seed", range(4))
def test_site_models_match_torchtree(torchtree_ref, seed):
    """The package's Weibull rates (with invariant sites and mu) and the
    proportion-invariant model against torchtree's own site models on random
    batched parameters, values and shape gradients."""
    from torchtree import Parameter
    from torchtree.evolution.site_model import InvariantSiteModel, WeibullSiteModel

    from torchtree_gb300 import site_models

    rng = np.random.default_rng(1100 + seed)
    b, K = int(rng.integers(1, 4)), int(rng.integers(1, 9))
    shape_v = rng.uniform(0.05, 5.0, (b, 1))
    inv_v = rng.uniform(0.0, 0.6, (b, 1)) if seed % 2 else None
    mu_v = rng.uniform(0.5, 2.0, (b, 1)) if seed >= 2 else None
    leaf = lambda a: torch.tensor(a, requires_grad=True)  # noqa: E731
    s_ref = leaf(shape_v)
    ref = WeibullSiteModel(None, Parameter(None, s_ref), K,
                           invariant=Parameter(None, torch.tensor(inv_v)) if inv_v is not None else None,
                           mu=Parameter(None, torch.tensor(mu_v)) if mu_v is not None else None)
    s_ours = leaf(shape_v)
    rates, probs = site_models.weibull_rates(s_ours, K, invariant=torch.tensor(inv_v) if inv_v is not None else None,
                                             mu=torch.tensor(mu_v) if mu_v is not None else None)
    np.testing.assert_allclose(rates.detach().numpy(), ref.rates().detach().numpy(), rtol=1e-13, atol=1e-300)
    np.testing.assert_allclose(probs.numpy(), ref.probabilities().expand(probs.shape).numpy(), rtol=1e-14)
    wts = torch.tensor(rng.normal(size=rates.shape))
    (g_ref,) = torch.autograd.grad((ref.rates() * wts).sum(), s_ref)
    (g_ours,) = torch.autograd.grad((rates * wts).sum(), s_ours)
    np.testing.assert_allclose(g_ours.numpy(), g_ref.numpy(), rtol=1e-11, atol=1e-300)
    p = torch.tensor(rng.uniform(0.0, 0.9, (b, 1)))
    inv_ref = InvariantSiteModel(None, Parameter(None, p), Parameter(None, torch.tensor(mu_v)) if mu_v is not None
                                 else None)
    r2, p2 = site_models.invariant_rates(p, mu=torch.tensor(mu_v) if mu_v is not None else None)
    np.testing.assert_allclose(r2.numpy(), inv_ref.rates().numpy(), rtol=1e-14)
    np.testing.assert_allclose(p2.numpy(), inv_ref.probabilities().numpy(), rtol=1e-14)


def test_gamma_site_model_from_json(torchtree_ref):
    """``torchtree_gb300.GammaSiteModel`` resolves by its dotted path and gives
    the package's Gamma rates (plain, with invariant sites and mu, batched),
    with the shape gradient flowing into the torchtree Parameter."""
    from torchtree import Parameter
    from torchtree.core.utils import process_object

    from torchtree_gb300 import site_models
    from torchtree_gb300.model import GammaSiteModel

    shape = torch.tensor([[0.3], [1.7]], dtype=torch.float64, requires_grad=True)
    inv = torch.tensor([[0.1], [0.25]], dtype=torch.float64, requires_grad=True)
    mu = torch.tensor([[1.5], [0.5]], dtype=torch.float64)
    dic = {"shape": Parameter("shape", shape), "inv": Parameter("inv", inv), "mu": Parameter("mu", mu)}
    for extra in ({}, {"invariant": "inv", "mu": "mu"}):
        site = process_object({"id": "sm", "type": "torchtree_gb300.GammaSiteModel", "shape": "shape",
                               "categories": 4, **extra}, dic)
        assert isinstance(site, GammaSiteModel)
        want_r, want_p = site_models.gamma_rates(shape, 4, inv if extra else None, mu if extra else None)
        np.testing.assert_allclose(site.rates().detach().numpy(), want_r.detach().numpy(), rtol=1e-14)
        got_p = site.probabilities().detach().numpy()  # [K] without invariant sites, as torchtree keeps it
        np.testing.assert_allclose(np.broadcast_to(got_p, want_p.shape), want_p.detach().numpy(), rtol=1e-14)
        (g,) = torch.autograd.grad(site.rates()[:, -1].sum(), shape)
        (gw,) = torch.autograd.grad(want_r[:, -1].sum(), shape)
        np.testing.assert_allclose(g.numpy(), gw.numpy(), rtol=1e-12)
        dic.pop("sm")


@pytest.mark.parametrize("b", [1, 2])
def test_model_inputs_for_a_nonreversible_model(torchtree_ref, b):
    """torchtree's GeneralNonSymmetricSubstitutionModel (12 free rates) takes the
    plug-in's matrix-exponential route; its gathered inputs give torchtree's
    own lnL (unscaled and rescaled) and gradients (1e-12 / 1e-9)."""
    from torchtree import Parameter
    from torchtree.evolution.datatype import NucleotideDataType
    from torchtree.evolution.substitution_model.general import GeneralNonSymmetricSubstitutionModel
    from torchtree.evolution.tree_likelihood import TreeLikelihoodModel as Reference

    from torchtree_gb300 import synthetic
    from torchtree_gb300.model import TreeLikelihoodModel

    wl = synthetic.dna_workload("nr", tip_count=10, site_count=200, batch=2, seed=94, shape=0.5,
                                site_model="weibull")
    rng = np.random.default_rng(7)
    rates0 = rng.gamma(1.0, 1.0, (b, 12))
    for rescale in (False, True):
        def build():
            tree, sp, _, site, clock, tip_states, leaves = _models("gtr_weibull", wl, b)
            r = torch.tensor(rates0, requires_grad=True)
            pi = torch.tensor(wl.pi[:b], requires_grad=True)
            subst = GeneralNonSymmetricSubstitutionModel(None, NucleotideDataType(None),
                                                         Parameter(None, torch.arange(12)), Parameter(None, r),
                                                         Parameter(None, pi), True)
            return tree, sp, subst, site, [leaves[0], r, pi, leaves[-1]]

        tree, sp, subst, site, leaves = build()
        ref = Reference(None, sp, tree, subst, site)
        ref.rescale = rescale
        want = ref().reshape(-1)
        gwant = torch.autograd.grad(want.sum(), leaves)
        tree, sp, subst, site, leaves = build()
        ours = TreeLikelihoodModel(None, sp, tree, subst, site)
        route, tensors, _, (nb, S, _) = ours.engine_inputs(torch.device("cpu"))
        assert route == "general_rate_matrix" and (nb, S) == (b, 4)
        got = _oracle_lnl(route, tensors, wl.topology, ours._alignment, rescale)
        np.testing.assert_allclose(got.detach().numpy(), want.detach().numpy(), rtol=1e-12)
        for g, w in zip(torch.autograd.grad(got.sum(), leaves), gwant):
            np.testing.assert_allclose(g.numpy(), w.numpy(), rtol=1e-9, atol=1e-9 * float(w.abs().max()))
