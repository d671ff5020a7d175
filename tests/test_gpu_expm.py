"""Transition matrices of non-reversible rate matrices on the device.

``tt_transition_matrices_expm`` (scaling and squaring, [13/13] Pade) against
``torch.linalg.matrix_exp`` on the CPU (what NonSymmetricSubstitutionModel.p_t
calls, abstract.py:86-94), its Frechet adjoint against torch autograd through
that ``matrix_exp``, the likelihood route built on them against the oracle,
and the plug-in class on torchtree's GeneralNonSymmetricSubstitutionModel
against torchtree's own TreeLikelihoodModel.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _random_q(rng, b, S):
    r = rng.gamma(1.0, 1.0, (b, S, S))
    for i in range(b):
        np.fill_diagonal(r[i], 0.0)
    q = r - np.eye(S)[None] * r.sum(-1, keepdims=True)
    pi = rng.dirichlet(np.ones(S), size=b)
    q = q / (-(np.diagonal(q, axis1=-2, axis2=-1) * pi).sum(-1))[:, None, None]
    return torch.tensor(q), torch.tensor(pi)


def _engine_stub(b, S, B, K):
    """An engine with the right shape for the expm entry points (any topology
    with B = 2T - 2 branches; B even)."""
    assert B % 2 == 0
    from torchtree_gb300 import synthetic
    from torchtree_gb300.engine import LikelihoodEngine

    T = B // 2 + 1
    topo = synthetic.yule_topology(T, np.random.default_rng(0))
    codes = np.zeros((T, 4), dtype=np.uint8)
    return LikelihoodEngine(topo.postorder, T, S, K, codes, np.eye(S), np.ones(4), batch=b, precision="f64")


@pytest.mark.parametrize("S", [2, 4, 20, 32, 61, 64])
def test_expm_matches_torch_matrix_exp(S):
    rng = np.random.default_rng(500 + S)
    b, B, K = 2, 6, 3
    q, _ = _random_q(rng, b, S)
    bl = torch.tensor(rng.exponential(0.3, (b, B)))
    bl[:, 0] = 0.0
    bl[:, 1] = 40.0  # a long branch: many squarings
    rates = torch.tensor(rng.gamma(2.0, 0.5, (b, K)))
    eng = _engine_stub(b, S, B, K)
    got = eng.expm_matrices(q.cuda(), bl.cuda(), rates.cuda()).cpu()
    times = bl.unsqueeze(-1) * rates.unsqueeze(-2)
    want = torch.linalg.matrix_exp(q[:, None, None] * times[..., None, None])
    assert float((got - want).abs().max()) <= 1e-12, float((got - want).abs().max())


@pytest.mark.parametrize("S", [2, 4, 20, 32])
def test_expm_adjoint_matches_autograd(S):
    rng = np.random.default_rng(600 + S)
    b, B, K = 2, 6, 2  # B = 2T - 2 branches of the stub engine's tree
    q, _ = _random_q(rng, b, S)
    bl = torch.tensor(rng.exponential(0.3, (b, B)))
    bl[:, 1] = 12.0
    rates = torch.tensor(rng.gamma(2.0, 0.5, (b, K)))
    G = torch.tensor(rng.normal(size=(b, B, K, S, S)))
    eng = _engine_stub(b, S, B, K)
    dq, dt, dr = (x.cpu() for x in eng.expm_gradient(q.cuda(), bl.cuda(), rates.cuda(), G.cuda()))
    qq, bb, rr = (x.clone().requires_grad_() for x in (q, bl, rates))
    times = bb.unsqueeze(-1) * rr.unsqueeze(-2)
    P = torch.linalg.matrix_exp(qq[:, None, None] * times[..., None, None])
    wq, wt, wr = torch.autograd.grad((P * G).sum(), (qq, bb, rr))
    for name, g, w in (("dQ", dq, wq), ("dt", dt, wt), ("dr", dr, wr)):
        err = float((g - w).abs().max() / w.abs().max())
        assert err <= 1e-10, (name, err)


def test_nonreversible_route_matches_oracle():
    """PhyloLikelihood.evaluate_general (device Pade + Frechet adjoint) on a
    non-reversible GTR-like Q with 12 free rates, against the oracle (matrix_exp
    + rescaled pruning + autograd, FP64)."""
    from oracle import likelihood as OL
    from torchtree_gb300 import patterns, synthetic
    from torchtree_gb300.likelihood import PhyloLikelihood

    wl = synthetic.dna_workload("nr", tip_count=40, site_count=500, batch=2, seed=62, shape=0.5,
                                site_model="weibull")
    ca = patterns.compress(wl.sequences)
    rng = np.random.default_rng(3)
    off0 = torch.tensor(rng.gamma(1.0, 1.0, (2, 12)))
    pi0 = torch.tensor(wl.pi)

    def q_of(r, pi):
        mask = ~torch.eye(4, dtype=torch.bool, device=r.device)
        q = torch.zeros(r.shape[0], 4, 4, dtype=torch.float64, device=r.device).masked_scatter(mask.expand(
            r.shape[0], 4, 4), r)
        q = q - torch.diag_embed(q.sum(-1))
        return q / (-(torch.diagonal(q, dim1=-2, dim2=-1) * pi).sum(-1))[:, None, None]

    rates0, probs = OL.weibull_rates(torch.tensor(wl.shape), 4)
    tips = [torch.tensor(t) for t in ca.tip_partials()]
    leaves = [x.clone().requires_grad_() for x in (torch.tensor(wl.branch_lengths), off0, pi0, rates0)]
    bl, off, pi, rates = leaves
    times = OL.model_branch_lengths(bl).unsqueeze(-1) * rates.unsqueeze(-2)
    mats = torch.linalg.matrix_exp(q_of(off, pi)[:, None, None] * times[..., None, None])
    ref = OL.treelikelihood_discrete_rescaled(tips + [None] * (len(tips) - 1), torch.tensor(ca.weights),
                                              wl.topology.postorder_list(), mats, pi.unsqueeze(-2),
                                              probs.reshape(-1, 4)[:, :, None, None]).reshape(-1)
    gref = torch.autograd.grad(ref.sum(), leaves)
    for precision, ltol, gtol in (("f64", 1e-10, 1e-9), ("f32", 1e-6, 1e-4)):
        lik = PhyloLikelihood(wl.topology, ca, 4, 4, batch=2, precision=precision)
        lik.rescale = True
        dl = [x.detach().cuda().requires_grad_() for x in leaves]
        lnl = lik.evaluate_general(q_of(dl[1], dl[2]), lik.node_branch_lengths(dl[0]), dl[3],
                                   probs.reshape(-1, 4).expand(2, 4).cuda(), dl[2])
        grads = torch.autograd.grad(lnl.sum(), dl)
        np.testing.assert_allclose(lnl.detach().cpu().numpy(), ref.detach().numpy(), rtol=ltol)
        for g, w, name in zip(grads, gref, ("bl", "rates12", "pi", "category rates")):
            np.testing.assert_allclose(g.cpu().numpy(), w.numpy(), rtol=gtol, atol=gtol * float(w.abs().max()),
                                       err_msg=f"{precision} {name}")


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_plugin_with_torchtree_nonreversible_model(precision):
    from tests.reference_models import import_torchtree, reference_objects

    if not import_torchtree():
        pytest.skip("torchtree not present (neither a source tree nor baseline/_ref)")
    from torchtree import Parameter
    from torchtree.evolution.datatype import NucleotideDataType
    from torchtree.evolution.substitution_model.general import GeneralNonSymmetricSubstitutionModel
    from torchtree.evolution.tree_likelihood import TreeLikelihoodModel as Reference

    from torchtree_gb300 import synthetic
    from torchtree_gb300.model import TreeLikelihoodModel

    torch.set_default_dtype(torch.float64)
    try:
        wl = synthetic.dna_workload("nr", tip_count=30, site_count=600, batch=2, seed=95, shape=0.5,
                                    site_model="weibull")
        rates0 = np.random.default_rng(8).gamma(1.0, 1.0, (2, 12))

        def build():
            tree, sp, _, site, _, _, leaves = reference_objects("gtr_weibull", wl, 2)
            r = torch.tensor(rates0, requires_grad=True)
            pi = torch.tensor(wl.pi[:2], requires_grad=True)
            subst = GeneralNonSymmetricSubstitutionModel(None, NucleotideDataType(None),
                                                         Parameter(None, torch.arange(12)), Parameter(None, r),
                                                         Parameter(None, pi), True)
            return tree, sp, subst, site, [leaves[0], r, pi, leaves[-1]]

        tree, sp, subst, site, leaves = build()
        ref = Reference(None, sp, tree, subst, site)
        ref.rescale = True
        want = ref().reshape(-1)
        gwant = torch.autograd.grad(want.sum(), leaves)
        tree, sp, subst, site, leaves = build()
        like = TreeLikelihoodModel(None, sp, tree, subst, site, precision=precision)
        like.rescale = True
        got = like().reshape(-1)
        got.sum().backward()
        ltol, gtol = (1e-10, 1e-9) if precision == "f64" else (1e-6, 1e-4)
        np.testing.assert_allclose(got.detach().numpy(), want.detach().numpy(), rtol=ltol)
        for x, w in zip(leaves, gwant):
            np.testing.assert_allclose(x.grad.numpy(), w.numpy(), rtol=gtol, atol=gtol * float(w.abs().max()))
    finally:
        torch.set_default_dtype(torch.float32)
