"""GPU parity: the sm_103a engine against the reference's own numbers.

Every case of tests/golden/likelihood.json (produced by the reference
torchtree's TreeLikelihoodModel + autograd in FP64) is evaluated through the
package's public path (pattern compression -> C-ABI plan -> kernels ->
autograd chain):

* FP64 drop-in: lnL within 1e-10 relative, gradients within 1e-10 of the
  largest component (``rtol=atol/max = 1e-10``);
* FP32 rescaled: lnL within 1e-6 relative, gradients within 1e-4 of the
  largest component.
"""
import math

import numpy as np
import pytest
import torch

from tests.oracle_cases import GRAD_KEYS, as_np, record_inputs

pytestmark = pytest.mark.gpu

F64_RTOL = 1e-10
F32_LNL_RTOL = 1e-6
F32_GRAD_TOL = 1e-4


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from torchtree_gb300 import _native

    _native.load()


def _keys():
    import json

    from tests.conftest import GOLDEN

    return sorted(json.loads((GOLDEN / "likelihood.json").read_text()))


def engine_eval(rec, precision, rescale=None, route="eigen"):
    """lnL [b] and gradients of sum(lnL) w.r.t. the record's leaves, via the package.

    The 4x4 eigendecompositions run on the CPU (one LAPACK call per matrix),
    so a batch member's inputs are bit-identical to its single evaluation.
    """
    from torchtree_gb300 import datatype, patterns, site_models, substitution
    from torchtree_gb300.likelihood import PhyloLikelihood
    from torchtree_gb300.tree import Topology

    dev = torch.device("cuda")
    x = {k: v.detach().to(dev).requires_grad_() for k, v in record_inputs(rec, False).items()}
    batched = x["bl"].dim() == 2
    b = x["bl"].shape[0] if batched else 1
    lead = lambda t: t if batched else t.unsqueeze(0)  # noqa: E731
    topo = Topology(rec["postorder"], rec["names"])
    dt = datatype.get(rec.get("data_type", "nucleotide"))
    S = dt.state_count
    ca = patterns.compress(rec["sequences"], dt, use_ambiguities=rec.get("use_ambiguities", False),
                           tip_states=rec.get("tip_states", False))
    if rec["site_model"] == "weibull":
        rates, probs = site_models.weibull_rates(lead(x["shape"]), rec["categories"],
                                                 lead(x["invariant"]) if "invariant" in x else None)
    elif rec["site_model"] == "constant":
        rates = torch.ones(b, 1, dtype=torch.float64, device=dev)
        probs = torch.ones(b, 1, dtype=torch.float64, device=dev)
    else:
        rates = torch.tensor(rec["category_rates"], dtype=torch.float64, device=dev).expand(b, -1)
        probs = torch.full((b, rec["categories"]), 1.0 / rec["categories"], dtype=torch.float64, device=dev)
    K = rates.shape[-1]
    probs = probs.expand(b, K)
    lik = PhyloLikelihood(topo, ca, S, K, batch=b, precision=precision)
    if rescale is not None:
        lik.rescale = rescale
    bls = lik.node_branch_lengths(lead(x["bl"]))
    if rec["model"] == "jc69":
        t = bls.unsqueeze(-1) * rates.unsqueeze(-2)
        e = torch.exp(-4.0 / 3.0 * t)
        eye = torch.eye(4, dtype=torch.float64, device=dev)
        mats = (0.25 - 0.25 * e)[..., None, None] * (1 - eye) + (0.25 + 0.75 * e)[..., None, None] * eye
        pi = torch.full((b, 4), 0.25, dtype=torch.float64, device=dev)
        lnl = lik.evaluate_matrices(mats, probs, pi)
    else:
        pi = lead(x["pi"])
        ex = lead(x["exch"])
        if rec["model"] == "gtr":
            q = substitution.gtr_q(ex, pi)
        elif rec["model"] == "hky":
            q = substitution.hky_q(ex, pi)
        elif rec["model"] == "general":
            q = substitution.general_symmetric_q(ex, pi, S)
        else:  # mg94: (kappa, omega), alpha = 1
            q = substitution.mg94_q(torch.ones_like(ex[..., 0:1]), ex[..., 1:2], ex[..., 0:1], pi)
        if route == "q":  # dlnL/dQ through the matrix-exponential derivative
            lnl = lik.evaluate_rate_matrix(substitution.normalise(q, pi), pi, bls, rates, probs, pi)
        else:
            lam, u, w = (t.to(dev) for t in substitution.eigen_system(q.cpu(), pi.cpu()))
            lnl = lik.evaluate_eigen(lam, u, w, bls, rates, probs, pi)
    leaves = [(k, g) for k, g in GRAD_KEYS if k in x and g in rec]
    grads = torch.autograd.grad(lnl.sum(), [x[k] for k, _ in leaves])
    return lnl.detach().cpu().numpy(), {g: gr.cpu().numpy() for (_, g), gr in zip(leaves, grads)}, lik


@pytest.mark.parametrize("key", _keys())
def test_fp64_dropin_matches_reference(golden_likelihood, key):
    rec = golden_likelihood[key]
    lnl, grads, _ = engine_eval(rec, "f64")
    np.testing.assert_allclose(lnl, rec["lnl"], rtol=F64_RTOL)
    for g, got in grads.items():
        exp = as_np(rec[g])
        np.testing.assert_allclose(got, exp, rtol=F64_RTOL, atol=F64_RTOL * np.abs(exp).max(), err_msg=g)


@pytest.mark.parametrize("key", _keys())
def test_fp32_rescaled_matches_reference(golden_likelihood, key):
    rec = golden_likelihood[key]
    lnl, grads, _ = engine_eval(rec, "f32")
    np.testing.assert_allclose(lnl, rec["lnl"], rtol=F32_LNL_RTOL)
    for g, got in grads.items():
        exp = as_np(rec[g])
        np.testing.assert_allclose(got, exp, rtol=F32_GRAD_TOL, atol=F32_GRAD_TOL * np.abs(exp).max(),
                                   err_msg=g)


@pytest.mark.parametrize("precision", ["f64", "f32"])
@pytest.mark.parametrize("key", [k for k in _keys() if k != "tiny_jc69"])
def test_rate_matrix_gradient_route_matches_reference(golden_likelihood, key, precision):
    rec = golden_likelihood[key]
    lnl, grads, _ = engine_eval(rec, precision, route="q")
    tol = F64_RTOL if precision == "f64" else F32_GRAD_TOL
    np.testing.assert_allclose(lnl, rec["lnl"], rtol=F64_RTOL if precision == "f64" else F32_LNL_RTOL)
    for g, got in grads.items():
        exp = as_np(rec[g])
        np.testing.assert_allclose(got, exp, rtol=tol, atol=tol * np.abs(exp).max(), err_msg=g)


def test_tiny_known_answer_on_gpu(golden_likelihood):
    lnl, _, _ = engine_eval(golden_likelihood["tiny_jc69"], "f64")
    assert abs(lnl[0] - (-83.329016)) < 1e-6  # test_tree_likelihood.py:84


def test_underflow_switch_is_sticky(golden_likelihood):
    rec = golden_likelihood["gtr_w4_t700_underflow"]
    lnl, _, lik = engine_eval(rec, "f64")
    assert lik.rescale is True  # tree_likelihood.py:378-388
    np.testing.assert_allclose(lnl, rec["lnl"], rtol=F64_RTOL)


def test_batch_element_equals_single(golden_likelihood):
    # test_tree_likelihood.py:204-297: a batch member equals its own evaluation exactly
    rec = golden_likelihood["hky_w4_t12_b3"]
    lnl_b, _, _ = engine_eval(rec, "f64")
    single = dict(rec)
    for k in ("branch_lengths", "exch", "pi", "shape"):
        single[k] = rec[k][1]
    lnl_1, _, _ = engine_eval(single, "f64")
    assert lnl_b[1] == lnl_1[0]
    lnl_b32, _, _ = engine_eval(rec, "f32")
    lnl_132, _, _ = engine_eval(single, "f32")
    assert lnl_b32[1] == lnl_132[0]


def test_rescaled_equals_unscaled_fp64(golden_likelihood):
    rec = golden_likelihood["gtr_w4_t69"]
    a, _, _ = engine_eval(rec, "f64", rescale=False)
    b_, _, _ = engine_eval(rec, "f64", rescale=True)
    np.testing.assert_allclose(a, b_, rtol=1e-13)


def test_finite_differences_fp64(golden_likelihood):
    """Central differences of the engine's own FP64 lnL vs its adjoint gradient."""
    from torchtree_gb300 import datatype, patterns, site_models, substitution
    from torchtree_gb300.likelihood import PhyloLikelihood
    from torchtree_gb300.tree import Topology

    rec = golden_likelihood["gtr_w4_t9_ambiguities"]
    dev = torch.device("cuda")
    topo = Topology(rec["postorder"], rec["names"])
    ca = patterns.compress(rec["sequences"], datatype.Nucleotide(), use_ambiguities=True)
    lik = PhyloLikelihood(topo, ca, 4, 4, batch=1, precision="f64")

    def f(bl, exch, pi, shape):
        rates, probs = site_models.weibull_rates(shape, 4)
        q = substitution.gtr_q(exch, pi)
        lam, u, w = substitution.eigen_system(q, pi)
        return lik.evaluate_eigen(lam, u, w, lik.node_branch_lengths(bl), rates, probs.expand(1, 4), pi).sum()

    def t(v):
        x = torch.tensor(v, dtype=torch.float64, device=dev)
        return (x if x.dim() == 2 else x.unsqueeze(0)).requires_grad_()

    args = [t(rec["branch_lengths"]), t(rec["exch"]), t(rec["pi"]), t(rec["shape"])]
    grads = torch.autograd.grad(f(*args), args)
    for a, g in zip(args, grads):
        flat = a.detach().clone()
        fd = torch.empty_like(flat)
        for i in range(flat.numel()):
            h = 1e-6 * max(1.0, abs(flat.view(-1)[i].item()))
            up = flat.clone(); up.view(-1)[i] += h
            dn = flat.clone(); dn.view(-1)[i] -= h
            with torch.no_grad():
                vals = []
                for z in (up, dn):
                    call = [z if b is a else b.detach() for b in args]
                    vals.append(f(*call).item())
            fd.view(-1)[i] = (vals[0] - vals[1]) / (2 * h)
        np.testing.assert_allclose(g.cpu().numpy(), fd.cpu().numpy(), rtol=1e-5, atol=1e-6)


def test_functional_mirrors_match_oracle(golden_likelihood):
    """torchtree_gb300.functional vs the oracle's restatement of the same functions."""
    from oracle import likelihood as OL
    from tests.oracle_cases import model_pieces, tips_from_record
    from torchtree_gb300 import functional as F

    rec = golden_likelihood["hky_w4_t12_b3"]
    x = record_inputs(rec, requires_grad=False)
    tips, w = tips_from_record(rec)
    q, pi, rates, probs, bls = model_pieces(rec, x)
    mats = OL.p_t_symmetric(q, pi, bls.unsqueeze(-1) * rates.unsqueeze(-2)).detach()
    freqs = pi.unsqueeze(-2).detach()
    props = probs.unsqueeze(-1).unsqueeze(-1).detach()
    parts = list(tips) + [None] * (len(tips) - 1)
    post = rec["postorder"]
    for ref_fn, gpu_fn in ((OL.treelikelihood_discrete, F.calculate_treelikelihood_discrete),
                           (OL.treelikelihood_discrete_rescaled, F.calculate_treelikelihood_discrete_rescaled)):
        m1 = mats.clone().requires_grad_()
        expected = ref_fn(parts, w, post, m1, freqs, props)
        (g_ref,) = torch.autograd.grad(expected.sum(), [m1])
        m2 = mats.cuda().requires_grad_()
        got = gpu_fn(parts, w, post, m2, freqs.cuda(), props.cuda())
        assert got.shape == expected.shape
        np.testing.assert_allclose(got.detach().cpu().numpy(), expected.detach().numpy(), rtol=1e-12)
        (g_gpu,) = torch.autograd.grad(got.sum(), [m2])
        np.testing.assert_allclose(g_gpu.cpu().numpy(), g_ref.numpy(), rtol=1e-9,
                                   atol=1e-9 * g_ref.abs().max().item())
    # tip-state variants
    srec = dict(rec, tip_states=True)
    stips, sw = tips_from_record(srec)
    sparts = list(stips) + [None] * (len(stips) - 1)
    expected = OL.treelikelihood_tip_states_discrete_rescaled(sparts, sw, post, mats, freqs, props)
    got = F.calculate_treelikelihood_tip_states_discrete_rescaled(sparts, sw, post, mats.cuda(), freqs.cuda(),
                                                                  props.cuda())
    np.testing.assert_allclose(got.cpu().numpy(), expected.numpy(), rtol=1e-12)
    # single-category function (tree_likelihood.py:14-37)
    m0 = mats[..., 0, :, :]
    expected = OL.treelikelihood(parts, w, post, m0, freqs)
    got = F.calculate_treelikelihood(parts, w, post, m0.cuda(), freqs.cuda())
    np.testing.assert_allclose(got.cpu().numpy(), expected.numpy(), rtol=1e-12)


def test_large_tree_properties():
    """Size-independent checks at a larger size: FP32 vs FP64, determinism, batch slicing."""
    from torchtree_gb300 import patterns, site_models, substitution, synthetic
    from torchtree_gb300.likelihood import PhyloLikelihood, batch_inputs

    wl = synthetic.dna_workload("prop", tip_count=400, site_count=6000, batch=4, seed=21, model="gtr",
                                site_model="gamma", shape=0.5)
    ca = patterns.compress(wl.sequences)
    dev = torch.device("cuda")
    bl, exch, pi, shape = batch_inputs(wl, dev)
    rates, probs = site_models.gamma_rates(shape, 4)
    q = substitution.gtr_q(exch, pi)
    lam, u, w = substitution.eigen_system(q, pi)
    out = {}
    for prec in ("f64", "f32"):
        lik = PhyloLikelihood(wl.topology, ca, 4, 4, batch=4, precision=prec)
        lik.rescale = True
        bls = lik.node_branch_lengths(bl)
        b = bl.clone().requires_grad_()
        l1 = lik.evaluate_eigen(lam, u, w, lik.node_branch_lengths(b), rates, probs, pi)
        (g1,) = torch.autograd.grad(l1.sum(), [b])
        l2 = lik.evaluate_eigen(lam, u, w, bls, rates, probs, pi)
        assert torch.equal(l1.detach(), l2.detach())  # deterministic
        out[prec] = (l1.detach().cpu().numpy(), g1.cpu().numpy())
    np.testing.assert_allclose(out["f32"][0], out["f64"][0], rtol=F32_LNL_RTOL)
    g64 = out["f64"][1]
    np.testing.assert_allclose(out["f32"][1], g64, rtol=F32_GRAD_TOL, atol=F32_GRAD_TOL * np.abs(g64).max())
    assert math.isfinite(float(out["f64"][0].sum()))


def test_forward_without_gradient_matches(golden_likelihood):
    """keep_partials=0 (forward only, no HBM partials) gives the same lnL."""
    rec = golden_likelihood["gtr_w4_t69"]
    lnl, _, lik = engine_eval(rec, "f32")
    eng = lik.engine
    # the last forward kept partials; rerun without keeping them on the same matrices
    with torch.no_grad():
        p = torch.full((1, 4), 0.25, dtype=torch.float64, device="cuda")
        f = torch.tensor(rec["pi"], dtype=torch.float64, device="cuda").reshape(1, 4)
        a = eng.log_likelihood(p, f, rescale=True, keep_partials=False)
        b = eng.log_likelihood(p, f, rescale=True, keep_partials=True)
    assert torch.equal(a, b)
    np.testing.assert_allclose(a.cpu().numpy(), rec["lnl"], rtol=F32_LNL_RTOL)
    assert eng.device_status() == 0


def test_pair_thread_kernels_match_one_thread_kernels():
    """FP32 4-state kernels: one thread per (pattern, category pair) vs one per
    pattern, and the adjoint with a shared-memory stack vs the one that stores
    outside partials over the post-order tiles (which consumes them), with all
    category pairs of a pattern in one thread or on adjacent threads."""
    from torchtree_gb300 import _native, patterns, site_models, substitution, synthetic
    from torchtree_gb300.engine import LikelihoodEngine

    for K, shape in ((4, 0.5), (1, 1.0), (8, 0.7)):
        wl = synthetic.dna_workload("pt", tip_count=70, site_count=500, batch=2, seed=51 + K, shape=shape,
                                    categories=K, site_model="gamma")
        ca = patterns.compress(wl.sequences)
        dev = torch.device("cuda")
        pi = torch.tensor(wl.pi, dtype=torch.float64)
        q = substitution.gtr_q(torch.tensor(wl.exch, dtype=torch.float64), pi)
        lam, u, w = (t.to(dev).contiguous() for t in substitution.eigen_system(q, pi))
        rates, probs = site_models.gamma_rates(torch.tensor(wl.shape, dtype=torch.float64), K)
        b = wl.branch_lengths.shape[0]
        bls = torch.cat([torch.tensor(wl.branch_lengths), torch.zeros(b, 1, dtype=torch.float64)], -1).to(dev)
        eig = [lam, u, w, bls.contiguous(), rates.to(dev).contiguous()]
        props, pid = probs.expand(b, K).to(dev).contiguous(), pi.to(dev)
        eng = LikelihoodEngine(wl.topology.postorder, wl.topology.tip_count, 4, K, ca.codes, ca.table, ca.weights,
                               batch=b, precision="f32")
        out = {}
        modes = {"stack": (0, 0, 0), "inplace": (0, 1, 0), "pair": (1, 0, 0), "pair_adjoint": (0, 1, 1)}
        for mode, (pair, inplace, pair_adjoint) in modes.items():
            eng.set_option(_native.TT_OPT_PAIR_THREADS, pair)
            eng.set_option(_native.TT_OPT_INPLACE_ADJOINT, inplace)
            eng.set_option(_native.TT_OPT_PAIR_ADJOINT, pair_adjoint)
            eng.set_eigen(*eig)
            lnl = eng.log_likelihood(props, pid, rescale=True, keep_partials=True)
            dP, dpi, dc = eng.gradient(props, pid, want_matrices=True)
            out[mode] = (lnl.cpu().numpy(), dP.cpu().numpy(), dpi.cpu().numpy(), dc.cpu().numpy())
            if inplace:  # the post-order tiles are gone: a second adjoint is refused
                with pytest.raises(_native.EngineError):
                    eng.gradient(props, pid)
        for mode in ("inplace", "pair", "pair_adjoint"):
            # identical FP32 partials; the FP64 root sums run in a different order
            np.testing.assert_allclose(out[mode][0], out["stack"][0], rtol=1e-13)
            for a_, b_ in zip(out["stack"][1:], out[mode][1:]):
                np.testing.assert_allclose(b_, a_, rtol=1e-5, atol=1e-5 * np.abs(a_).max())


def _newick_shape(shape: str, T: int) -> str:
    names = [f"t{i}" for i in range(T)]
    if shape == "caterpillar":
        s = names[0]
        for n in names[1:]:
            s = f"({s},{n})"
        return s + ";"

    def bal(xs):
        if len(xs) == 1:
            return xs[0]
        h = len(xs) // 2
        return f"({bal(xs[:h])},{bal(xs[h:])})"

    return bal(names) + ";"


@pytest.mark.gpu
@pytest.mark.parametrize("K", [1, 3, 5])
@pytest.mark.parametrize("shape,T", [("balanced", 2), ("caterpillar", 3), ("balanced", 4), ("caterpillar", 50),
                                     ("balanced", 64)])
def test_fp32_adjoints_on_edge_trees(shape, T, K):
    """FP32 adjoints against the FP64 engine on trees that drive the in-place
    adjoint's paths: a root with tips only, carried children only (caterpillar),
    a root with two cherries (one child stored in place), and a balanced tree
    (half of all internal children stored); odd category counts pad a pair."""
    from torchtree_gb300 import _native, patterns, site_models, substitution, synthetic
    from torchtree_gb300.engine import LikelihoodEngine
    from torchtree_gb300.tree import Topology

    rng = np.random.default_rng(7 * T + K)
    topo = Topology.from_newick(_newick_shape(shape, T))
    pi = rng.dirichlet(np.ones(4))
    exch = rng.dirichlet(np.ones(6))
    q = synthetic.normalised_q_np(synthetic.gtr_q_np(exch, pi), pi)
    rates_np = synthetic.discrete_gamma_np(0.6, K)
    node_bl = np.concatenate([rng.exponential(0.2, 2 * T - 3), [0.0]])
    seqs = synthetic.simulate_alignment(topo, node_bl, q, pi, rates_np, np.full(K, 1.0 / K), 700, rng)
    ca = patterns.compress(seqs)
    dev = torch.device("cuda")
    b = 2
    pit = torch.tensor(pi, dtype=torch.float64)
    qt = substitution.gtr_q(torch.tensor(exch, dtype=torch.float64), pit)
    lam, u, w = (t.expand(b, *t.shape).to(dev).contiguous() for t in substitution.eigen_system(qt, pit))
    rates, probs = site_models.gamma_rates(torch.tensor([[0.6]] * b, dtype=torch.float64), K)
    bls = torch.tensor(np.stack([node_bl, node_bl * 1.3]), dtype=torch.float64, device=dev)
    eig = [lam, u, w, bls, rates.to(dev).contiguous()]
    props, pid = probs.expand(b, K).to(dev).contiguous(), pit.to(dev)
    out = {}
    variants = [("f64", "f64", None, 0), ("f32", "f32", 1, 0), ("f32_stack", "f32", 0, 0)]
    if (K + 1) // 2 in (1, 2, 4):  # the pair-thread adjoint takes 1, 2 or 4 category pairs
        variants.append(("f32_pair_adjoint", "f32", 1, 1))
    for name, precision, inplace, pair_adjoint in variants:
        eng = LikelihoodEngine(topo.postorder, T, 4, K, ca.codes, ca.table, ca.weights, batch=b, precision=precision)
        if inplace is not None:
            eng.set_option(_native.TT_OPT_INPLACE_ADJOINT, inplace)
            eng.set_option(_native.TT_OPT_PAIR_ADJOINT, pair_adjoint)
        eng.set_eigen(*eig)
        lnl = eng.log_likelihood(props, pid, rescale=precision == "f32", keep_partials=True)
        dP, dpi, dc = eng.gradient(props, pid, want_matrices=True)
        out[name] = [x.cpu().numpy() for x in (lnl, dP, dpi, dc)]
    ref = out["f64"]
    for name in [v[0] for v in variants[1:]]:
        np.testing.assert_allclose(out[name][0], ref[0], rtol=1e-6)
        for got, want in zip(out[name][1:], ref[1:]):
            np.testing.assert_allclose(got, want, rtol=1e-4, atol=1e-4 * np.abs(want).max())


def test_bounded_wait_times_out_and_the_plan_stays_usable():
    """The failure path without a fault: a kernel waits, with the bounded wait
    of every staged kernel, on a barrier that nothing completes; after 1 ms it
    gives up and the plan's status word says so (read once, then reset).  The
    context and the plan stay usable: the next evaluation is unchanged."""
    from torchtree_gb300 import _native, patterns, site_models, substitution, synthetic
    from torchtree_gb300.likelihood import PhyloLikelihood, batch_inputs

    wl = synthetic.dna_workload("wait", tip_count=20, site_count=500, batch=2, seed=5, shape=0.5)
    lik = PhyloLikelihood(wl.topology, patterns.compress(wl.sequences), 4, 4, batch=2, precision="f32")
    bl, ex, pi, sh = batch_inputs(wl, torch.device("cuda"))

    def lnl():
        r, p = site_models.gamma_rates(sh, 4)
        return lik(bl, substitution.gtr_q(ex, pi), pi, r, p.expand(2, 4)).detach().cpu()

    before = lnl()
    assert lik.engine.device_status() == 0
    lik.engine.selftest_timeout(1_000_000)
    assert lik.engine.device_status() == _native.TT_ERR_DEVICE_TIMEOUT
    assert lik.engine.device_status() == 0
    assert torch.equal(lnl(), before)
