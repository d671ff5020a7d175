"""Pattern slabs (TT_OPT_SLAB_PATTERNS): the gradient recomputed one slab of
patterns at a time equals the gradient from partials stored for the whole
alignment, in every 4-state kernel shape and both precisions.

Patterns are independent, so each slab's tiles carry the same arithmetic as
the whole-alignment pass; only the FP64 sums over slabs are grouped
differently.  Tolerances: lnL relative 1e-14, gradients relative 1e-12.
"""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from torchtree_gb300 import _native

    _native.load()


def _problem(T=40, sites=4000, b=2, K=4, seed=71):
    from torchtree_gb300 import patterns, site_models, substitution, synthetic

    rng = np.random.default_rng(seed)
    topo = synthetic.yule_topology(T, rng)
    pi = rng.dirichlet(np.ones(4))
    exch = rng.dirichlet(np.ones(6))
    q = synthetic.normalised_q_np(synthetic.gtr_q_np(exch, pi), pi)
    rates_np = synthetic.discrete_gamma_np(0.5, K)
    node_bl = np.concatenate([rng.exponential(0.1, 2 * T - 3), [0.0]])
    seqs = synthetic.simulate_alignment(topo, node_bl, q, pi, rates_np, np.full(K, 1.0 / K), sites, rng)
    ca = patterns.compress(seqs)
    dev = torch.device("cuda")
    pit = torch.tensor(pi, dtype=torch.float64)
    qt = substitution.gtr_q(torch.tensor(exch, dtype=torch.float64), pit)
    lam, u, w = (t.expand(b, *t.shape).to(dev).contiguous() for t in substitution.eigen_system(qt, pit))
    rates, probs = site_models.gamma_rates(torch.tensor([[0.5]] * b, dtype=torch.float64), K)
    bls = torch.tensor(np.stack([node_bl * (1 + 0.2 * i) for i in range(b)]), dtype=torch.float64, device=dev)
    eig = [lam, u, w, bls, rates.to(dev).contiguous()]
    return topo, ca, eig, probs.expand(b, K).to(dev).contiguous(), pit.to(dev), b, K


def _evaluate(eng, eig, props, pi, rescale, second=False):
    eng.set_eigen(*eig)
    lnl = eng.log_likelihood(props, pi, rescale=rescale, keep_partials=True)
    out = [x.cpu().numpy() for x in (lnl, *eng.gradient(props, pi, want_matrices=True))]
    if second:  # slab mode recomputes: a second gradient needs no new post-order
        again = [x.cpu().numpy() for x in eng.gradient(props, pi, want_matrices=True)]
        for a, g in zip(again, out[1:]):
            np.testing.assert_array_equal(a, g)
    assert eng.device_status() == 0
    return out


def _close(got, want):
    np.testing.assert_allclose(got[0], want[0], rtol=1e-14)
    for g, w in zip(got[1:], want[1:]):
        np.testing.assert_allclose(g, w, rtol=1e-12, atol=1e-12 * np.abs(w).max())


@pytest.mark.parametrize("precision,options", [
    ("f64", {}),
    ("f32", {}),
    ("f32", {"TT_OPT_INPLACE_ADJOINT": 0}),
    ("f32", {"TT_OPT_PAIR_THREADS": 1}),
    ("f32", {"TT_OPT_PRODUCER_WARP": 0}),
])
def test_slabbed_gradient_equals_whole_alignment(precision, options):
    from torchtree_gb300 import _native
    from torchtree_gb300.engine import LikelihoodEngine

    topo, ca, eig, props, pi, b, K = _problem()
    N = ca.weights.shape[0]
    assert N > 1600  # several slabs of 512, the last one ragged
    eng = LikelihoodEngine(topo.postorder, topo.tip_count, 4, K, ca.codes, ca.table, ca.weights, batch=b,
                           precision=precision)
    for name, v in options.items():
        eng.set_option(getattr(_native, name), v)
    rescale = precision == "f32"
    assert eng.get_option(_native.TT_OPT_SLAB_PATTERNS) == 0
    whole = _evaluate(eng, eig, props, pi, rescale)
    whole_bytes = eng.workspace_bytes
    for slab, held in ((512, 512), (700, 1024), (1536, 1536)):
        eng.set_option(_native.TT_OPT_SLAB_PATTERNS, slab)
        assert eng.get_option(_native.TT_OPT_SLAB_PATTERNS) == held
        assert eng.workspace_bytes < whole_bytes
        _close(_evaluate(eng, eig, props, pi, rescale, second=True), whole)
    eng.set_option(_native.TT_OPT_SLAB_PATTERNS, 10 * N)  # at least the alignment: no slabs
    assert eng.get_option(_native.TT_OPT_SLAB_PATTERNS) == 0
    assert eng.workspace_bytes == whole_bytes
    _close(_evaluate(eng, eig, props, pi, rescale), whole)


def test_plan_picks_slabs_when_the_gradient_buffers_exceed_the_budget():
    from torchtree_gb300 import _native
    from torchtree_gb300.engine import LikelihoodEngine

    topo, ca, eig, props, pi, b, K = _problem(seed=72)
    args = (topo.postorder, topo.tip_count, 4, K, ca.codes, ca.table, ca.weights)
    whole = LikelihoodEngine(*args, batch=b, precision="f32")
    want = _evaluate(whole, eig, props, pi, True)
    os.environ["TT_GRADIENT_BUDGET_BYTES"] = str(whole.workspace_bytes // 3)
    try:
        eng = LikelihoodEngine(*args, batch=b, precision="f32")
    finally:
        del os.environ["TT_GRADIENT_BUDGET_BYTES"]
    slab = eng.get_option(_native.TT_OPT_SLAB_PATTERNS)
    assert slab > 0 and slab % 512 == 0
    assert eng.workspace_bytes < whole.workspace_bytes
    _close(_evaluate(eng, eig, props, pi, True), want)


def _wide_problem(kind, precision):
    from torchtree_gb300 import datatype, patterns, site_models, substitution, synthetic

    if kind == "protein":
        wl = synthetic.protein_workload("p", tip_count=30, site_count=3000, batch=2, seed=81, shape=0.5)
    else:
        wl = synthetic.codon_workload("c", tip_count=20, site_count=3000, batch=2, seed=82, shape=0.5)
    dt = datatype.get(wl.data_type)
    ca = patterns.compress(wl.sequences, dt)
    b, K, S = wl.branch_lengths.shape[0], wl.categories, dt.state_count
    pi = torch.tensor(wl.pi, dtype=torch.float64)
    ex = torch.tensor(wl.exch, dtype=torch.float64)
    if wl.model == "mg94":
        q = substitution.mg94_q(torch.ones_like(ex[:, :1]), ex[:, 1:2], ex[:, :1], pi)
    else:
        q = substitution.general_symmetric_q(ex, pi, S)
    dev = torch.device("cuda")
    lam, u, w = (t.to(dev).contiguous() for t in substitution.eigen_system(q, pi))
    rates, probs = site_models.gamma_rates(torch.tensor(wl.shape, dtype=torch.float64), K)
    bls = torch.cat([torch.tensor(wl.branch_lengths), torch.zeros(b, 1, dtype=torch.float64)], -1)
    eig = [lam, u, w, bls.to(dev).contiguous(), rates.to(dev).contiguous()]
    return wl.topology, ca, S, K, b, eig, probs.expand(b, K).to(dev).contiguous(), pi.to(dev)


@pytest.mark.parametrize("kind,precision,tc,tca", [
    ("protein", "f64", None, None), ("protein", "f32", None, None),
    ("codon", "f64", None, None), ("codon", "f32", 1, 1), ("codon", "f32", 0, 1), ("codon", "f32", 1, 0),
])
def test_wide_slabs_equal_the_whole_alignment(kind, precision, tc, tca):
    """20- and 61-state plans run both passes slab by slab.  Per-pattern
    results (site lnL) are bit-identical; lnL differs by the grouping of its
    FP64 sum; gradients by the grouping of the chunk sums (FP64 plans 1e-12,
    FP32 plans 1e-5 of the largest entry).  The first gradient after
    tt_log_likelihood reuses the last slab's post-order, the second
    recomputes it: both are bit-identical."""
    from torchtree_gb300 import _native
    from torchtree_gb300.engine import LikelihoodEngine

    topo, ca, S, K, b, eig, props, pi = _wide_problem(kind, precision)
    N = ca.weights.shape[0]
    assert N > 1100
    eng = LikelihoodEngine(topo.postorder, topo.tip_count, S, K, ca.codes, ca.table, ca.weights, batch=b,
                           precision=precision)
    if tc is not None:
        eng.set_option(_native.TT_OPT_TENSOR_CORES, tc)
    if tca is not None:
        eng.set_option(_native.TT_OPT_TENSOR_CORE_ADJOINT, tca)
        assert eng.get_option(_native.TT_OPT_TENSOR_CORE_ADJOINT) == tca

    def run(second=False):
        eng.set_eigen(*eig)
        lnl, site = eng.log_likelihood(props, pi, rescale=True, keep_partials=True, site=True)
        out = [x.cpu().numpy() for x in (lnl, site, *eng.gradient(props, pi, want_matrices=True))]
        if second:
            again = [x.cpu().numpy() for x in eng.gradient(props, pi, want_matrices=True)]
            for a, g in zip(again, out[2:]):
                np.testing.assert_array_equal(a, g)
        assert eng.device_status() == 0
        return out

    whole = run()
    whole_bytes = eng.workspace_bytes
    gtol = 1e-12 if precision == "f64" else 1e-5
    for slab in (512, 1024):
        eng.set_option(_native.TT_OPT_SLAB_PATTERNS, slab)
        assert eng.get_option(_native.TT_OPT_SLAB_PATTERNS) == slab
        assert eng.workspace_bytes < whole_bytes
        got = run(second=True)
        np.testing.assert_allclose(got[0], whole[0], rtol=1e-13)
        np.testing.assert_array_equal(got[1], whole[1])
        for g, w in zip(got[2:], whole[2:]):
            np.testing.assert_allclose(g, w, rtol=gtol, atol=gtol * np.abs(w).max())
    eng.set_option(_native.TT_OPT_SLAB_PATTERNS, 0)
    assert eng.workspace_bytes == whole_bytes
    again = run()
    for a, w in zip(again, whole):
        np.testing.assert_array_equal(a, w)
