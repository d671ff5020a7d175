"""Several plans in one call: ``tt_plans_log_likelihood`` / ``tt_plans_gradient``.

Plans on the default FP32 4-state kernels are merged into one post-order and
one adjoint launch over all their tiles; every other plan (FP64, another
category-pair count in a group of its own, a pattern-slab plan) runs its own
calls.  Each plan's lnL and gradients (dlnL/dpi, dlnL/dc and, through
``rate_matrix_gradient``, dlnL/dQ, dt, dr) must be bit-identical to the
plan's own calls, and the FP32 ones must match the FP64 oracle within the
FP32 tolerances of the parity tests.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _plan(tips, sites, K, seed, b, precision="f32", slab=0):
    from torchtree_gb300 import _native, patterns, site_models, substitution, synthetic
    from torchtree_gb300.engine import LikelihoodEngine

    wl = synthetic.dna_workload("m", tip_count=tips, site_count=sites, batch=b, seed=seed, shape=0.6,
                                categories=K, site_model="gamma", branch_mean=0.04)
    ca = patterns.compress(wl.sequences)
    dev = torch.device("cuda")
    eng = LikelihoodEngine(wl.topology.postorder, tips, 4, K, ca.codes, ca.table, ca.weights, batch=b,
                           precision=precision, device=dev)
    if slab:
        eng.set_option(_native.TT_OPT_SLAB_PATTERNS, slab)
    pi = torch.tensor(wl.pi, dtype=torch.float64, device=dev)
    q = substitution.normalise(substitution.gtr_q(torch.tensor(wl.exch, dtype=torch.float64, device=dev), pi), pi)
    lam, u, w = substitution.device_eigen(q, pi)
    rates, probs = site_models.gamma_rates(torch.tensor(wl.shape, dtype=torch.float64, device=dev), K)
    bls = torch.cat([torch.tensor(wl.branch_lengths, device=dev), torch.zeros(b, 1, dtype=torch.float64, device=dev)],
                    -1).contiguous()
    eig = (lam, u, w, bls, rates.contiguous())
    return dict(eng=eng, eig=eig, props=probs.expand(b, K).contiguous(), pi=pi)


def _alone(c):
    e = c["eng"]
    e.set_eigen(*c["eig"])
    lnl = e.log_likelihood(c["props"], c["pi"], rescale=True, keep_partials=True)
    _, dpi, dc = e.gradient(c["props"], c["pi"])
    dq, dt, dr = e.rate_matrix_gradient(*c["eig"])
    return [x.cpu().numpy() for x in (lnl, dpi, dc, dq, dt, dr)]


def test_plans_in_one_call_equal_their_own_calls():
    from torchtree_gb300.engine import plans_gradient, plans_log_likelihood

    cases = [_plan(40, 600, 4, 1, 2), _plan(150, 2000, 4, 2, 3), _plan(7, 90, 4, 3, 1),
             _plan(300, 5000, 3, 4, 2),   # 3 categories: the same pair count as 4, merged
             _plan(60, 700, 1, 5, 2),     # 1 category: a group of its own
             _plan(30, 400, 4, 6, 2, precision="f64"),  # FP64: its own calls
             _plan(90, 1800, 4, 7, 2, slab=512)]        # pattern slabs: its own calls
    alone = [_alone(c) for c in cases]
    for c in cases:
        c["eng"].set_eigen(*c["eig"])
    engines = [c["eng"] for c in cases]
    lnls = plans_log_likelihood(engines, [c["props"] for c in cases], [c["pi"] for c in cases], rescale=True,
                                keep_partials=True)
    grads = plans_gradient(engines, [c["props"] for c in cases], [c["pi"] for c in cases])
    merged = []
    for c, lnl, (dpi, dc) in zip(cases, lnls, grads):
        dq, dt, dr = c["eng"].rate_matrix_gradient(*c["eig"])
        merged.append([x.cpu().numpy() for x in (lnl, dpi, dc, dq, dt, dr)])
    for i, (a_, m_) in enumerate(zip(alone, merged)):
        for name, x, y in zip(("lnl", "dpi", "dc", "dq", "dt", "dr"), a_, m_):
            np.testing.assert_array_equal(y, x, err_msg=f"plan {i} {name}")


def test_merged_plans_match_the_oracle():
    """FP32 results of a merged call against the FP64 oracle (the reference's
    rescaled pruning with autograd), two plans of different trees."""
    from oracle import likelihood as OL
    from torchtree_gb300 import patterns, synthetic
    from torchtree_gb300.engine import plans_gradient, plans_log_likelihood

    specs = [(35, 500, 11), (80, 900, 12)]
    cases, refs = [], []
    for tips, sites, seed in specs:
        c = _plan(tips, sites, 4, seed, 2)
        wl = synthetic.dna_workload("m", tip_count=tips, site_count=sites, batch=2, seed=seed, shape=0.6,
                                    categories=4, site_model="gamma", branch_mean=0.04)
        ca = patterns.compress(wl.sequences)
        lam, u, w, bls, rates = (x.cpu() for x in c["eig"])
        mats = (u[:, None, None] * torch.exp(lam[:, None, None, :] * (bls[..., None] * rates[:, None, :])[..., None])
                .unsqueeze(-2)) @ w[:, None, None]
        tips_t = [torch.tensor(t) for t in ca.tip_partials()]
        ref = OL.treelikelihood_discrete_rescaled(tips_t + [None] * (tips - 1), torch.tensor(ca.weights),
                                                  wl.topology.postorder_list(), mats, c["pi"].cpu().unsqueeze(-2),
                                                  c["props"].cpu()[:, :, None, None]).reshape(-1)
        cases.append(c)
        refs.append(ref.numpy())
    for c in cases:
        c["eng"].set_eigen(*c["eig"])
    engines = [c["eng"] for c in cases]
    lnls = plans_log_likelihood(engines, [c["props"] for c in cases], [c["pi"] for c in cases], keep_partials=True)
    plans_gradient(engines, [c["props"] for c in cases], [c["pi"] for c in cases])
    for lnl, ref in zip(lnls, refs):
        np.testing.assert_allclose(lnl.cpu().numpy(), ref, rtol=1e-6)


@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_active_samples_equal_the_whole_batch_for_those_samples(precision):
    """TT_OPT_ACTIVE_SAMPLES: the pruning passes and their reductions over the
    first n samples only, alone and in a merged call (FP64 plans: each its own
    calls), give those samples' results of a call over every sample bit for
    bit."""
    from torchtree_gb300 import _native
    from torchtree_gb300.engine import plans_gradient, plans_log_likelihood

    cases = [_plan(120, 1500, 4, 21, 4, precision=precision), _plan(45, 700, 4, 22, 3, precision=precision)]
    full = [_alone(c) for c in cases]
    e0 = cases[0]["eng"]
    with pytest.raises(ValueError):
        e0.set_option(_native.TT_OPT_ACTIVE_SAMPLES, 5)  # more than the batch
    for n in (1, 2, 4):  # one plan's own calls
        e0.set_option(_native.TT_OPT_ACTIVE_SAMPLES, n)
        assert e0.get_option(_native.TT_OPT_ACTIVE_SAMPLES) == n
        got = _alone(cases[0])
        for name, x, y in zip(("lnl", "dpi", "dc", "dq", "dt", "dr"), full[0], got):
            np.testing.assert_array_equal(y[:n], x[:n], err_msg=f"n={n} {name}")
    active = (3, 2)  # a merged call with a different count per plan
    for c, n in zip(cases, active):
        c["eng"].set_option(_native.TT_OPT_ACTIVE_SAMPLES, n)
        c["eng"].set_eigen(*c["eig"])
    engines = [c["eng"] for c in cases]
    lnls = plans_log_likelihood(engines, [c["props"] for c in cases], [c["pi"] for c in cases], rescale=True,
                                keep_partials=True)
    grads = plans_gradient(engines, [c["props"] for c in cases], [c["pi"] for c in cases])
    for c, n, ref, lnl, (dpi, dc) in zip(cases, active, full, lnls, grads):
        dq, dt, dr = c["eng"].rate_matrix_gradient(*c["eig"])
        for name, x, y in zip(("lnl", "dpi", "dc", "dq", "dt", "dr"), ref, (lnl, dpi, dc, dq, dt, dr)):
            np.testing.assert_array_equal(y.cpu().numpy()[:n], x[:n], err_msg=f"merged n={n} {name}")
        c["eng"].set_option(_native.TT_OPT_ACTIVE_SAMPLES, 0)
        assert c["eng"].get_option(_native.TT_OPT_ACTIVE_SAMPLES) == 0
