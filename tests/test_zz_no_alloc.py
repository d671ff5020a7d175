"""tt_log_likelihood_static: the log-likelihood for callers that cannot allocate.

Callers that run under an application's own device-memory manager, or that
are handed device buffers by a host without the right to allocate, cannot
create a plan (tt_plan_create allocates its workspace).  They call
tt_log_likelihood_static, which keeps its scratch in a static device array.
These tests call it through the C ABI:

* twice in a row, with different matrices and rescaling settings, checking
  each result against the plan-based entry points on the same inputs and
  against the FP64 oracle (tolerance 1e-10 relative);
* a smaller problem (fewer tips and patterns) right after a larger one, so
  that a read of the larger call's leftover scratch would show;
* a tip code equal to code_count, which must give NaN (the table rows past
  code_count are NaN), not a stale or made-up value;
* an oversized problem and a capturing stream, which are refused.

The file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

F64_RTOL = 1e-10


def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _problem(tip_count, site_count, seed):
    from torchtree_gb300 import patterns, synthetic

    wl = synthetic.dna_workload("static", tip_count=tip_count, site_count=site_count, batch=2, seed=seed,
                                model="gtr", site_model="weibull", shape=0.6, branch_mean=0.05)
    return wl, patterns.compress(wl.sequences)


def _matrices(wl, scale):
    """FP64 transition matrices [b, B, K, 4, 4], category weights [b, K], frequencies [b, 4] (CPU)."""
    from torchtree_gb300 import site_models, substitution

    bl = torch.tensor(wl.branch_lengths * scale, dtype=torch.float64)
    pi = torch.tensor(wl.pi, dtype=torch.float64)
    q = substitution.gtr_q(torch.tensor(wl.exch, dtype=torch.float64), pi)
    lam, u, w = substitution.eigen_system(q, pi)
    rates, probs = site_models.weibull_rates(torch.tensor(wl.shape, dtype=torch.float64), wl.categories)
    bls = torch.cat([bl, torch.zeros(bl.shape[0], 1, dtype=torch.float64)], -1)
    t = bls.unsqueeze(-1) * rates.unsqueeze(-2)
    e = torch.exp(lam[:, None, None, :] * t.unsqueeze(-1))
    mats = (u[:, None, None] * e.unsqueeze(-2)) @ w[:, None, None]
    b = bl.shape[0]
    return mats.contiguous(), probs.expand(b, -1).contiguous(), pi.contiguous()


def _oracle(wl, ca, mats, probs, pi, rescale):
    from oracle import likelihood as OL

    tips = [torch.tensor(t) for t in ca.tip_partials()]
    parts = tips + [None] * (len(tips) - 1)
    fn = OL.treelikelihood_discrete_rescaled if rescale else OL.treelikelihood_discrete
    return fn(parts, torch.tensor(ca.weights), wl.topology.postorder_list(), mats, pi.unsqueeze(-2),
              probs[:, :, None, None]).reshape(-1).numpy()


def _call(lib, wl, ca, mats, probs, pi, rescale, codes=None, stream=None):
    from torchtree_gb300 import _native

    dev = torch.device("cuda", torch.cuda.current_device())
    T, N, K = wl.topology.tip_count, ca.pattern_count, wl.categories
    b = mats.shape[0]
    post = np.ascontiguousarray(wl.topology.postorder, dtype=np.int32)
    codes = torch.tensor(ca.codes, dtype=torch.uint8, device=dev).contiguous() if codes is None else codes
    table = torch.tensor(ca.table, dtype=torch.float64, device=dev).contiguous()
    weights = torch.tensor(ca.weights, dtype=torch.float64, device=dev)
    m, p, f = (x.to(dev).contiguous() for x in (mats, probs, pi))
    out = torch.full((b,), float("nan"), dtype=torch.float64, device=dev)
    stream = stream if stream is not None else torch.cuda.current_stream()
    rc = lib.tt_log_likelihood_static(T, post.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), 4, K, N, b,
                                      _native.ptr(codes), _native.ptr(table), int(ca.table.shape[0]),
                                      _native.ptr(weights), _native.ptr(m), _native.ptr(p), _native.ptr(f),
                                      rescale, _native.ptr(out), ctypes.c_void_p(stream.cuda_stream))
    return rc, out


def test_static_entry_point_matches_plan_path_and_oracle():
    _need_gpu()
    from torchtree_gb300 import _native
    from torchtree_gb300.engine import LikelihoodEngine

    lib = _native.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    wl, ca = _problem(150, 3000, 31)
    T, K, b = wl.topology.tip_count, wl.categories, 2
    plan = LikelihoodEngine(np.ascontiguousarray(wl.topology.postorder, dtype=np.int32), T, 4, K, ca.codes,
                            ca.table, ca.weights, batch=b, precision="f64", device=dev)
    for call, (scale, rescale) in enumerate(((1.0, 1), (3.0, 0))):
        mats, probs, pi = _matrices(wl, scale)
        plan.set_matrices(mats.to(dev))
        expected = plan.log_likelihood(probs.to(dev), pi.to(dev), rescale=bool(rescale)).cpu().numpy()
        rc, out = _call(lib, wl, ca, mats, probs, pi, rescale)
        _native.check(rc)
        got = out.cpu().numpy()
        assert np.all(np.isfinite(got)), f"call {call}: {got}"
        np.testing.assert_allclose(got, expected, rtol=F64_RTOL, err_msg=f"call {call} vs plan")
        np.testing.assert_allclose(got, _oracle(wl, ca, mats, probs, pi, rescale), rtol=F64_RTOL,
                                   err_msg=f"call {call} vs oracle")


def test_static_entry_point_smaller_problem_after_larger():
    _need_gpu()
    from torchtree_gb300 import _native

    lib = _native.load()
    for tips, sites, seed in ((300, 4000, 41), (37, 500, 42)):
        wl, ca = _problem(tips, sites, seed)
        mats, probs, pi = _matrices(wl, 1.0)
        rc, out = _call(lib, wl, ca, mats, probs, pi, 1)
        _native.check(rc)
        np.testing.assert_allclose(out.cpu().numpy(), _oracle(wl, ca, mats, probs, pi, 1), rtol=F64_RTOL,
                                   err_msg=f"{tips} tips x {ca.pattern_count} patterns")


def test_static_entry_point_out_of_range_code_gives_nan():
    _need_gpu()
    from torchtree_gb300 import _native

    lib = _native.load()
    wl, ca = _problem(20, 300, 43)
    mats, probs, pi = _matrices(wl, 1.0)
    codes = torch.tensor(ca.codes, dtype=torch.uint8, device="cuda").contiguous()
    codes[3, 5] = int(ca.table.shape[0])  # one past the last table row
    rc, out = _call(lib, wl, ca, mats, probs, pi, 1, codes=codes)
    _native.check(rc)
    assert torch.isnan(out).all(), out
    # and the next in-range call is clean again
    rc, out = _call(lib, wl, ca, mats, probs, pi, 1)
    _native.check(rc)
    np.testing.assert_allclose(out.cpu().numpy(), _oracle(wl, ca, mats, probs, pi, 1), rtol=F64_RTOL)


def test_static_entry_point_rejects_oversized_problem():
    _need_gpu()
    from torchtree_gb300 import _native, synthetic

    lib = _native.load()
    topo = synthetic.yule_topology(1024, np.random.default_rng(0))
    post = np.ascontiguousarray(topo.postorder, dtype=np.int32)
    dummy = torch.zeros(16, dtype=torch.float64, device="cuda")
    rc = lib.tt_log_likelihood_static(1024, post.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), 4, 8, 10, 64,
                                      _native.ptr(dummy), _native.ptr(dummy), 4, _native.ptr(dummy),
                                      _native.ptr(dummy), _native.ptr(dummy), _native.ptr(dummy), 1,
                                      _native.ptr(dummy), None)
    assert rc == _native.TT_ERR_INVALID_ARGUMENT
    assert "static scratch" in lib.tt_last_error().decode()


def test_static_entry_point_refuses_a_capturing_stream():
    _need_gpu()
    from torchtree_gb300 import _native

    lib = _native.load()
    wl, ca = _problem(12, 200, 44)
    mats, probs, pi = _matrices(wl, 1.0)
    dev = torch.device("cuda", torch.cuda.current_device())
    T, N, K, b = wl.topology.tip_count, ca.pattern_count, wl.categories, 2
    post = np.ascontiguousarray(wl.topology.postorder, dtype=np.int32)
    codes = torch.tensor(ca.codes, dtype=torch.uint8, device=dev).contiguous()
    table = torch.tensor(ca.table, dtype=torch.float64, device=dev).contiguous()
    weights = torch.tensor(ca.weights, dtype=torch.float64, device=dev)
    m, p, f = (x.to(dev).contiguous() for x in (mats, probs, pi))
    out = torch.zeros(b, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    side = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=side):
        rc = lib.tt_log_likelihood_static(T, post.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), 4, K, N, b,
                                          _native.ptr(codes), _native.ptr(table), int(ca.table.shape[0]),
                                          _native.ptr(weights), _native.ptr(m), _native.ptr(p), _native.ptr(f),
                                          1, _native.ptr(out), ctypes.c_void_p(side.cuda_stream))
        out.add_(1.0)  # the capture holds one node of its own
    assert rc == _native.TT_ERR_UNSUPPORTED
    assert "capturing" in lib.tt_last_error().decode()
    graph.replay()
    torch.cuda.synchronize()
    assert torch.equal(out.cpu(), torch.ones(b, dtype=torch.float64))
    # the stream is usable afterwards
    rc, res = _call(lib, wl, ca, mats, probs, pi, 1)
    _native.check(rc)
    np.testing.assert_allclose(res.cpu().numpy(), _oracle(wl, ca, mats, probs, pi, 1), rtol=F64_RTOL)
