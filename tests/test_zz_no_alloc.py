"""tt_log_likelihood_static: the log-likelihood for callers that cannot allocate.

Callers that run under an application's own device-memory manager, or that
are handed device buffers by a host without the right to allocate, cannot
create a plan (tt_plan_create allocates its workspace).  They call
tt_log_likelihood_static, which keeps its scratch in a static device array.
This test calls it through the C ABI twice in a row, with different
matrices and rescaling settings, and checks each result against the
plan-based entry points on the same inputs (FP64 tolerance 1e-10 relative).
The file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

F64_RTOL = 1e-10


def _matrices(wl, scale, dev):
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
    return (mats.contiguous().to(dev), probs.expand(b, -1).contiguous().to(dev), pi.contiguous().to(dev))


def test_static_entry_point_matches_plan_path():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from torchtree_gb300 import _native, patterns, synthetic
    from torchtree_gb300.engine import LikelihoodEngine

    lib = _native.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    wl = synthetic.dna_workload("static", tip_count=150, site_count=3000, batch=2, seed=31, model="gtr",
                                site_model="weibull", shape=0.6, branch_mean=0.05)
    ca = patterns.compress(wl.sequences)
    T, N, K, b = wl.topology.tip_count, ca.pattern_count, wl.categories, 2
    post = np.ascontiguousarray(wl.topology.postorder, dtype=np.int32)
    codes = torch.tensor(ca.codes, dtype=torch.uint8, device=dev).contiguous()
    table = torch.tensor(ca.table, dtype=torch.float64, device=dev).contiguous()
    weights = torch.tensor(ca.weights, dtype=torch.float64, device=dev)
    plan = LikelihoodEngine(post, T, 4, K, ca.codes, ca.table, ca.weights, batch=b, precision="f64", device=dev)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    p32 = ctypes.POINTER(ctypes.c_int32)

    for call, (scale, rescale) in enumerate(((1.0, 1), (3.0, 0))):
        mats, props, freqs = _matrices(wl, scale, dev)
        plan.set_matrices(mats)
        expected = plan.log_likelihood(props, freqs, rescale=bool(rescale)).cpu().numpy()
        out = torch.full((b,), float("nan"), dtype=torch.float64, device=dev)
        rc = lib.tt_log_likelihood_static(T, post.ctypes.data_as(p32), 4, K, N, b, _native.ptr(codes),
                                          _native.ptr(table), int(ca.table.shape[0]), _native.ptr(weights),
                                          _native.ptr(mats), _native.ptr(props), _native.ptr(freqs), rescale,
                                          _native.ptr(out), stream)
        _native.check(rc)
        got = out.cpu().numpy()
        assert np.all(np.isfinite(got)), f"call {call}: {got}"
        np.testing.assert_allclose(got, expected, rtol=F64_RTOL, err_msg=f"call {call}")


def test_static_entry_point_rejects_oversized_problem():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
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
