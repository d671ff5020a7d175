"""GPU checks of the amino-acid / codon (wide-state) path beyond the golden cases.

* the tensor-core codon post-order (split-TF32 tcgen05) equals the CUDA-core
  kernel within FP32 rounding;
* a batch member equals its own evaluation, rescaled equals unscaled (FP64);
* FP32 against FP64 on a larger codon problem (lnL within 1e-6 relative).
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


def _setup(wl):
    from torchtree_gb300 import datatype, patterns, site_models, substitution

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
    return ca, S, K, b, [lam, u, w, bls.to(dev).contiguous(), rates.to(dev).contiguous()], \
        probs.expand(b, K).to(dev).contiguous(), pi.to(dev)


def _run(wl, precision, tc=True, rescale=True, grads=True, tca=None, halve_row=None, active=None):
    from torchtree_gb300.engine import LikelihoodEngine

    ca, S, K, b, eig, probs, pi = _setup(wl)
    table = ca.table
    if halve_row is not None:  # a code-table row that is not 0 / 1 (tip partials with weights)
        table = np.array(table, dtype=np.float64, copy=True)
        table[halve_row] *= 0.5
    old = os.environ.get("TT_WIDE_TC")
    os.environ["TT_WIDE_TC"] = "1" if tc else "0"
    try:
        eng = LikelihoodEngine(wl.topology.postorder, wl.topology.tip_count, S, K, ca.codes, table, ca.weights,
                               batch=b, precision=precision)
    finally:
        if old is None:
            del os.environ["TT_WIDE_TC"]
        else:
            os.environ["TT_WIDE_TC"] = old
    if tca is not None:
        from torchtree_gb300 import _native

        eng.set_option(_native.TT_OPT_TENSOR_CORE_ADJOINT, tca)
    if active is not None:
        from torchtree_gb300 import _native

        eng.set_option(_native.TT_OPT_ACTIVE_SAMPLES, active)
        assert eng.get_option(_native.TT_OPT_ACTIVE_SAMPLES) == active
    eng.set_eigen(*eig)
    lnl = eng.log_likelihood(probs, pi, rescale=rescale, keep_partials=grads)
    out = {"lnl": lnl.cpu().numpy()}
    if grads:
        _, dpi, dc = eng.gradient(probs, pi)
        dlam, du, dw, dt, dr = eng.eigen_gradient(*eig)
        out.update(dpi=dpi.cpu().numpy(), dc=dc.cpu().numpy(), dt=dt.cpu().numpy(), dr=dr.cpu().numpy(),
                   dlam=dlam.cpu().numpy(), du=du.cpu().numpy(), dw=dw.cpu().numpy())
    assert eng.device_status() == 0
    return out


def test_codon_tensor_core_matches_cuda_core():
    from torchtree_gb300 import synthetic

    wl = synthetic.codon_workload("c", tip_count=40, site_count=400, batch=2, seed=31, shape=0.5)
    a = _run(wl, "f32", tc=True)
    c = _run(wl, "f32", tc=False)
    np.testing.assert_allclose(a["lnl"], c["lnl"], rtol=1e-6)  # split-TF32 products, FP32 tensor accumulation
    np.testing.assert_allclose(a["dt"], c["dt"], rtol=1e-4, atol=1e-4 * np.abs(c["dt"]).max())


def _poison_free_memory(nbytes: int = 4 << 30):
    """Fill device memory with NaN and hand it back to the driver, so that the
    next plan's buffers likely start out as NaN where a kernel does not write
    them (padding patterns, unused rows): a result that reads such memory
    turns into NaN instead of passing on zeroed fresh pages."""
    free, _ = torch.cuda.mem_get_info()
    junk = torch.full((min(nbytes, free // 2) // 4,), float("nan"), device="cuda")
    del junk
    torch.cuda.synchronize()
    torch.cuda.empty_cache()


@pytest.mark.parametrize("tips,sites,batch,seed", [(40, 700, 2, 34), (7, 300, 3, 35)])
def test_codon_tensor_core_adjoint_matches_cuda_core(tips, sites, batch, seed):
    """The tcgen05 codon adjoint (split-TF32 GEMMs, 128-pattern tiles, outside
    partials stored in place) against the CUDA-core adjoint on the same stored
    post-order: every gradient within FP32 rounding of the largest entry, on a
    tree deep enough to store outside partials and on one whose internal
    children are few."""
    from torchtree_gb300 import synthetic

    wl = synthetic.codon_workload("c", tip_count=tips, site_count=sites, batch=batch, seed=seed, shape=0.5)
    _poison_free_memory()
    a = _run(wl, "f32", tca=1)
    c = _run(wl, "f32", tca=0)
    for key, val in a.items():
        assert np.isfinite(val).all(), key
    np.testing.assert_array_equal(a["lnl"], c["lnl"])  # the same post-order
    for key in ("dt", "dpi", "dc", "dr", "dlam", "du", "dw"):
        scale = np.abs(c[key]).max()
        np.testing.assert_allclose(a[key], c[key], rtol=1e-4, atol=1e-4 * scale, err_msg=key)
    d = _run(wl, "f64")
    for key in ("dt", "dpi", "dr"):
        np.testing.assert_allclose(a[key], d[key], rtol=1e-4, atol=1e-4 * np.abs(d[key]).max(), err_msg=key)


def test_codon_tensor_core_adjoint_with_a_non_binary_code_table():
    """A code table with a row that is not 0 / 1 keeps the tcgen05 adjoint off
    its bit-mask copy of the table (tip rows read from global memory): still
    the CUDA-core adjoint's gradients within FP32 rounding."""
    from torchtree_gb300 import datatype, patterns, synthetic

    wl = synthetic.codon_workload("c", tip_count=12, site_count=300, batch=2, seed=36, shape=0.5)
    codes = patterns.compress(wl.sequences, datatype.get(wl.data_type)).codes
    row = int(np.bincount(np.asarray(codes).ravel()).argmax())  # the most used code
    a = _run(wl, "f32", tca=1, halve_row=row)
    c = _run(wl, "f32", tca=0, halve_row=row)
    np.testing.assert_array_equal(a["lnl"], c["lnl"])
    for key in ("dt", "dpi", "dc", "dr"):
        scale = np.abs(c[key]).max()
        np.testing.assert_allclose(a[key], c[key], rtol=1e-4, atol=1e-4 * scale, err_msg=key)


def test_codon_fp32_against_fp64():
    from torchtree_gb300 import synthetic

    wl = synthetic.codon_workload("c", tip_count=60, site_count=600, batch=2, seed=32, shape=0.5)
    a = _run(wl, "f32")
    d = _run(wl, "f64")
    np.testing.assert_allclose(a["lnl"], d["lnl"], rtol=1e-6)
    np.testing.assert_allclose(a["dt"], d["dt"], rtol=1e-3, atol=1e-3 * np.abs(d["dt"]).max())


def test_protein_batch_member_and_rescaling():
    from torchtree_gb300 import synthetic

    wl = synthetic.protein_workload("p", tip_count=50, site_count=800, batch=3, seed=33, shape=0.5)
    full = _run(wl, "f64")
    single = synthetic.protein_workload("p", tip_count=50, site_count=800, batch=3, seed=33, shape=0.5)
    single.branch_lengths = single.branch_lengths[1:2]
    single.exch, single.pi, single.shape = single.exch[1:2], single.pi[1:2], single.shape[1:2]
    one = _run(single, "f64")
    assert one["lnl"][0] == full["lnl"][1]
    unscaled = _run(wl, "f64", rescale=False, grads=False)
    np.testing.assert_allclose(unscaled["lnl"], full["lnl"], rtol=1e-13)
    f32 = _run(wl, "f32")
    np.testing.assert_allclose(f32["lnl"], full["lnl"], rtol=1e-6)


def test_nonreversible_model_through_given_matrices():
    """Non-reversible Q (no eigen form): P = matrix_exp(Q t) in torch, handed to
    the engine (tt_set_transition_matrices); lnL and dlnL/dQ-rates vs the oracle."""
    from oracle import likelihood as OL
    from torchtree_gb300 import patterns, synthetic
    from torchtree_gb300.likelihood import PhyloLikelihood

    wl = synthetic.dna_workload("nr", tip_count=25, site_count=300, batch=1, seed=61, shape=0.5,
                                site_model="weibull")
    ca = patterns.compress(wl.sequences)
    rng = np.random.default_rng(2)
    off = torch.tensor(rng.gamma(1.0, 1.0, 12), dtype=torch.float64)  # 12 free off-diagonal rates
    rates, probs = OL.weibull_rates(torch.tensor(wl.shape[0], dtype=torch.float64), 4)

    def q_of(r):
        q = torch.zeros(4, 4, dtype=torch.float64, device=r.device)
        mask = ~torch.eye(4, dtype=torch.bool, device=r.device)
        q = q.masked_scatter(mask, r)
        q = q - torch.diag(q.sum(-1))
        return q

    def mats_of(r, bl):
        node_bl = torch.cat((bl, bl.new_zeros(1)))  # node 2T-3 hangs from the root by a zero-length branch
        times = node_bl.unsqueeze(-1) * rates.to(bl.device).unsqueeze(-2)  # [B,K]
        return torch.linalg.matrix_exp(q_of(r) * times[..., None, None])  # [B,K,4,4]

    # stationary distribution of the non-reversible Q as root frequencies
    qn = q_of(off).numpy()
    w, v = np.linalg.eig(qn.T)
    pi = np.real(v[:, np.argmin(np.abs(w))])
    pi = torch.tensor(pi / pi.sum())
    bl = torch.tensor(wl.branch_lengths[0])
    r_cpu = off.clone().requires_grad_()
    tips = [torch.tensor(t) for t in ca.tip_partials()]
    ref = OL.treelikelihood_discrete_rescaled(tips + [None] * (len(tips) - 1), torch.tensor(ca.weights),
                                              wl.topology.postorder_list(), mats_of(r_cpu, bl), pi.unsqueeze(-2),
                                              probs[:, None, None])
    (gref,) = torch.autograd.grad(ref.sum(), r_cpu)
    for precision, ltol, gtol in (("f64", 1e-10, 1e-9), ("f32", 1e-6, 1e-4)):
        lik = PhyloLikelihood(wl.topology, ca, 4, 4, batch=1, precision=precision)
        r = off.cuda().requires_grad_()
        lnl = lik.evaluate_matrices(mats_of(r, bl.cuda()).unsqueeze(0), probs.cuda().unsqueeze(0),
                                    pi.cuda().unsqueeze(0))
        (g,) = torch.autograd.grad(lnl.sum(), r)
        np.testing.assert_allclose(lnl.detach().cpu().numpy(), ref.detach().numpy().reshape(-1), rtol=ltol)
        np.testing.assert_allclose(g.cpu().numpy(), gref.numpy(), rtol=gtol, atol=gtol * np.abs(gref.numpy()).max())


@pytest.mark.parametrize("kind,precision,tc", [("protein", "f32", True), ("protein", "f64", True),
                                               ("codon", "f32", True), ("codon", "f32", False)])
def test_active_samples_equal_the_whole_batch_for_those_samples(kind, precision, tc):
    """TT_OPT_ACTIVE_SAMPLES on 20- and 61-state plans (CUDA-core and
    tensor-core kernels): the passes over the first n samples give those
    samples' lnL and gradients of a call over every sample bit for bit (the
    adjoint's chunking stays that of the whole batch)."""
    from torchtree_gb300 import synthetic

    if kind == "protein":
        wl = synthetic.protein_workload("p", tip_count=30, site_count=600, batch=3, seed=41, shape=0.5)
    else:
        wl = synthetic.codon_workload("c", tip_count=20, site_count=300, batch=3, seed=42, shape=0.5)
    full = _run(wl, precision, tc=tc)
    for n in (1, 2):
        got = _run(wl, precision, tc=tc, active=n)
        for key in ("lnl", "dpi", "dc", "dt", "dr"):
            np.testing.assert_array_equal(got[key][:n], full[key][:n], err_msg=f"n={n} {key}")
