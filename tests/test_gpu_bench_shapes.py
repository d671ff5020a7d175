"""GPU parity at the benchmark workloads' tree sizes, against the FP64 oracle.

The golden cases reach at most 69 tips x 1,701 sites.  These tests take the
benchmark workloads' own trees, models and parameters at full tip count
(500-tip HKY+Gamma4, 1,000-tip GTR+Gamma4, 200-tip MG94 codon+Gamma4) with a
bounded alignment (about 3,000 DNA patterns, 300 codons; same seeds, so the
same tree and parameters as the benchmark) and two samples, and compare
lnL and the gradients with respect to branch lengths, exchangeabilities (or
kappa, omega), frequencies and category rates with the oracle
(``oracle/likelihood.py``: the reference's rescaled pruning, eigen-form P(t)
and autograd, FP64, CPU).

Tolerances:

* FP64 drop-in: lnL within 1e-10 relative, every gradient within 1e-10 of
  its largest entry;
* FP32 rescaled: lnL within 1e-6 relative, the branch, exchangeability and
  frequency gradients within 1e-4 of their largest entry;
* FP32 category-rate gradient: dlnL/dr_k = sum_b t_b dlnL/dtau_bk is a sum
  with heavy cancellation (near the simulating parameters it is 40-50 times
  smaller than the sum of its terms' magnitudes).  Its error is held to 1e-4
  of its largest entry OR 1e-5 of the cancellation-free scale
  max_k sum_b |t_b dlnL/dtau_bk|, whichever is looser.  The error comes from
  the FP32 post-order partials themselves: a CPU emulation of the kernels'
  arithmetic gives 6e-5 to 1e-4 of the largest entry on the 500-tip case,
  and 1e-6 when only the stored partials are made FP64 (outside partials,
  matrices and sums left in FP32).
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

F64_RTOL = 1e-10
F32_LNL_RTOL = 1e-6
F32_GRAD_TOL = 1e-4
F32_RATE_SCALE_TOL = 1e-5

CASES = {
    # name: (workload, overrides)
    "hky_g4_t500": ("hky_g4_t500_b64", dict(site_count=4000, batch=2)),
    "gtr_g4_t1000": ("gtr_g4_t1000_b8", dict(site_count=3200, batch=2)),
    "codon_g4_t200": ("codon_g4_t200_b16", dict(site_count=300, batch=2)),
}


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


_ORACLE = {}


def _case(name):
    from torchtree_gb300 import datatype, patterns, synthetic

    wl_name, over = CASES[name]
    wl = synthetic.named_workload(wl_name, **over)
    ca = patterns.compress(wl.sequences, datatype.get(wl.data_type))
    return wl, ca


def _rates(wl):
    from torchtree_gb300 import synthetic

    k = wl.categories
    r = np.stack([synthetic.discrete_gamma_np(float(s), k) for s in wl.shape[:, 0]])
    return torch.tensor(r, dtype=torch.float64), torch.full((wl.branch_lengths.shape[0], k), 1.0 / k, dtype=torch.float64)


def _q(model, exch, pi, on_gpu):
    """Unnormalised Q of the workload's model: the package's builders on the
    GPU path, the oracle's on the CPU."""
    if on_gpu:
        from torchtree_gb300 import substitution as M

        gtr, general, mg94 = M.gtr_q, M.general_symmetric_q, M.mg94_q
    else:
        from oracle import likelihood as M

        gtr, general, mg94 = M.q_gtr, M.q_general_symmetric, M.q_mg94
    if model in ("gtr", "hky"):
        return gtr(exch, pi)
    if model == "general":
        return general(exch, pi, pi.shape[-1])
    return mg94(torch.ones_like(exch[..., :1]), exch[..., 1:2], exch[..., :1], pi)


def oracle(name):
    """FP64 lnL [b], gradients (bl, exch, pi, rates) and the category-rate scale, per sample."""
    if name in _ORACLE:
        return _ORACLE[name]
    from oracle import likelihood as OL

    wl, ca = _case(name)
    rates0, probs = _rates(wl)
    out = {"lnl": [], "bl": [], "exch": [], "pi": [], "rates": [], "rate_scale": []}
    tips = [torch.tensor(t) for t in ca.tip_partials()]
    w = torch.tensor(ca.weights)
    for s in range(wl.branch_lengths.shape[0]):
        bl = torch.tensor(wl.branch_lengths[s], requires_grad=True)
        exch = torch.tensor(wl.exch[s], requires_grad=True)
        pi = torch.tensor(wl.pi[s], requires_grad=True)
        rates = rates0[s].clone().requires_grad_()
        bls = OL.model_branch_lengths(bl)
        times = bls.unsqueeze(-1) * rates.unsqueeze(-2)
        times.retain_grad()
        mats = OL.p_t_symmetric(_q(wl.model, exch, pi, False), pi, times)
        parts = list(tips) + [None] * (len(tips) - 1)
        lnl = OL.treelikelihood_discrete_rescaled(parts, w, wl.topology.postorder_list(), mats,
                                                  pi.unsqueeze(-2), probs[s][:, None, None])
        lnl.sum().backward()
        out["lnl"].append(float(lnl.detach().sum()))
        for k, v in (("bl", bl), ("exch", exch), ("pi", pi), ("rates", rates)):
            out[k].append(v.grad.numpy().copy())
        # cancellation-free scale of dlnL/dr_k = sum_b t_b dlnL/dtau_bk
        out["rate_scale"].append(float((bls.detach().unsqueeze(-1) * times.grad).abs().sum(0).max()))
    res = {k: np.asarray(v) for k, v in out.items()}
    _ORACLE[name] = res
    return res


def gpu(name, precision):
    from torchtree_gb300.likelihood import PhyloLikelihood

    wl, ca = _case(name)
    dev = torch.device("cuda")
    b = wl.branch_lengths.shape[0]
    rates0, probs = _rates(wl)
    bl = torch.tensor(wl.branch_lengths, device=dev, requires_grad=True)
    exch = torch.tensor(wl.exch, device=dev, requires_grad=True)
    pi = torch.tensor(wl.pi, device=dev, requires_grad=True)
    rates = rates0.to(dev).requires_grad_()
    lik = PhyloLikelihood(wl.topology, ca, wl.state_count, wl.categories, batch=b, precision=precision, device=dev)
    lik.rescale = True
    lnl = lik(bl, _q(wl.model, exch, pi, True), pi, rates, probs.to(dev))
    grads = torch.autograd.grad(lnl.sum(), [bl, exch, pi, rates])
    return lnl.detach().cpu().numpy(), [g.cpu().numpy() for g in grads]


def _rel_to_max(got, want):
    return float(np.abs(got - want).max() / np.abs(want).max())


@pytest.mark.parametrize("name", sorted(CASES))
def test_fp64_dropin_at_benchmark_shape(name):
    ref = oracle(name)
    lnl, grads = gpu(name, "f64")
    np.testing.assert_allclose(lnl, ref["lnl"], rtol=F64_RTOL)
    for key, got in zip(("bl", "exch", "pi", "rates"), grads):
        for s in range(got.shape[0]):
            assert _rel_to_max(got[s], ref[key][s]) <= F64_RTOL, (key, s, _rel_to_max(got[s], ref[key][s]))


@pytest.mark.parametrize("name", sorted(CASES))
def test_fp32_at_benchmark_shape(name):
    ref = oracle(name)
    lnl, grads = gpu(name, "f32")
    errs = {"lnl": float(np.max(np.abs(lnl - ref["lnl"]) / np.abs(ref["lnl"])))}
    for key, got in zip(("bl", "exch", "pi", "rates"), grads):
        errs[key] = max(_rel_to_max(got[s], ref[key][s]) for s in range(got.shape[0]))
    errs["rates_vs_scale"] = max(float(np.abs(grads[3][s] - ref["rates"][s]).max() / ref["rate_scale"][s])
                                 for s in range(grads[3].shape[0]))
    print(f"{name} FP32 errors: {errs}")
    assert errs["lnl"] <= F32_LNL_RTOL, errs
    for key in ("bl", "exch", "pi"):
        assert errs[key] <= F32_GRAD_TOL, (key, errs)
    assert errs["rates"] <= F32_GRAD_TOL or errs["rates_vs_scale"] <= F32_RATE_SCALE_TOL, errs


def test_functional_cache_sees_in_place_changes():
    """The functional mirror keeps tip data resident between calls; an
    in-place change to a tip tensor must make it upload the new data."""
    from oracle import likelihood as OL
    from torchtree_gb300 import functional, synthetic
    from torchtree_gb300 import patterns as P

    wl = synthetic.dna_workload("cache", tip_count=12, site_count=200, batch=1, seed=9, model="gtr",
                                site_model="weibull", shape=0.7, branch_mean=0.1)
    ca = P.compress(wl.sequences)
    tips = [torch.tensor(t) for t in ca.tip_partials()]
    w = torch.tensor(ca.weights)
    post = wl.topology.postorder_list()
    rates, probs = OL.weibull_rates(torch.tensor(wl.shape), 4)
    pi = torch.tensor(wl.pi)
    mats = OL.p_t_symmetric(OL.q_gtr(torch.tensor(wl.exch), pi), pi,
                            OL.model_branch_lengths(torch.tensor(wl.branch_lengths)).unsqueeze(-1)
                            * rates.unsqueeze(-2))
    args = (w, post, mats, pi.unsqueeze(-2), probs.reshape(-1, 4)[:, :, None, None])

    def both():
        got = functional.calculate_treelikelihood_discrete_rescaled(list(tips) + [None] * 11, *args)
        want = OL.treelikelihood_discrete_rescaled(list(tips) + [None] * 11, *args)
        return got.reshape(-1).cpu().numpy(), want.reshape(-1).numpy()

    got, want = both()
    np.testing.assert_allclose(got, want, rtol=F64_RTOL)
    tips[0][:, :] = 1.0  # tip 0 becomes all-unknown in place
    got2, want2 = both()
    assert abs(want2[0] - want[0]) > 1e-3
    np.testing.assert_allclose(got2, want2, rtol=F64_RTOL)
