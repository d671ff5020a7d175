"""Per-step model set-up computed by the engine: the discretised Gamma rates
(``tt_gamma_quantiles``) and the eigen system of reversible rate matrices
(``tt_reversible_eigen``).

The Gamma quantiles replace scipy in the product path; torchtree itself ships
no Gamma site model, so they are checked against scipy's ``gammaincinv``
(values, 1e-12) and the shape derivative against a 50-digit mpmath
central difference of the same construction (1e-9).  The CPU tests run the host entry point; the GPU
tests run the device kernels and compare them with the host code and with
LAPACK (``torch.linalg.eigh`` on the CPU), which is what the reference's
``SymmetricSubstitutionModel.eigen`` calls (abstract.py:78-79).
"""
import numpy as np
import pytest
import torch

SHAPES = [0.02, 0.1, 0.3, 0.5, 1.0, 2.7, 10.0, 40.0, 250.0, 3000.0]


def _scipy_rates(shapes, k):
    from scipy.special import gammaincinv

    q = (2.0 * np.arange(k) + 1.0) / (2.0 * k)
    x = gammaincinv(np.asarray(shapes)[:, None], q[None])
    return x / x.mean(-1, keepdims=True)


@pytest.mark.parametrize("k", [1, 4, 8, 32])
def test_gamma_rates_match_scipy_on_the_host(k):
    from torchtree_gb300 import site_models

    a = torch.tensor(SHAPES, dtype=torch.float64).unsqueeze(-1).requires_grad_()
    rates, probs = site_models.gamma_rates(a, k)
    want = _scipy_rates(SHAPES, k)
    np.testing.assert_allclose(rates.detach().numpy(), want, rtol=1e-12, atol=1e-300)
    np.testing.assert_allclose(probs.numpy(), np.full((len(SHAPES), k), 1.0 / k))
    if k == 1:
        return
    # analytic shape derivative of the last category's rate against a
    # 50-digit central difference (mpmath: roots of P(a, e^y) = q in log space)
    mpmath = pytest.importorskip("mpmath")
    (g,) = torch.autograd.grad(rates[:, -1].sum(), a)
    from scipy.special import gammaincinv

    def rate_last(aa):
        xs = []
        for i in range(k):
            q = mpmath.mpf(2 * i + 1) / (2 * k)
            y0 = mpmath.log(mpmath.mpf(gammaincinv(float(aa), float(q))))
            y = mpmath.findroot(lambda y: mpmath.gammainc(aa, 0, mpmath.exp(y), regularized=True) - q, y0,
                                tol=mpmath.mpf(10) ** -40)
            xs.append(mpmath.exp(y))
        return xs[-1] / (sum(xs) / k)

    with mpmath.workdps(50):
        for ai, gi in zip(SHAPES, g.numpy()[:, 0]):
            aa = mpmath.mpf(ai)
            h = aa * mpmath.mpf(10) ** -15
            d = float((rate_last(aa + h) - rate_last(aa - h)) / (2 * h))
            assert abs(gi - d) <= 1e-9 * abs(d), (ai, gi, d)


def test_gamma_rates_reject_bad_shapes_on_the_host():
    from torchtree_gb300 import site_models

    for bad in (0.0, -1.0, float("nan"), float("inf")):
        with pytest.raises(ValueError):
            site_models.gamma_rates(torch.tensor([[bad]], dtype=torch.float64), 4)


def _random_reversible(rng, b, S):
    pi = rng.dirichlet(np.ones(S), size=b)
    out = []
    for i in range(b):
        r = rng.gamma(1.0, 1.0, (S, S))
        r = r + r.T
        np.fill_diagonal(r, 0.0)
        q = r * pi[i][None]
        np.fill_diagonal(q, -q.sum(1))
        q /= -(np.diag(q) * pi[i]).sum()
        out.append(q)
    return np.stack(out), pi


@pytest.mark.gpu
@pytest.mark.parametrize("S", [2, 3, 4, 5, 20, 61, 64])
def test_device_eigen_system_matches_lapack(S):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from torchtree_gb300 import substitution

    rng = np.random.default_rng(300 + S)
    q, pi = _random_reversible(rng, 6, S)
    qt, pit = torch.tensor(q), torch.tensor(pi)
    lam, u, w = (t.cpu() for t in substitution.device_eigen(qt.cuda(), pit.cuda()))
    sp = pit.sqrt()
    a = sp.unsqueeze(-1) * qt / sp.unsqueeze(-2)
    lam_ref, v_ref = torch.linalg.eigh(a)  # LAPACK, lower triangle
    scale = lam_ref.abs().amax(-1, keepdim=True).clamp_min(1e-300)
    assert float(((lam - lam_ref).abs() / scale).max()) <= 1e-12
    eye = torch.eye(S, dtype=torch.float64)
    assert float((u @ w - eye).abs().max()) <= 1e-12
    recon = u @ torch.diag_embed(lam) @ w
    assert float(((recon - qt).abs().amax((-1, -2)) / qt.abs().amax((-1, -2))).max()) <= 1e-11
    # transition matrices against LAPACK's eigen form, for a short and a long branch
    u_ref, w_ref = v_ref / sp.unsqueeze(-1), v_ref.transpose(-1, -2) * sp.unsqueeze(-2)
    for t in (0.01, 0.7):
        p = u @ torch.diag_embed(torch.exp(lam * t)) @ w
        p_ref = u_ref @ torch.diag_embed(torch.exp(lam_ref * t)) @ w_ref
        assert float((p - p_ref).abs().max()) <= 1e-12, (S, t)


@pytest.mark.gpu
@pytest.mark.parametrize("k", [4, 8])
def test_device_gamma_quantiles_match_host_and_scipy(k):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from torchtree_gb300 import site_models

    a_host = torch.tensor(SHAPES, dtype=torch.float64).unsqueeze(-1).requires_grad_()
    a_dev = a_host.detach().cuda().requires_grad_()
    r_host, _ = site_models.gamma_rates(a_host, k)
    r_dev, _ = site_models.gamma_rates(a_dev, k)
    np.testing.assert_allclose(r_dev.detach().cpu().numpy(), r_host.detach().numpy(), rtol=1e-13)
    np.testing.assert_allclose(r_dev.detach().cpu().numpy(), _scipy_rates(SHAPES, k), rtol=1e-12)
    (g_host,) = torch.autograd.grad(r_host[:, 1].sum(), a_host)
    (g_dev,) = torch.autograd.grad(r_dev[:, 1].sum(), a_dev)
    np.testing.assert_allclose(g_dev.cpu().numpy(), g_host.numpy(), rtol=1e-12, atol=1e-14)
    bad = site_models.gamma_rates(torch.tensor([[-1.0]], dtype=torch.float64, device="cuda"), k)[0]
    assert torch.isnan(bad).all()
