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
@pytest.mark.parametrize("S", [2, 3, 4, 5, 20, 32, 33, 47, 61, 64])
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


def _eigen_cases(case):
    """Rate matrices with repeated or nearly repeated eigenvalues: JC69 and
    F81 (one eigenvalue of multiplicity S - 1), K80 (two repeated), a 61-state
    matrix with a pair of eigenvalues 1e-9 apart, and a sparse codon-like one."""
    rng = np.random.default_rng(7)
    if case in ("jc4", "f81_20"):
        S = 4 if case == "jc4" else 20
        pi = np.full(S, 1.0 / S) if case == "jc4" else rng.dirichlet(np.ones(S))
        q = np.tile(pi, (S, 1))
    elif case == "k80_4":
        S, pi = 4, np.full(4, 0.25)
        q = np.ones((4, 4))
        for i, j in ((0, 2), (2, 0), (1, 3), (3, 1)):
            q[i, j] = 3.0  # transitions
        q = q * pi[None]
    elif case == "sparse61":
        S, pi = 61, rng.dirichlet(np.ones(61))
        r = rng.gamma(1.0, 1.0, (S, S)) * (rng.random((S, S)) < 0.15)
        r = np.triu(r, 1) + np.triu(r, 1).T + 1e-3 * (np.ones((S, S)) - np.eye(S))
        q = r * pi[None]
    else:  # near_tie61: A = V diag(lambda) V^T with lambda_1 - lambda_0 = 1e-9
        S, pi = 61, rng.dirichlet(np.ones(61))
        lam = -np.sort(rng.uniform(0.1, 3.0, S))
        lam[1] = lam[0] + 1e-9
        v, _ = np.linalg.qr(rng.standard_normal((S, S)))
        a = (v * lam) @ v.T
        sp = np.sqrt(pi)
        return (a / sp[:, None] * sp[None, :])[None], pi[None]
    np.fill_diagonal(q, 0.0)
    np.fill_diagonal(q, -q.sum(1))
    q /= -(np.diag(q) * pi).sum()
    return q[None], pi[None]


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["jc4", "k80_4", "f81_20", "sparse61", "near_tie61"])
def test_device_eigen_with_repeated_or_close_eigenvalues(case):
    """Checks that do not depend on the basis chosen inside a repeated
    eigenspace: eigenvalues against LAPACK, W = U^-1, Q = U diag(lambda) W and
    P(t) against LAPACK's eigen form."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from torchtree_gb300 import substitution

    q, pi = _eigen_cases(case)
    S = q.shape[-1]
    qt, pit = torch.tensor(q), torch.tensor(pi)
    lam, u, w = (t.cpu() for t in substitution.device_eigen(qt.cuda(), pit.cuda()))
    sp = pit.sqrt()
    a = sp.unsqueeze(-1) * qt / sp.unsqueeze(-2)
    lam_ref, v_ref = torch.linalg.eigh(a)
    scale = lam_ref.abs().amax(-1, keepdim=True)
    assert float(((lam - lam_ref).abs() / scale).max()) <= 1e-12, case
    assert float((u @ w - torch.eye(S, dtype=torch.float64)).abs().max()) <= 1e-12, case
    recon = u @ torch.diag_embed(lam) @ w
    assert float(((recon - qt).abs().amax((-1, -2)) / qt.abs().amax((-1, -2))).max()) <= 1e-11, case
    u_ref, w_ref = v_ref / sp.unsqueeze(-1), v_ref.transpose(-1, -2) * sp.unsqueeze(-2)
    for t in (0.01, 0.7):
        pt = u @ torch.diag_embed(torch.exp(lam * t)) @ w
        p_ref = u_ref @ torch.diag_embed(torch.exp(lam_ref * t)) @ w_ref
        assert float((pt - p_ref).abs().max()) <= 1e-12, (case, t)


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
