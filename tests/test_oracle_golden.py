"""Pin the CPU oracle against vectors produced by the reference torchtree.

Fixtures: tests/golden/*.json (tests/golden/make_golden.py) plus the known
answers of torchtree's own tests (test/test_tree_likelihood.py:84,
test/test_substitution_model.py:60-70, test/test_site_model.py:51-56,
test/test_site_pattern.py:18).
"""
import numpy as np
import pytest
import torch

from oracle import likelihood as OL
from oracle import patterns as OP
from tests.oracle_cases import GRAD_KEYS, as_np, oracle_lnl, record_inputs


# ----------------------------------------------------------------- encodings
def test_nucleotide_codes_and_partials(golden_encodings):
    for o, (code, amb, noamb) in enumerate(golden_encodings["nucleotide"]):
        ch = chr(o)
        assert OP.nucleotide_code(ch) == code, repr(ch)
        assert list(OP.nucleotide_partial(ch, True)) == amb, repr(ch)
        assert list(OP.nucleotide_partial(ch, False)) == noamb, repr(ch)


def test_amino_acid_codes_and_partials(golden_encodings):
    for o, (code, amb, noamb) in enumerate(golden_encodings["amino_acid"]):
        ch = chr(o)
        assert OP.amino_acid_code(ch) == code, repr(ch)
        assert list(OP.amino_acid_partial(ch, True)) == amb, repr(ch)
        assert list(OP.amino_acid_partial(ch, False)) == noamb, repr(ch)


def test_codon_codes(golden_encodings):
    g = golden_encodings["codon_universal"]
    cc = OP.CodonCode(OP.GENETIC_CODES["universal"])
    assert cc.state_count == g["state_count"] == 61
    for trip, code in g["codes"].items():
        assert cc.code(trip) == code, trip


def test_general_codes(golden_encodings):
    gc = OP.GeneralCode(("A", "C", "T", "G"), {"U": "T", "R": ["A", "G"]})
    for ch, (code, partial) in golden_encodings["general_ACTG"].items():
        assert gc.code(ch) == code, ch
        assert list(gc.partial(ch)) == partial, ch


# ----------------------------------------------------------------- patterns
def _sorted_by_names(case):
    order = sorted(range(len(case["names"])), key=lambda i: case["names"][i])
    return order


def test_site_pattern_known_answer():
    tips, w = OP.compress_partials(["AAG", "AAC", "AAC", "AAT"], OP.nucleotide_partial)
    assert w == [2, 1]  # test_site_pattern.py:18
    assert np.asarray(tips[0]).shape == (4, 2)


@pytest.mark.parametrize("case_index", [0, 1])
def test_compression_matches_reference(golden_patterns, case_index):
    case = golden_patterns[case_index]
    seqs = case["sequences"]  # the reference keeps the given taxa order here (names are the taxa)
    for amb in (False, True):
        tips, w = OP.compress_partials(seqs, lambda c: OP.nucleotide_partial(c, amb))
        assert w == case["weights"]
        assert tips == case[f"partials_amb{int(amb)}"]
    states, w = OP.compress_states(seqs, OP.nucleotide_code, 4)
    assert states == case["states"]
    idx = [slice(*i) if isinstance(i, list) else i for i in case["indices"]]
    tips, w = OP.compress_partials(seqs, lambda c: OP.nucleotide_partial(c, False), indices=idx)
    assert w == case["indexed_weights"]
    assert tips == case["indexed_partials"]


def test_codon_compression_matches_reference(golden_patterns):
    case = golden_patterns[2]
    cc = OP.CodonCode(OP.GENETIC_CODES["universal"])
    tips, w = OP.compress_partials(case["sequences"], cc.partial, size=3)
    assert w == case["weights"]
    argmax = [[int(np.argmax(c)) if sum(c) == 1 else -1 for c in np.asarray(t).T] for t in tips]
    assert argmax == case["argmax_partials"]
    states, _ = OP.compress_states(case["sequences"], cc.code, cc.state_count, size=3)
    assert states == case["states"]


# ------------------------------------------------------- transition / rates
def test_gtr_known_answer():
    # test_substitution_model.py:53-70 (R-computed P(0.1), rtol 1e-5)
    r = torch.tensor([0.060602, 0.402732, 0.028230, 0.047910, 0.407249, 0.053277], dtype=torch.float64)
    pi = torch.tensor([0.479367, 0.172572, 0.140933, 0.207128], dtype=torch.float64)
    P = OL.p_t_symmetric(OL.q_gtr(r, pi), pi, torch.tensor([[0.1]], dtype=torch.float64)).squeeze()
    exp = np.array([[0.93717830, 0.009506685, 0.047505899, 0.005809115],
                    [0.02640748, 0.894078744, 0.006448058, 0.073065722],
                    [0.16158572, 0.007895626, 0.820605951, 0.009912704],
                    [0.01344433, 0.060875872, 0.006744752, 0.918935042]])
    np.testing.assert_allclose(P.numpy(), exp, rtol=1e-5)


def test_transition_matrices_match_reference(golden_transition):
    g = golden_transition
    t = torch.tensor(g["gtr"]["t"], dtype=torch.float64).unsqueeze(-1)
    pi = torch.tensor(g["gtr"]["pi"], dtype=torch.float64)
    P = OL.p_t_symmetric(OL.q_gtr(torch.tensor(g["gtr"]["rates"], dtype=torch.float64), pi), pi, t)
    np.testing.assert_allclose(P.squeeze(-3).numpy(), as_np(g["gtr"]["P"]), rtol=1e-12, atol=1e-15)
    P = OL.p_t_symmetric(OL.q_hky(torch.tensor([g["hky"]["kappa"]], dtype=torch.float64), pi), pi, t)
    np.testing.assert_allclose(P.squeeze(-3).numpy(), as_np(g["hky"]["P"]), rtol=1e-12, atol=1e-15)
    P = OL.p_t_jc69(t)
    np.testing.assert_allclose(P.squeeze(-3).numpy(), as_np(g["jc69"]["P"]), rtol=1e-14)
    pi20 = torch.tensor(g["general20"]["pi"], dtype=torch.float64)
    q20 = OL.q_general_symmetric(torch.tensor(g["general20"]["rates"], dtype=torch.float64), pi20, 20)
    P = OL.p_t_symmetric(q20, pi20, torch.tensor(g["general20"]["t"], dtype=torch.float64).unsqueeze(-1))
    np.testing.assert_allclose(P.squeeze(-3).numpy(), as_np(g["general20"]["P"]), rtol=1e-10, atol=1e-13)


def test_mg94_rate_matrix_matches_reference(golden_transition):
    g = golden_transition["mg94"]
    pi = torch.tensor(g["pi"], dtype=torch.float64)
    one = lambda v: torch.tensor([v], dtype=torch.float64)  # noqa: E731
    q = OL.q_mg94(one(g["alpha"]), one(g["beta"]), one(g["kappa"]), pi)
    np.testing.assert_allclose(torch.diagonal(q).numpy(), as_np(g["Q_diag"]), rtol=1e-13)
    for i, row in g["Q_rows"].items():
        np.testing.assert_allclose(q[int(i)].numpy(), as_np(row), rtol=1e-13, atol=1e-16)


def test_mg94_known_answer():
    # test_substitution_model.py:298-310: omega = kappa = 1 -> 1/61 off the diagonal
    pi = torch.full((61,), 1.0 / 61, dtype=torch.float64)
    one = torch.ones(1, dtype=torch.float64)
    q = OL.q_mg94(one, one, one, pi)
    np.testing.assert_allclose(q[0, 1].item(), 1.0 / 61, rtol=1e-14)
    np.testing.assert_allclose(q[0, 0].item(), -60.0 / 61, rtol=1e-14)


def test_weibull_known_answer(golden_transition):
    # test_site_model.py:51-56
    rates, _ = OL.weibull_rates(torch.tensor([1.0], dtype=torch.float64), 4)
    np.testing.assert_allclose(rates.numpy(), [0.1457844, 0.5131316, 1.0708310, 2.2702530], rtol=1e-6)
    for key, vals in golden_transition["weibull"].items():
        if "+I" in key:
            r, p = OL.weibull_rates(torch.tensor([0.5], dtype=torch.float64), 4,
                                    invariant=torch.tensor([0.2], dtype=torch.float64))
        else:
            r, p = OL.weibull_rates(torch.tensor([float(key)], dtype=torch.float64), 4)
        np.testing.assert_allclose(r.numpy(), as_np(vals["rates"]), rtol=1e-13)
        np.testing.assert_allclose(p.numpy(), as_np(vals["probs"]), rtol=1e-14)


# ------------------------------------------------------------- likelihoods
def test_tiny_known_answer(golden_likelihood):
    rec = golden_likelihood["tiny_jc69"]
    x = record_inputs(rec, requires_grad=False)
    lnl = oracle_lnl(rec, x)
    assert torch.allclose(lnl, torch.tensor(-83.329016, dtype=torch.float64))  # test_tree_likelihood.py:84
    np.testing.assert_allclose(lnl.reshape(-1).numpy(), rec["lnl"], rtol=1e-13)


def _likelihood_keys():
    import json

    from tests.conftest import GOLDEN

    return sorted(json.loads((GOLDEN / "likelihood.json").read_text()))


@pytest.mark.parametrize("key", _likelihood_keys())
def test_oracle_matches_reference_likelihood_and_gradient(golden_likelihood, key):
    rec = golden_likelihood[key]
    x = record_inputs(rec)
    lnl = oracle_lnl(rec, x)
    np.testing.assert_allclose(lnl.detach().reshape(-1).numpy(), rec["lnl"], rtol=1e-12)
    leaves = [(x[k], rec[g]) for k, g in GRAD_KEYS if k in x and g in rec]
    grads = torch.autograd.grad(lnl.sum(), [v for v, _ in leaves])
    for (v, expected), got in zip(leaves, grads):
        np.testing.assert_allclose(got.numpy(), as_np(expected), rtol=1e-9, atol=1e-9)


def test_rescaled_equals_unscaled(golden_likelihood):
    # test_tree_likelihood.py:87-102
    a = golden_likelihood["gtr_w4_t69"]["lnl"]
    b = golden_likelihood["gtr_w4_t69_rescaled"]["lnl"]
    np.testing.assert_allclose(a, b, rtol=1e-13)


def test_underflow_switches_to_rescaling(golden_likelihood):
    rec = golden_likelihood["gtr_w4_t700_underflow"]
    assert rec["rescaled_after"] is True
    x = record_inputs(rec, requires_grad=False)
    tips, w = __import__("tests.oracle_cases", fromlist=["tips_from_record"]).tips_from_record(rec)
    from tests.oracle_cases import model_pieces

    q, pi, rates, probs, bls = model_pieces(rec, x)
    mats = OL.p_t_symmetric(q, pi, bls.unsqueeze(-1) * rates.unsqueeze(-2))
    parts = list(tips) + [None] * (len(tips) - 1)
    plain = OL.treelikelihood_discrete(parts, w, rec["postorder"], mats, pi.unsqueeze(-2),
                                       probs[:, None, None])
    assert torch.isinf(plain).all()
    lnl, switched = OL.unscaled_then_safe(parts, w, rec["postorder"], mats, pi.unsqueeze(-2),
                                          probs[:, None, None], 1e-40)
    assert switched
    np.testing.assert_allclose(lnl.reshape(-1).numpy(), rec["lnl"], rtol=1e-12)


def test_gamma_rates_by_scipy():
    # no Gamma model in the reference: pinned only by scipy's inverse incomplete gamma
    from scipy.special import gammainc, gammaincinv

    shape = 0.3
    rates, probs = OL.gamma_rates(torch.tensor([shape], dtype=torch.float64), 4)
    q = (2 * np.arange(4) + 1) / 8.0
    raw = gammaincinv(shape, q) / shape
    np.testing.assert_allclose(rates.numpy(), raw / raw.mean(), rtol=1e-14)
    np.testing.assert_allclose(gammainc(shape, raw * shape), q, rtol=1e-10)
    assert abs(float((rates * probs).sum()) - 1.0) < 1e-14


# ------------------------------------------------------- time-tree operations
def _timetree_cases():
    import json

    from tests.conftest import GOLDEN

    return json.loads((GOLDEN / "timetree.json").read_text())


@pytest.mark.parametrize("key", sorted(_timetree_cases()))
def test_oracle_time_tree_operations_match_reference(key):
    from oracle import timetree as OT

    c = _timetree_cases()[key]
    x = torch.tensor(c["ratios"], dtype=torch.float64, requires_grad=True)
    h, bl, ld = OT.ratio_transform(c["postorder"], c["sampling_times"], x)
    np.testing.assert_allclose(h.detach().numpy(), c["heights"], rtol=1e-12)
    np.testing.assert_allclose(bl.detach().numpy(), c["branch_lengths"], rtol=1e-12, atol=1e-13)
    assert abs(ld.item() - c["log_det"]) < 1e-12 * max(1.0, abs(c["log_det"]))
    w1 = torch.tensor(c["w_heights"], dtype=torch.float64)
    w3 = torch.tensor(c["w_branch_lengths"], dtype=torch.float64)
    obj = (h * w1).sum() + c["w_log_det"] * ld + (bl * w3).sum()
    (gx,) = torch.autograd.grad(obj, x)
    np.testing.assert_allclose(gx.numpy(), c["grad_ratios"], rtol=1e-10, atol=1e-12)
    hh = torch.tensor(c["internal_heights"], dtype=torch.float64, requires_grad=True)
    th = torch.tensor([c["theta"]], dtype=torch.float64, requires_grad=True)
    lp = OT.constant_coalescent(c["sampling_times"], hh, th)
    assert abs(lp.item() - c["coalescent_log_prob"]) < 1e-12 * abs(c["coalescent_log_prob"])
    gh, gth = torch.autograd.grad(lp.sum(), [hh, th])
    np.testing.assert_allclose(gh.numpy(), c["coalescent_grad_heights"], rtol=1e-12, atol=1e-12)
    assert abs(gth.item() - c["coalescent_grad_theta"]) < 1e-12 * max(1.0, abs(c["coalescent_grad_theta"]))


# torchtree's constant-coalescent known answers (test_coalescent.py:46-67):
# tips A-D sampled at 0, ((A,B),C),D with ratios 2/6, 6/12 and root height 12
# (heights 2, 6, 12) under theta 3, and the batch member with every value
# doubled (heights 16, 24, 24) under theta 6.
COALESCENT_KAT = ((2.0, 6.0, 12.0, 3.0, -13.295836866), (16.0, 24.0, 24.0, 6.0, -25.375278407684164))


def test_constant_coalescent_known_answers():
    from oracle import timetree as OT

    for h0, h1, h2, theta, want in COALESCENT_KAT:
        lp = OT.constant_coalescent([0.0] * 4, torch.tensor([[h0, h1, h2]], dtype=torch.float64),
                                    torch.tensor([theta], dtype=torch.float64))
        assert abs(float(lp[0]) - want) < 1e-8 * abs(want)
    # the same heights from the ratio transform of ((A,B),C),D
    post = [[4, 0, 1], [5, 4, 2], [6, 5, 3]]
    h, _, _ = OT.ratio_transform(post, [0.0] * 4, torch.tensor([2.0 / 6.0, 6.0 / 12.0, 12.0], dtype=torch.float64))
    np.testing.assert_allclose(h.numpy(), [2.0, 6.0, 12.0], rtol=1e-15)
