"""Host-side checks that need no GPU: the C-ABI library and its exports, the
schedule, the package's tip encodings / pattern compression / tree glue
against the reference's golden vectors, the eigen form, the site-model
gradient, and the replica timing over two gloo ranks."""
import ctypes
import os
import re
import sys
from pathlib import Path

import numpy as np
import pytest
import torch

ROOT = Path(__file__).resolve().parents[1]


# ------------------------------------------------------------------ C ABI
def _header_functions():
    text = "\n".join(p.read_text() for p in sorted((ROOT / "include").glob("*.h")))
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(tt_[a-z0-9_]+)\s*\(", text)))


def test_library_loads_and_exports_every_header_symbol():
    from torchtree_gb300 import _build, _native

    _build.build()
    lib = ctypes.CDLL(str(_native.LIB_PATH))
    names = _header_functions()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(_native.SIGNATURES) == set(names)  # every export is declared to ctypes
    lib.tt_version.restype = ctypes.c_char_p
    assert lib.tt_version().startswith(b"torchtree_gb300")


def test_option_and_status_constants_match_the_header():
    from torchtree_gb300 import _native

    text = "\n".join(p.read_text() for p in sorted((ROOT / "include").glob("*.h")))
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    header = {k: int(v) for k, v in re.findall(r"\b(TT_OPT_[A-Z_]+)\s*=\s*(\d+)", text)}
    assert "TT_OPT_ACTIVE_SAMPLES" in header
    mirrored = {k: getattr(_native, k) for k in dir(_native) if k.startswith("TT_OPT_")}
    assert mirrored == header


def test_invalid_postorder_is_rejected_by_the_schedule():
    from torchtree_gb300 import _native

    with pytest.raises(ValueError):
        _native.schedule(3, [[3, 0, 1], [3, 2, 3]])  # node 3 parents itself
    with pytest.raises(ValueError):
        _native.schedule(3, [[4, 0, 1], [3, 4, 2]])  # child used before it is computed


@pytest.mark.parametrize("T,seed", [(2, 0), (9, 1), (200, 2), (1000, 3)])
def test_schedule_is_a_valid_walk_with_logarithmic_stack(T, seed):
    from torchtree_gb300 import _native, synthetic

    topo = synthetic.yule_topology(T, np.random.default_rng(seed))
    steps, (fs, bs) = _native.schedule(T, topo.postorder)
    assert steps.shape == (T - 1, 12)
    assert fs <= int(np.ceil(np.log2(T))) + 1 and bs <= int(np.ceil(np.log2(T))) + 2
    done = set(range(T))
    live = {}  # forward slot -> node
    for s in range(T - 1):
        v, l, r, sl, sr, so = steps[s, :6]
        assert l in done and r in done and v not in done
        for c, slot in ((l, sl), (r, sr)):
            if c >= T:
                assert live.pop(slot) == c
            else:
                assert slot == -1
        if s < T - 2:
            assert so >= 0 and so not in live
            live[so] = v
        else:
            assert v == 2 * T - 2 and so == -1
        done.add(v)
    assert not live
    # the reversed walk: a node's outside slot is assigned by its parent before use
    have = {2 * T - 2: -1}
    for s in range(T - 2, -1, -1):
        v, l, r = steps[s, :3]
        assert steps[s, 6] == have.pop(v)
        for c, slot in ((l, steps[s, 7]), (r, steps[s, 8])):
            if c >= T:
                assert slot >= 0 and slot not in have.values()
                have[c] = slot
            else:
                assert slot == -1
    assert not have
    # in-place adjoint: an internal child is either carried to the next
    # reversed step (which is that child) or stored, and then staged back at
    # a step at least two after its parent's, whose reversed index it holds
    rev = steps[::-1]
    at = {int(rev[j, 0]): j for j in range(T - 1)}
    pre_from = {}
    for j in range(T - 1):
        l, r, fl = int(rev[j, 1]), int(rev[j, 2]), int(rev[j, 9])
        for c, carry, store in ((l, 2, 8), (r, 4, 16)):
            if c < T:
                assert not fl & (carry | store)
                continue
            assert bool(fl & carry) != bool(fl & store)
            if fl & carry:
                assert at[c] == j + 1
                pre_from[c] = "carry"
            else:
                assert at[c] >= j + 2 and rev[at[c], 10] == j
                pre_from[c] = "stored"
    for j in range(T - 1):
        v = int(rev[j, 0])
        if j == 0:
            assert v == 2 * T - 2 and rev[j, 9] & 1 == 0
        else:
            assert bool(rev[j, 9] & 1) == (pre_from[v] == "stored")
            if pre_from[v] == "carry":
                assert rev[j, 10] == -1


# --------------------------------------------------- encodings and patterns
def test_package_encodings_match_the_reference(golden_encodings):
    from torchtree_gb300 import datatype

    for name, dt in (("nucleotide", datatype.Nucleotide()), ("amino_acid", datatype.AminoAcid())):
        S = dt.state_count
        for o, (enc, amb, plain) in enumerate(golden_encodings[name]):
            assert dt.partial_vector(o, True) == tuple(amb), (name, chr(o))
            assert dt.partial_vector(o, False) == tuple(plain), (name, chr(o))
            assert dt.state_code(o) == min(enc, S), (name, chr(o))
    codon = datatype.Codon()
    g = golden_encodings["codon_universal"]
    assert codon.state_count == g["state_count"]
    for t, enc in g["codes"].items():
        b = np.frombuffer(t.encode(), dtype=np.uint8)
        assert int(codon.triplet_codes(b[0:1], b[1:2], b[2:3])[0]) == min(enc, codon.state_count), t


def test_package_compression_matches_the_reference(golden_patterns):
    from torchtree_gb300 import datatype, patterns

    for case in golden_patterns:
        if case.get("codon"):
            ca = patterns.compress(case["sequences"], datatype.Codon())
            assert ca.weights.tolist() == case["weights"]
            assert ca.codes.tolist() == case["states"]
            continue
        for amb in (0, 1):
            ca = patterns.compress(case["sequences"], datatype.Nucleotide(), use_ambiguities=bool(amb))
            assert ca.weights.tolist() == case["weights"]
            np.testing.assert_array_equal(ca.tip_partials(), np.asarray(case[f"partials_amb{amb}"]))
        st = patterns.compress(case["sequences"], datatype.Nucleotide(), tip_states=True)
        assert st.codes.tolist() == case["states"]
        idx = [slice(*i) if isinstance(i, list) else i for i in case["indices"]]
        ca = patterns.compress(case["sequences"], datatype.Nucleotide(), indices=idx)
        assert ca.weights.tolist() == case["indexed_weights"]
        np.testing.assert_array_equal(ca.tip_partials(), np.asarray(case["indexed_partials"]))


def test_newick_topology_and_unrooted_lengths_match_the_reference(golden_likelihood):
    from torchtree_gb300.tree import Topology

    rec = golden_likelihood["tiny_jc69"]
    topo = Topology.from_newick(rec["newick"], rec["names"])
    assert topo.postorder.tolist() == rec["postorder"]
    np.testing.assert_allclose(topo.unrooted_branch_lengths(), rec["branch_lengths"], rtol=0, atol=0)


# --------------------------------------------------------- models
def test_eigen_form_reproduces_reference_transition_matrices(golden_transition):
    from torchtree_gb300 import substitution

    g = golden_transition["gtr"]
    pi = torch.tensor(g["pi"], dtype=torch.float64)
    lam, u, w = substitution.eigen_system(substitution.gtr_q(torch.tensor(g["rates"], dtype=torch.float64), pi), pi)
    for t, P in zip(g["t"], g["P"]):
        mine = u @ torch.diag(torch.exp(lam * t)) @ w
        np.testing.assert_allclose(mine.numpy(), np.asarray(P), rtol=1e-10, atol=1e-13)
    g = golden_transition["general20"]
    pi = torch.tensor(g["pi"], dtype=torch.float64)
    q = substitution.general_symmetric_q(torch.tensor(g["rates"], dtype=torch.float64), pi, 20)
    lam, u, w = substitution.eigen_system(q, pi)
    np.testing.assert_allclose((u @ torch.diag(lam) @ w).numpy(), substitution.normalise(q, pi).numpy(),
                               atol=1e-12)
    for t, P in zip(g["t"], g["P"]):
        mine = u @ torch.diag(torch.exp(lam * t)) @ w
        np.testing.assert_allclose(mine.numpy(), np.asarray(P), rtol=1e-9, atol=1e-12)
    g = golden_transition["mg94"]
    pi = torch.tensor(g["pi"], dtype=torch.float64)
    q = substitution.mg94_q(torch.tensor(g["alpha"], dtype=torch.float64), torch.tensor(g["beta"], dtype=torch.float64),
                            torch.tensor(g["kappa"], dtype=torch.float64), pi)
    np.testing.assert_allclose(torch.diagonal(q).numpy(), np.asarray(g["Q_diag"]), rtol=1e-12)
    for i, row in g["Q_rows"].items():
        np.testing.assert_allclose(q[int(i)].numpy(), np.asarray(row), rtol=1e-12, atol=1e-15)


def test_gamma_rates_shape_derivative_matches_finite_differences():
    from torchtree_gb300 import site_models

    shape = torch.tensor([0.37], dtype=torch.float64, requires_grad=True)
    rates, _ = site_models.gamma_rates(shape, 4)
    wts = torch.tensor([0.3, -1.2, 0.7, 2.0], dtype=torch.float64)
    (g,) = torch.autograd.grad((rates * wts).sum(), shape)
    h = 1e-6
    f = lambda a: float((site_models.gamma_rates(torch.tensor([a], dtype=torch.float64), 4)[0] * wts).sum())  # noqa
    fd = (f(0.37 + h) - f(0.37 - h)) / (2 * h)
    assert abs(g.item() - fd) < 1e-6 * max(1.0, abs(fd))


# ------------------------------------------------------ replicas (gloo)
def _replica_rank(rank, world, port, out):
    import torch.distributed as dist

    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    seconds = 1.0 + rank  # rank 1 is the slow one
    slowest, value = bench.replica_throughput(seconds, units_per_rank=8 * 10, world=world)
    out[rank] = (slowest, value)
    dist.destroy_process_group()


def test_replica_throughput_uses_the_slowest_of_two_gloo_ranks():
    import socket

    import torch.multiprocessing as mp

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    out = mp.Manager().dict()
    mp.spawn(_replica_rank, args=(2, port, out), nprocs=2, join=True)
    for r in range(2):
        slowest, value = out[r]
        assert slowest == 2.0 and value == pytest.approx(2 * 80 / 2.0)


def test_native_column_compression_matches_numpy_and_reference_order(golden_patterns):
    from torchtree_gb300 import _build, datatype, patterns

    _build.build()
    rng = np.random.default_rng(5)
    for T, L in ((1, 1), (3, 10), (9, 700), (40, 5000)):
        m = rng.choice(np.frombuffer(b"ACGT-N?R", dtype=np.uint8), size=(T, L))
        if L > 10:
            m[:, L // 2:] = m[:, : L - L // 2]  # many repeated columns
        a = patterns.unique_columns(m, native=True)
        b = patterns.unique_columns(m, native=False)
        np.testing.assert_array_equal(a[0], b[0])
        np.testing.assert_array_equal(a[1], b[1])
    for case in golden_patterns:  # the reference's own order and counts
        if case.get("codon"):
            continue
        m = patterns.as_byte_matrix(case["sequences"])
        cols, w = patterns.unique_columns(m, native=True)
        assert w.tolist() == case["weights"]
        st = datatype.Nucleotide().byte_luts(False, tip_states=True)[1][cols]
        assert st.tolist() == case["states"]


def test_site_models_match_the_reference_known_answers():
    """test_site_model.py: Weibull rates for shapes 1.0 and 0.1 (51-56,
    108-127), the mu scaling (130-138), and the proportion-invariant model's
    probabilities, unit mean rate and mu scaling (80-105)."""
    from torchtree_gb300 import site_models

    f64 = lambda *v: torch.tensor(v, dtype=torch.float64)  # noqa: E731
    rates, probs = site_models.weibull_rates(f64(1.0), 4)
    np.testing.assert_allclose(rates.numpy(), [0.1457844, 0.5131316, 1.0708310, 2.2702530], rtol=1e-6)
    np.testing.assert_allclose(probs.numpy(), [0.25] * 4)
    rates, _ = site_models.weibull_rates(f64(0.1), 4)
    np.testing.assert_allclose(rates.numpy(), [4.766392e-12, 1.391131e-06, 2.179165e-03, 3.997819], rtol=1e-6)
    rates, _ = site_models.weibull_rates(f64(1.0), 4, mu=f64(2.0))
    np.testing.assert_allclose(rates.numpy(), np.array([0.1457844, 0.5131316, 1.0708310, 2.2702530]) * 2, rtol=1e-6)
    rates, probs = site_models.invariant_rates(f64(0.2))
    assert probs.tolist() == [0.2, 0.8] and float((rates * probs).sum()) == 1.0
    rates, _ = site_models.invariant_rates(f64(0.2), mu=f64(2.0))
    assert float(rates[1]) == 2 / 0.8
    rates, probs = site_models.invariant_rates(torch.tensor([[0.2], [0.3]], dtype=torch.float64))
    assert torch.all((rates * probs).sum(-1) == 1.0)


def test_tip_partials_to_codes_fast_path_and_fallbacks(monkeypatch):
    """Plug-in and functional tips arrive as partial tensors: the codes and table
    decode back to them exactly, by fingerprints or, after a fingerprint shared
    by different columns, by the exact lexicographic path."""
    from torchtree_gb300 import patterns

    rng = np.random.default_rng(12)
    table = np.vstack([np.eye(4), np.ones((1, 4)), [[1, 0, 1, 0]], [[0, 1, 0, 1]], [[-0.0, 0, 0, 1]]])
    tips = [table[c].T.copy() for c in rng.integers(0, len(table), size=(9, 700))]
    w = np.arange(700.0)
    fast = patterns.from_tip_partials(tips, w)
    assert fast.table.shape[0] <= len(table) + 1 and fast.codes.dtype == np.uint8
    np.testing.assert_array_equal(fast.table[fast.codes].transpose(0, 2, 1), np.stack(tips))
    np.testing.assert_array_equal(fast.weights, w)
    monkeypatch.setattr(patterns, "_fingerprints", lambda rows: np.zeros(rows.shape[0], dtype=np.uint64))
    exact = patterns.from_tip_partials(tips, w)  # every column collides: exact path
    np.testing.assert_array_equal(exact.table[exact.codes].transpose(0, 2, 1), np.stack(tips))
    monkeypatch.undo()
    many = [rng.random((4, 300)) for _ in range(2)]  # 600 distinct columns
    with pytest.raises(ValueError):
        patterns.from_tip_partials(many, np.ones(300))


def test_every_header_entry_point_cites_what_it_replaces():
    """Each function the C ABI declares sits under a comment that names the
    reference code it replaces (file.py:line) or says that it has no
    counterpart there; declarations grouped under one comment share it."""
    text = "\n".join(p.read_text() for p in sorted((ROOT / "include").glob("*.h")))
    last, prev_end, missing = "", 0, []
    for m in re.finditer(r"\b(?:int|const char \*|void)\s+(tt_[a-z0-9_]+)\s*\(", text):
        comments = re.findall(r"/\*(.*?)\*/", text[prev_end:m.start()], re.S)
        if comments:
            last = comments[-1]
        prev_end = m.end()
        if m.group(1) in ("tt_version", "tt_last_error"):
            continue
        if not (re.search(r"\.py:\d", last) or "counterpart" in last.lower()):
            missing.append(m.group(1))
    assert not missing, missing
