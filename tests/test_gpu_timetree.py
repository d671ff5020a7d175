"""GPU time-tree kernels (ratio transform, constant coalescent) against the
reference's vectors and, batched, against the CPU oracle."""
import json

import numpy as np
import pytest
import torch

from tests.conftest import GOLDEN

pytestmark = pytest.mark.gpu
CASES = json.loads((GOLDEN / "timetree.json").read_text())


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


@pytest.mark.parametrize("key", sorted(CASES))
def test_time_tree_kernels_match_reference(key):
    from torchtree_gb300.timetree import TimeTree

    c = CASES[key]
    tree = TimeTree(c["postorder"], c["sampling_times"])
    dev = torch.device("cuda")
    x = torch.tensor([c["ratios"]], dtype=torch.float64, device=dev, requires_grad=True)
    h, bl, ld = tree.ratio_transform(x)
    np.testing.assert_allclose(h.detach().cpu().numpy()[0], c["heights"], rtol=1e-12)
    np.testing.assert_allclose(bl.detach().cpu().numpy()[0], c["branch_lengths"], rtol=1e-12, atol=1e-13)
    assert abs(ld.item() - c["log_det"]) < 1e-12 * max(1.0, abs(c["log_det"]))
    w1 = torch.tensor(c["w_heights"], dtype=torch.float64, device=dev)
    w3 = torch.tensor(c["w_branch_lengths"], dtype=torch.float64, device=dev)
    obj = (h[0] * w1).sum() + c["w_log_det"] * ld.sum() + (bl[0] * w3).sum()
    (gx,) = torch.autograd.grad(obj, x)
    np.testing.assert_allclose(gx.cpu().numpy()[0], c["grad_ratios"], rtol=1e-10, atol=1e-12)
    hh = torch.tensor([c["internal_heights"]], dtype=torch.float64, device=dev, requires_grad=True)
    th = torch.tensor([c["theta"]], dtype=torch.float64, device=dev, requires_grad=True)
    lp = tree.constant_coalescent(hh, th)
    assert abs(lp.item() - c["coalescent_log_prob"]) < 1e-12 * abs(c["coalescent_log_prob"])
    gh, gth = torch.autograd.grad(lp.sum(), [hh, th])
    np.testing.assert_allclose(gh.cpu().numpy()[0], c["coalescent_grad_heights"], rtol=1e-12, atol=1e-12)
    assert abs(gth.item() - c["coalescent_grad_theta"]) < 1e-12 * max(1.0, abs(c["coalescent_grad_theta"]))


def test_batched_time_tree_kernels_match_the_oracle():
    from oracle import timetree as OT
    from torchtree_gb300 import synthetic
    from torchtree_gb300.timetree import TimeTree

    rng = np.random.default_rng(3)
    T, b = 300, 64
    topo = synthetic.yule_topology(T, rng)
    times = rng.uniform(0.0, 1.0, T)
    x = np.column_stack([rng.uniform(0.05, 0.95, (b, T - 2)), rng.uniform(4.0, 6.0, (b, 1))])
    tree = TimeTree(topo.postorder, times)
    xd = torch.tensor(x, device="cuda", requires_grad=True)
    h, bl, ld = tree.ratio_transform(xd)
    xc = torch.tensor(x, requires_grad=True)
    hc, blc, ldc = OT.ratio_transform(topo.postorder.tolist(), times.tolist(), xc)
    np.testing.assert_allclose(h.detach().cpu().numpy(), hc.detach().numpy(), rtol=1e-12)
    np.testing.assert_allclose(ld.detach().cpu().numpy(), ldc.detach().numpy(), rtol=1e-12)
    theta = torch.linspace(0.5, 2.0, b, dtype=torch.float64)
    lp = tree.constant_coalescent(h, theta.cuda())
    lpc = OT.constant_coalescent(times.tolist(), hc, theta)
    np.testing.assert_allclose(lp.detach().cpu().numpy(), lpc.detach().numpy(), rtol=1e-11)
    (g,) = torch.autograd.grad(lp.sum() + ld.sum() + bl.sum(), xd)
    (gc,) = torch.autograd.grad(lpc.sum() + ldc.sum() + blc.sum(), xc)
    np.testing.assert_allclose(g.cpu().numpy(), gc.numpy(), rtol=1e-9, atol=1e-9 * np.abs(gc.numpy()).max())


@pytest.mark.parametrize("T", [2, 3, 17])
def test_small_trees_and_tied_heights(T):
    """Tiny trees against the oracle (values and gradients), and internal nodes
    placed exactly at a tip's sampling time (ratio 0): the log-density is the
    same in any order of tied heights (their interval is empty)."""
    from oracle import timetree as OT
    from torchtree_gb300 import synthetic
    from torchtree_gb300.timetree import TimeTree

    rng = np.random.default_rng(T)
    topo = synthetic.yule_topology(T, rng)
    times = np.round(rng.uniform(0.0, 1.0, T), 1)  # repeated sampling times
    b = 8
    x = np.column_stack([rng.uniform(0.05, 0.95, (b, T - 2)), rng.uniform(2.0, 3.0, (b, 1))])
    tree = TimeTree(topo.postorder, times)
    theta = torch.linspace(0.5, 2.0, b, dtype=torch.float64)
    xd = torch.tensor(x, device="cuda", requires_grad=True)
    xc = torch.tensor(x, requires_grad=True)
    h, bl, ld = tree.ratio_transform(xd)
    hc, blc, ldc = OT.ratio_transform(topo.postorder.tolist(), times.tolist(), xc)
    lp = tree.constant_coalescent(h, theta.cuda())
    lpc = OT.constant_coalescent(times.tolist(), hc, theta)
    np.testing.assert_allclose(h.detach().cpu().numpy(), hc.detach().numpy(), rtol=1e-12)
    np.testing.assert_allclose(lp.detach().cpu().numpy(), lpc.detach().numpy(), rtol=1e-11)
    (g,) = torch.autograd.grad(lp.sum() + ld.sum() + bl.sum(), xd)
    (gc,) = torch.autograd.grad(lpc.sum() + ldc.sum() + blc.sum(), xc)
    np.testing.assert_allclose(g.cpu().numpy(), gc.numpy(), rtol=1e-9, atol=1e-9 * np.abs(gc.numpy()).max())
    if T > 2:  # ratio 0: a node at its lower bound, the sampling time of a tip below it
        x0 = x.copy()
        x0[:, : T - 2 : 2] = 0.0
        h0, _, _ = tree.ratio_transform(torch.tensor(x0, device="cuda"))
        hc0, _, _ = OT.ratio_transform(topo.postorder.tolist(), times.tolist(), torch.tensor(x0))
        lp0 = tree.constant_coalescent(h0, theta.cuda())
        lpc0 = OT.constant_coalescent(times.tolist(), hc0, theta)
        np.testing.assert_allclose(lp0.cpu().numpy(), lpc0.numpy(), rtol=1e-11)


def test_constant_coalescent_known_answers():
    """torchtree's own numbers (test_coalescent.py:46-67) through the kernels:
    ((A,B),C),D sampled at 0, ratios (2/6, 6/12, 12) under theta 3 and the
    doubled batch member (4/6, 1, 24) under theta 6."""
    from torchtree_gb300.timetree import TimeTree

    tree = TimeTree([[4, 0, 1], [5, 4, 2], [6, 5, 3]], np.zeros(4))
    ratios = torch.tensor([[2.0 / 6.0, 6.0 / 12.0, 12.0], [4.0 / 6.0, 1.0, 24.0]], dtype=torch.float64, device="cuda")
    h, _, _ = tree.ratio_transform(ratios)
    np.testing.assert_allclose(h.cpu().numpy(), [[2.0, 6.0, 12.0], [16.0, 24.0, 24.0]], rtol=1e-15)
    lp = tree.constant_coalescent(h, torch.tensor([3.0, 6.0], dtype=torch.float64, device="cuda"))
    np.testing.assert_allclose(lp.cpu().numpy(), [-13.295836866, -25.375278407684164], rtol=1e-9)
