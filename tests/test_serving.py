"""Serving loop: continuous batching, admission by HBM footprint, and results
that are the same alone and in a mix.

The scheduler tests run on the CPU with stand-in executors; the end-to-end
test (``gpu``) serves four resident data sets (three DNA, one of them held in
pattern slabs, and one amino-acid) alone through captured CUDA graphs and in
a mix with the DNA work merged across data sets.
"""
import threading
import time

import numpy as np
import pytest

from torchtree_gb300 import serving


class FakeExecutor:
    """Stands in for a GraphExecutor: a batch completes when the test says so."""

    def __init__(self, ds, footprint, log):
        self.ds, self.footprint, self.log = ds, footprint, log
        self.busy, self.batch, self.release = False, None, False
        self.last_used = time.perf_counter()
        self.closed = False

    def launch(self, reqs):
        self.busy, self.batch, self.release = True, reqs, False
        self.log.append((self.ds.name, [r.params["i"] for r in reqs]))

    def poll(self):
        if not self.busy or not self.release:
            return None
        done = [(r, {"lnl": -float(r.params["i"])}, None) for r in self.batch]
        self.batch, self.busy = None, False
        self.last_used = time.perf_counter()
        return done

    def close(self):
        self.closed = True


def _server(budget, slots, sizes):
    log, made = [], {}

    def factory(ds):
        ex = FakeExecutor(ds, sizes[ds.name], log)
        made[ds.name] = ex
        return ex

    srv = serving.LikelihoodServer(slots=slots, hbm_budget=budget, executor_factory=factory, device="cpu")
    srv.estimate = lambda ds: sizes[ds.name]
    for name in sizes:
        srv.add_dataset(name, None, None, 4, serving.ModelSpec("gtr"))
    return srv, log, made


def test_continuous_batching_admits_arrivals_after_the_batch_in_flight():
    srv, log, made = _server(budget=100, slots=4, sizes={"a": 10})
    futs = [srv.submit("a", {"i": i}) for i in range(3)]
    srv.step()
    assert log == [("a", [0, 1, 2])]
    futs += [srv.submit("a", {"i": i}) for i in range(3, 9)]  # arrive while the batch is on the GPU
    srv.step()
    assert len(log) == 1  # one batch per data set in flight
    made["a"].release = True
    srv.step()  # completes the first batch and launches the next four waiting requests
    assert log[1] == ("a", [3, 4, 5, 6])
    made["a"].release = True
    srv.step()
    assert log[2] == ("a", [7, 8])
    made["a"].release = True
    srv.step()
    assert [f.result(timeout=1)["lnl"] for f in futs] == [-float(i) for i in range(9)]
    assert srv.latency_stats()["count"] == 9


def test_reset_stats_counts_one_phase_only():
    srv, log, made = _server(budget=100, slots=4, sizes={"a": 10})
    first = [srv.submit("a", {"i": i}) for i in range(2)]
    srv.step()
    made["a"].release = True
    srv.step()
    assert [f.result(timeout=1)["lnl"] for f in first] == [0.0, -1.0]
    assert srv.latency_stats()["launches"] == 1
    srv.reset_stats()
    assert srv.latency_stats() == {"count": 0}
    futs = [srv.submit("a", {"i": i}) for i in range(2, 10)]
    srv.step()  # four of the eight
    made["a"].release = True
    srv.step()  # completes them and launches the other four
    made["a"].release = True
    srv.step()
    assert [f.result(timeout=1)["lnl"] for f in futs] == [-float(i) for i in range(2, 10)]
    stats = srv.latency_stats()
    assert stats["count"] == 8 and stats["launches"] == 2 and stats["batches"] == 2
    assert stats["requests_per_launch"] == 4.0 and stats["admissions"] == 0


def test_admission_by_footprint_waits_and_evicts_idle_plans():
    srv, log, made = _server(budget=100, slots=2, sizes={"a": 60, "b": 60, "c": 30})
    fa = srv.submit("a", {"i": 0})
    fb = srv.submit("b", {"i": 1})
    fc = srv.submit("c", {"i": 2})
    srv.step()
    # a (60) and c (30) fit together; b (60) must wait for memory
    assert [name for name, _ in log] == ["a", "c"]
    assert "b" not in made and srv.used == 90
    made["a"].release = True
    made["c"].release = True
    srv.step()  # a and c complete; both idle -> the least recently used is evicted for b
    assert "b" in made and made["a"].closed and srv.evictions == 1
    made["b"].release = True
    srv.step()
    assert fa.result(timeout=1)["lnl"] == 0.0 and fb.result(timeout=1)["lnl"] == -1.0
    assert fc.result(timeout=1)["lnl"] == -2.0
    assert srv.used <= srv.budget


def test_request_for_unknown_dataset_is_rejected():
    srv, _, _ = _server(budget=100, slots=2, sizes={"a": 10})
    with pytest.raises(KeyError):
        srv.submit("zzz", {"i": 0})


# ------------------------------------------------------------------ GPU
def _datasets():
    from torchtree_gb300 import datatype, patterns, synthetic

    out = {}
    w1 = synthetic.dna_workload("d1", tip_count=20, site_count=300, batch=6, seed=41, model="gtr",
                                site_model="gamma", shape=0.5, branch_mean=0.05)
    w2 = synthetic.dna_workload("d2", tip_count=33, site_count=200, batch=6, seed=42, model="hky",
                                site_model="weibull", shape=0.8, branch_mean=0.05)
    w3 = synthetic.protein_workload("p1", tip_count=15, site_count=120, batch=6, seed=43, site_model="gamma",
                                    shape=0.5)
    w4 = synthetic.dna_workload("s1", tip_count=45, site_count=2500, batch=6, seed=44, model="gtr",
                                site_model="gamma", shape=0.7, branch_mean=0.05)
    for name, w, spec, dt in (("d1", w1, serving.ModelSpec("gtr"), datatype.Nucleotide()),
                              ("d2", w2, serving.ModelSpec("gtr", site_model="weibull"), datatype.Nucleotide()),
                              ("p1", w3, serving.ModelSpec("general"), datatype.AminoAcid()),
                              ("s1", w4, serving.ModelSpec("gtr"), datatype.Nucleotide())):
        ca = patterns.compress(w.sequences, dt)
        reqs = [{"branch_lengths": w.branch_lengths[i], "exch": w.exch[i], "pi": w.pi[i], "shape": w.shape[i]}
                for i in range(w.branch_lengths.shape[0])]
        out[name] = (w.topology, ca, dt.state_count, spec, reqs)
    return out


@pytest.mark.gpu
def test_results_same_alone_and_in_the_mix():
    """Each request's result is the same served alone through its data set's
    own captured graph and served in a mix where the DNA data sets' work goes
    out as merged steps (one post-order and one adjoint launch over all their
    tiles).  Data set "s1" is held in pattern slabs of 512 (the path a data set
    too large for the memory budget takes) in both runs."""
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    data = _datasets()

    def make(merge):
        dev = torch.device("cuda", torch.cuda.current_device())

        def factory(ds, slab=0):
            return serving.GraphExecutor(ds, 4, "f32", dev, tune=False, slab=512 if ds.name == "s1" else slab,
                                         merge=merge)

        srv = serving.LikelihoodServer(slots=4, precision="f32", executor_factory=factory, merge=merge,
                                       hbm_budget=int(0.5 * torch.cuda.mem_get_info()[0]), device=dev)
        for name, (topo, ca, S, spec, _) in data.items():
            srv.add_dataset(name, topo, ca, S, spec)
        return srv.start()

    alone = {}
    srv = make(merge=False)
    for name, (_, _, _, _, reqs) in data.items():
        for i, p in enumerate(reqs):
            alone[(name, i)] = srv.submit(name, p).result(timeout=300)
    srv.stop()

    srv = make(merge=True)
    futs = {}
    rng = np.random.default_rng(0)
    keys = [(name, i) for name, d in data.items() for i in range(len(d[4]))]
    order = rng.permutation(len(keys))

    def chain(idx):
        for j in idx:
            name, i = keys[j]
            time.sleep(float(rng.uniform(0, 0.002)))
            futs[(name, i)] = srv.submit(name, data[name][4][i])

    threads = [threading.Thread(target=chain, args=(order[t::4],)) for t in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    try:
        mixed = {k: f.result(timeout=300) for k, f in futs.items()}
        stats = srv.latency_stats()
    finally:
        srv.stop()  # raises the scheduler's own error, if it had one
    assert stats["count"] == len(keys) and stats["p99_ms"] >= stats["p50_ms"] > 0
    assert stats["requests_per_launch"] > 1.0, stats
    assert stats["merged_steps"] > 0 and stats["requests_per_merged_step"] > 1.0, stats
    for k in keys:
        a, b = alone[k], mixed[k]
        assert np.isfinite(a["lnl"])
        np.testing.assert_allclose(b["lnl"], a["lnl"], rtol=1e-12, err_msg=str(k))
        for g in ("grad_branch_lengths", "grad_exch", "grad_pi", "grad_shape"):
            np.testing.assert_allclose(b[g], a[g], rtol=1e-12, atol=1e-12 * np.abs(a[g]).max(), err_msg=f"{k} {g}")


def test_a_failing_step_fails_the_requests_in_flight():
    """An error in the scheduler fails every request it holds, waiting or in
    flight, instead of leaving their futures unresolved; stop() raises it."""
    srv, log, made = _server(budget=100, slots=2, sizes={"a": 10})
    futs = [srv.submit("a", {"i": i}) for i in range(3)]
    srv.step()  # admits "a" and launches its first batch

    def broken():
        raise RuntimeError("step failed")

    made["a"].poll = broken
    srv.start()
    for f in futs:
        with pytest.raises(RuntimeError, match="step failed"):
            f.result(timeout=5)
    with pytest.raises(RuntimeError, match="step failed"):
        srv.stop()


def test_slots_follow_the_data_set_size():
    """A plan batches enough samples to fill the GPU with pattern tiles and no
    more: every slot is computed whether or not a request waits for it."""
    from types import SimpleNamespace

    def ds(n, s=4, k=4):
        return serving.Dataset("d", None, SimpleNamespace(pattern_count=n), s, serving.ModelSpec("gtr", k))

    assert serving.slots_for(ds(500), 4) == 4       # 8 tiles of 64 patterns per sample
    assert serving.slots_for(ds(10_000), 4) == 2    # 157 tiles
    assert serving.slots_for(ds(50_000), 4) == 1    # 782 tiles fill the GPU alone
    assert serving.slots_for(ds(5_000, 20), 4) == 2  # 40 tiles of 128 x 4 categories
    assert serving.slots_for(ds(500), 8) == 8
    srv = serving.LikelihoodServer(slots=4, hbm_budget=100, executor_factory=lambda d: None, device="cpu",
                                   size_slots=False)
    assert srv.slots_of(ds(50_000)) == 4


def test_autotune_candidates_cover_the_kernel_shape_options():
    """Host logic only: the option sets the tuner times for each kind of plan."""
    from types import SimpleNamespace

    from torchtree_gb300 import _native, autotune

    dna = autotune.candidates(SimpleNamespace(precision="f32", state_count=4))
    assert len(dna) >= 3
    for opts in dna:
        assert 2 <= opts[_native.TT_OPT_FWD_STAGES] <= 8 and 2 <= opts[_native.TT_OPT_BWD_STAGES] <= 8
    # the default shape (in-place adjoint, producer warp, one thread per pattern) comes first
    first = dna[0]
    assert first[_native.TT_OPT_INPLACE_ADJOINT] == 1 and first[_native.TT_OPT_PRODUCER_WARP] == 1
    assert first[_native.TT_OPT_PAIR_THREADS] == 0
    assert {o[_native.TT_OPT_INPLACE_ADJOINT] for o in dna} == {0, 1}
    codon = autotune.candidates(SimpleNamespace(precision="f32", state_count=61))
    assert {o[_native.TT_OPT_TENSOR_CORES] for o in codon} == {0, 1}
    assert autotune.candidates(SimpleNamespace(precision="f64", state_count=4)) == [{}]


def test_a_data_set_larger_than_the_budget_is_served_in_pattern_slabs():
    """Host logic of the slab fallback: the whole-alignment estimate exceeds the
    budget, so the plan is made with the largest slab whose estimate fits;
    a data set that does not fit even in the smallest slab fails at once."""
    from types import SimpleNamespace

    ds_big = SimpleNamespace(name="big", topology=SimpleNamespace(tip_count=1000),
                             alignment=SimpleNamespace(pattern_count=81808), state_count=4,
                             spec=SimpleNamespace(categories=4))
    whole = serving.estimate_bytes(ds_big, 8, "f32")
    slab, need = serving.slab_fit(ds_big, 8, "f32", whole // 3)
    assert slab % serving.SLAB_ALIGN == 0 and 0 < slab < 81808 and need <= whole // 3
    assert serving.estimate_bytes(ds_big, 8, "f32", slab + serving.SLAB_ALIGN) > whole // 3
    assert serving.slab_fit(ds_big, 8, "f32", 1 << 20) == (0, None)

    log, made = [], {}

    def factory(ds, slab=0):
        ex = FakeExecutor(ds, 40 if slab else 300, log)
        ex.slab = slab
        made[ds.name] = ex
        return ex

    srv = serving.LikelihoodServer(slots=2, hbm_budget=100, executor_factory=factory, device="cpu")
    srv.estimate = lambda ds: {"big": 300, "huge": 10 ** 9}[ds.name]
    srv.slab_fit = lambda ds, room: (1024, 40) if ds.name == "big" else (0, None)
    srv.add_dataset("big", None, None, 4, serving.ModelSpec("gtr"))
    srv.add_dataset("huge", None, None, 4, serving.ModelSpec("gtr"))
    fb = srv.submit("big", {"i": 3})
    fh = srv.submit("huge", {"i": 4})
    srv.step()
    assert made["big"].slab == 1024 and srv.used == 40 and "huge" not in made
    with pytest.raises(MemoryError):
        fh.result(timeout=1)
    made["big"].release = True
    srv.step()
    assert fb.result(timeout=1)["lnl"] == -3.0
