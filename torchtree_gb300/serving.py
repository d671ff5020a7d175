"""Continuous-batching likelihood server.

Many concurrent samplers (HMC / ADVI chains) send lnL + gradient requests for
a set of resident data sets (tree topology + compressed alignment + model
family).  The server keeps each admitted data set's tip codes, pattern
weights and workspace resident in one plan with ``slots`` batch slots, and
runs its step -- transition matrices, post-order, adjoint, matrix-gradient
chain -- as captured CUDA graphs on the data set's own stream, one per number
of occupied slots, whose pruning passes skip the idle slots:

* continuous batching: a scheduler thread launches a data set's waiting
  requests (up to ``slots``) as soon as its previous batch has left the GPU;
  requests that arrive while a batch is in flight wait only for that batch,
  and batches of different data sets run concurrently on their streams;
* same-level work merged across data sets: the waiting batches of every
  FP32 4-state data set go out as one step, whose post-order and adjoint are
  each ONE launch over the pattern tiles of all those trees and alignments
  (``tt_plans_log_likelihood`` / ``tt_plans_gradient``: per-CTA arguments
  name each CTA's plan, sample and tile); other data sets (20 / 61 states,
  pattern slabs) run their own captured graphs;
* admission by HBM footprint: a data set's plan is created only when its
  workspace fits the budget, evicting idle plans (least recently used)
  otherwise; requests of a data set that does not fit wait.  A data set
  larger than the whole budget gets a plan whose partials are held in
  pattern slabs (TT_OPT_SLAB_PATTERNS) sized to the budget; one too large
  even for the smallest slab fails its requests with MemoryError;
* kernel shapes of each plan come from ``autotune.tune`` before capture;
* every request's result (lnL and the gradient with respect to its branch
  lengths, rate-matrix parameters, frequencies and site-model shape) is the
  same whether it runs alone or in a mix: slots are independent and the
  kernels are deterministic.

The rate-matrix construction and the site model stay in torch on the host
(FP64, autograd), as in ``PhyloLikelihood``; the step receives the
normalised Q, branch lengths, category rates and weights through pinned
host buffers, forms the eigen system on the device (device eigensolver) and
returns dlnL/dQ (matrix-exponential derivative), branch-length, rate, weight
and frequency gradients, which the host chains back to the request's
parameters.
"""
from __future__ import annotations

import queue
import threading
import time
from concurrent.futures import Future
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _native, autotune, site_models, substitution
from .engine import LikelihoodEngine, plans_gradient, plans_log_likelihood
from .patterns import CompressedAlignment
from .tree import Topology


@dataclass
class ModelSpec:
    """Substitution model family and site model of a data set.

    ``substitution``: "gtr" (6 exchangeabilities), "hky" (kappa), "general"
    (S(S-1)/2 exchangeabilities) or "mg94" ((kappa, omega), alpha = 1);
    ``site_model``: "gamma" or "weibull" with ``categories`` rates.
    """

    substitution: str
    categories: int = 4
    site_model: str = "gamma"


@dataclass
class Dataset:
    name: str
    topology: Topology
    alignment: CompressedAlignment
    state_count: int
    spec: ModelSpec


@dataclass
class Request:
    dataset: str
    params: dict
    future: Future = field(default_factory=Future)
    t_submit: float = 0.0
    t_launch: float = 0.0
    t_done: float = 0.0


def rate_matrix(spec: ModelSpec, exch: torch.Tensor, pi: torch.Tensor, state_count: int) -> torch.Tensor:
    if spec.substitution == "gtr":
        return substitution.gtr_q(exch, pi)
    if spec.substitution == "hky":
        return substitution.hky_q(exch, pi)
    if spec.substitution == "general":
        return substitution.general_symmetric_q(exch, pi, state_count)
    if spec.substitution == "mg94":
        return substitution.mg94_q(torch.ones_like(exch[..., :1]), exch[..., 1:2], exch[..., :1], pi)
    raise ValueError(f"unknown substitution model {spec.substitution!r}")


def host_prepare(ds: Dataset, params: dict) -> dict:
    """Leaf tensors and engine inputs of one request (host, FP64, autograd on)."""
    f64 = torch.float64
    exch = torch.tensor(np.asarray(params["exch"], dtype=np.float64), dtype=f64, requires_grad=True)
    pi = torch.tensor(np.asarray(params["pi"], dtype=np.float64), dtype=f64, requires_grad=True)
    shape = torch.tensor(np.asarray(params["shape"], dtype=np.float64).reshape(1), dtype=f64, requires_grad=True)
    q = substitution.normalise(rate_matrix(ds.spec, exch, pi, ds.state_count), pi)
    K = ds.spec.categories
    if ds.spec.site_model == "gamma":
        rates, probs = site_models.gamma_rates(shape, K)
    else:
        rates, probs = site_models.weibull_rates(shape, K)
    probs = probs.expand(K)
    bl = np.asarray(params["branch_lengths"], dtype=np.float64)
    bls = np.concatenate([bl, [0.0]]) if bl.shape[-1] == 2 * ds.topology.tip_count - 3 else bl
    return {"leaves": (exch, pi, shape), "q": q, "rates": rates, "probs": probs, "pi": pi,
            "bls": torch.tensor(bls, dtype=f64), "free": bl.shape[-1]}


def host_finish(p: dict, out: dict) -> dict:
    """Chain the engine's gradients to the request's parameters."""
    exch, pi, shape = p["leaves"]
    pairs = [(p[k], out[g]) for k, g in (("q", "dq"), ("rates", "dr"), ("probs", "dc"), ("pi", "dpi"))
             if p[k].requires_grad]
    torch.autograd.backward([t for t, _ in pairs], [g.to(t.dtype).reshape(t.shape) for t, g in pairs])
    return {"lnl": float(out["lnl"]), "grad_branch_lengths": out["dt"][: p["free"]].numpy().copy(),
            "grad_exch": exch.grad.numpy().copy(), "grad_pi": pi.grad.numpy().copy(),
            "grad_shape": shape.grad.numpy().copy()}


SLAB_ALIGN = 512  # pattern-slab sizes are multiples of this (TT_OPT_SLAB_PATTERNS)


def slots_for(ds: Dataset, max_slots: int, fill_ctas: int = 2 * 152) -> int:
    """Batch slots of a data set's plan: enough samples that one launch's
    pattern tiles fill the GPU (``fill_ctas`` CTAs), at most ``max_slots``.
    A captured step computes every slot whatever the number of waiting
    requests (merged 4-state steps run only the slots that hold requests,
    TT_OPT_ACTIVE_SAMPLES), and every slot holds its own partials, so a large
    data set, which fills the GPU with one sample, gets fewer slots."""
    N, K = ds.alignment.pattern_count, ds.spec.categories
    per_sample = -(-N // 64) if ds.state_count == 4 else -(-N // 128) * K
    return max(1, min(max_slots, -(-fill_ctas // max(per_sample, 1))))


def estimate_bytes(ds: Dataset, slots: int, precision: str, slab: int = 0) -> int:
    """Device bytes a plan for ``ds`` with ``slots`` samples will hold (upper
    estimate); with ``slab`` > 0 its partials cover that many patterns at once."""
    T, N, S, K = ds.topology.tip_count, ds.alignment.pattern_count, ds.state_count, ds.spec.categories
    n = min(slab, N) if slab else N
    elem = 4 if precision == "f32" else 8
    B = 2 * T - 2
    if S == 4:
        npad = -(-n // 64) * 64
        kp = K + (K & 1)
        part = slots * T * kp * npad * S * elem
        grad = slots * B * (npad // 32) * K * S * S * elem
        return int(1.1 * (part + grad + slots * B * kp * S * S * elem + T * -(-N // 64) * 64)) + (64 << 20)
    sp = 20 if S <= 20 else 64
    npad = -(-n // 128) * 128
    # partials and exponents; FP32 codon plans also keep the children's products (2 rows per state)
    part = slots * T * K * npad * (sp * elem * (3 if precision == "f32" and sp == 64 else 1) + 4)
    chunks = min(64, max(1, -(-304 // (slots * K))))
    grad = slots * B * K * sp * sp * (chunks * elem + elem + 8)
    if precision == "f32" and sp == 64:  # the tensor-core kernels' split P and P^T images
        grad += slots * B * K * 2 * 2 * sp * sp * 4
    return int(1.1 * (part + grad + T * -(-N // 128) * 128)) + (64 << 20)


def slab_fit(ds: Dataset, slots: int, precision: str, room: int):
    """``(slab, bytes)``: the largest pattern slab whose plan fits in ``room``
    bytes, or ``(0, None)`` when even the smallest slab does not."""
    N = ds.alignment.pattern_count
    for k in range(max(1, -(-N // SLAB_ALIGN) - 1), 0, -1):
        need = estimate_bytes(ds, slots, precision, k * SLAB_ALIGN)
        if need <= room:
            return k * SLAB_ALIGN, need
    return 0, None


class GraphExecutor:
    """One admitted data set: plan, stream, static buffers, captured steps."""

    def __init__(self, ds: Dataset, slots: int, precision: str, device, use_graph: bool = True,
                 tune: bool = True, slab: int = 0, merge: bool = False):
        self.ds = ds
        self.slots = slots
        self.device = device
        T, S, K = ds.topology.tip_count, ds.state_count, ds.spec.categories
        # FP32 4-state plans with the whole alignment resident run in merged
        # steps (one post-order and one adjoint launch for many data sets) on
        # the default kernel shapes, without a graph of their own
        self.mergeable = merge and S == 4 and precision == "f32" and not slab
        if self.mergeable:
            use_graph, tune = False, False
        B = 2 * T - 2
        self.engine = LikelihoodEngine(ds.topology.postorder, T, S, K, ds.alignment.codes, ds.alignment.table,
                                       ds.alignment.weights, batch=slots, precision=precision, device=device)
        if slab:  # partials held one pattern slab at a time (before tuning and capture)
            self.engine.set_option(_native.TT_OPT_SLAB_PATTERNS, slab)
        kw = dict(dtype=torch.float64, device=device)
        jc = torch.full((S, S), 1.0 / (S - 1), **kw) - torch.eye(S, **kw) * (S / (S - 1))  # a valid placeholder Q
        self.inputs = {"q": jc.expand(slots, S, S).contiguous(),
                       "bls": torch.full((slots, B), 0.1, **kw), "rates": torch.ones(slots, K, **kw),
                       "props": torch.full((slots, K), 1.0 / K, **kw), "pi": torch.full((slots, S), 1.0 / S, **kw)}
        self.host_in = {k: torch.empty(v.shape, dtype=v.dtype, pin_memory=True) for k, v in self.inputs.items()}
        self.stream = torch.cuda.Stream(device)
        self.graphs: dict = {}  # occupied slots n -> (graph, outputs) of the step over slots 0 .. n-1
        with torch.cuda.device(device), torch.cuda.stream(self.stream):
            if tune:
                autotune.tune(self.engine, self._step)
            outs = self._step()  # eager warm-up (also sets the plan's state for capture)
            self.stream.synchronize()
            if use_graph:
                for n in range(1, slots + 1):
                    # the pruning passes over the slots that hold requests only
                    self.engine.set_option(_native.TT_OPT_ACTIVE_SAMPLES, n)
                    graph = torch.cuda.CUDAGraph()
                    # thread-local capture: CUDA calls that client threads make meanwhile
                    # (pinned copies of their own, allocations) cannot invalidate it
                    with torch.cuda.graph(graph, stream=self.stream, capture_error_mode="thread_local"):
                        self.graphs[n] = (graph, self._step())
                outs = self.graphs[slots][1]
        self.outputs = outs
        self.host_out = {k: torch.empty(v.shape, dtype=v.dtype, pin_memory=True) for k, v in outs.items()}
        self.event = torch.cuda.Event()
        self.footprint = self.engine.workspace_bytes + sum(v.numel() * 8 for v in self.inputs.values()) * 2
        self.busy = False
        self.batch = None
        self.last_used = time.perf_counter()

    def _step(self) -> dict:
        e, x = self.engine, self.inputs
        lam, u, w = substitution.device_eigen(x["q"], x["pi"])  # device eigensolver, no host round trip
        e.set_eigen(lam, u, w, x["bls"], x["rates"])
        lnl = e.log_likelihood(x["props"], x["pi"], rescale=True, keep_partials=True)
        _, dpi, dc = e.gradient(x["props"], x["pi"])
        dq, dt, dr = e.rate_matrix_gradient(lam, u, w, x["bls"], x["rates"])
        return {"lnl": lnl, "dpi": dpi, "dc": dc, "dq": dq, "dt": dt, "dr": dr}

    def fill(self, reqs: list) -> list:
        """Host side of a batch: each request's engine inputs into the pinned
        input buffers (idle slots repeat the last request)."""
        preps = [host_prepare(self.ds, r.params) for r in reqs]
        for name, key in (("q", "q"), ("bls", "bls"), ("rates", "rates"), ("props", "probs"), ("pi", "pi")):
            buf = self.host_in[name]
            for s in range(self.slots):
                buf[s].copy_(preps[min(s, len(preps) - 1)][key].detach())
        now = time.perf_counter()
        for r in reqs:
            r.t_launch = now
        return preps

    def launch(self, reqs: list) -> None:
        preps = self.fill(reqs)
        with torch.cuda.device(self.device), torch.cuda.stream(self.stream):
            for k, v in self.inputs.items():
                v.copy_(self.host_in[k], non_blocking=True)
            if self.graphs:
                graph, self.outputs = self.graphs[len(reqs)]
                graph.replay()
            else:
                self.engine.set_option(_native.TT_OPT_ACTIVE_SAMPLES, len(reqs))
                self.outputs = self._step()
            for k, v in self.outputs.items():
                self.host_out[k].copy_(v, non_blocking=True)
            self.event.record(self.stream)
        self.busy = True
        self.batch = (reqs, preps)

    def poll(self):
        """``[(request, result, exception)]`` of the batch in flight once it
        has left the GPU, else None.  The caller resolves the futures."""
        if not self.busy or not self.event.query():
            return None
        reqs, preps = self.batch
        done = []
        for s, (r, p) in enumerate(zip(reqs, preps)):
            out = {k: v[s] for k, v in self.host_out.items()}
            try:
                done.append((r, host_finish(p, out), None))
            except Exception as exc:  # report, keep serving
                done.append((r, None, exc))
        self.busy = False
        self.batch = None
        self.last_used = time.perf_counter()
        return done

    def close(self) -> None:
        self.graphs = {}
        self.engine.close()


def merged_step(batches: list, stream, device) -> torch.cuda.Event:
    """Launch the batches of several mergeable executors as one step on
    ``stream``: their inputs in, ONE eigendecomposition launch for all their
    rate matrices, transition matrices per data set, then ONE post-order and
    ONE adjoint launch over the tiles of all of them
    (``tt_plans_log_likelihood`` / ``tt_plans_gradient``; each plan's
    pruning passes cover only the slots that hold requests), the rate-matrix
    chain per data set, results out.  ``batches``: ``[(executor, requests)]``.
    Each request's result equals what its data set's own step gives.  Returns
    the event recorded after the step's last copy."""
    preps = [ex.fill(reqs) for ex, reqs in batches]
    execs = [ex for ex, _ in batches]
    event = torch.cuda.Event()
    with torch.cuda.device(device), torch.cuda.stream(stream):
        for ex in execs:
            for k, v in ex.inputs.items():
                v.copy_(ex.host_in[k], non_blocking=True)
        # all members are 4-state: their Q and pi stack into one eigensolver call
        lam, u, w = substitution.device_eigen(torch.cat([ex.inputs["q"] for ex in execs]),
                                              torch.cat([ex.inputs["pi"] for ex in execs]))
        eig = []
        first = 0
        for ex, reqs in batches:
            x, sl = ex.inputs, slice(first, first + ex.slots)
            first += ex.slots
            eig.append((lam[sl], u[sl], w[sl]))
            # the pruning passes run over the slots that hold requests only
            ex.engine.set_option(_native.TT_OPT_ACTIVE_SAMPLES, len(reqs))
            ex.engine.set_eigen(lam[sl], u[sl], w[sl], x["bls"], x["rates"])
        engines = [ex.engine for ex in execs]
        props = [ex.inputs["props"] for ex in execs]
        pis = [ex.inputs["pi"] for ex in execs]
        lnls = plans_log_likelihood(engines, props, pis, rescale=True, keep_partials=True)
        grads = plans_gradient(engines, props, pis)
        for ex, lnl, (dpi, dc), (lam, u, w) in zip(execs, lnls, grads, eig):
            x = ex.inputs
            dq, dt, dr = ex.engine.rate_matrix_gradient(lam, u, w, x["bls"], x["rates"])
            ex.outputs = {"lnl": lnl, "dpi": dpi, "dc": dc, "dq": dq, "dt": dt, "dr": dr}
            for k, v in ex.outputs.items():
                ex.host_out[k].copy_(v, non_blocking=True)
        event.record(stream)
    for (ex, reqs), pr in zip(batches, preps):
        ex.event = event
        ex.busy = True
        ex.batch = (reqs, pr)
    return event


class LikelihoodServer:
    """Persistent request loop over resident data sets (see the module docstring)."""

    def __init__(self, slots: int = 8, precision: str = "f32", device=None, hbm_budget: int | None = None,
                 use_graphs: bool = True, tune: bool = True, executor_factory=None, merge: bool = True,
                 merge_depth: int = 2, size_slots: bool = True):
        # slots: the most samples a plan batches; with size_slots a data set whose one sample
        # fills the GPU gets fewer (slots_for)
        self.slots = slots
        self.size_slots = size_slots
        self.merge = merge
        # merged steps in flight at once, each on its own stream: while they
        # run, the requests that arrive wait and go out together in the next one
        self.merge_depth = max(1, merge_depth)
        self.precision = precision
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        if hbm_budget is None and executor_factory is None:
            free, _ = torch.cuda.mem_get_info(self.device)
            hbm_budget = int(0.85 * free)
        self.budget = hbm_budget
        self.factory = executor_factory or (lambda ds, slab=0: GraphExecutor(ds, self.slots_of(ds), precision,
                                                                             self.device, use_graph=use_graphs,
                                                                             tune=tune, slab=slab, merge=merge))
        self.estimate = (lambda ds: estimate_bytes(ds, self.slots_of(ds), precision))
        self.slab_fit = (lambda ds, room: slab_fit(ds, self.slots_of(ds), precision, room))
        self.datasets: dict = {}
        self.executors: dict = {}
        self.pending: dict = {}
        self.used = 0
        self.completed: list = []
        self.admissions = 0
        self.evictions = 0
        self.batches = 0
        self.launches = 0  # merged steps plus single-data-set steps
        self.merged_steps = 0
        self.merged_requests = 0
        self.merge_host_s = 0.0  # host time spent issuing merged steps
        self.merge_streams: list = []
        self.merge_inflight: list = []  # (stream index, event) of merged steps not yet finished
        self._queue: queue.Queue = queue.Queue()
        self._stop = threading.Event()
        self._thread = None
        self._error = None

    def slots_of(self, ds: Dataset) -> int:
        return slots_for(ds, self.slots) if self.size_slots else self.slots

    # -------------------------------------------------------------- client API
    def add_dataset(self, name: str, topology: Topology, alignment: CompressedAlignment, state_count: int,
                    spec: ModelSpec) -> None:
        self.datasets[name] = Dataset(name, topology, alignment, state_count, spec)

    def submit(self, dataset: str, params: dict) -> Future:
        if dataset not in self.datasets:
            raise KeyError(f"unknown data set {dataset!r}")
        r = Request(dataset, params, t_submit=time.perf_counter())
        self._queue.put(r)
        return r.future

    def start(self) -> "LikelihoodServer":
        self._stop.clear()
        self._thread = threading.Thread(target=self._loop, name="likelihood-server", daemon=True)
        self._thread.start()
        return self

    def stop(self) -> None:
        self._stop.set()
        if self._thread is not None:
            self._thread.join()
            self._thread = None
        for ex in self.executors.values():
            ex.close()
        self.executors.clear()
        self.used = 0
        if self._error is not None:
            raise self._error

    def reset_stats(self) -> None:
        """Start a new measurement phase: forget completed requests and zero the
        launch, batch, merge, admission and eviction counters (call it while no
        request is waiting or in flight)."""
        self.completed.clear()
        self.batches = self.launches = self.merged_steps = self.merged_requests = 0
        self.merge_host_s = 0.0
        self.admissions = self.evictions = 0

    def latency_stats(self) -> dict:
        lat = np.array([r.t_done - r.t_submit for r in self.completed]) * 1e3
        if lat.size == 0:
            return {"count": 0}
        wait = np.array([r.t_launch - r.t_submit for r in self.completed]) * 1e3
        return {"count": int(lat.size), "p50_ms": float(np.percentile(lat, 50)),
                "p99_ms": float(np.percentile(lat, 99)), "mean_ms": float(lat.mean()),
                "wait_p50_ms": float(np.percentile(wait, 50)), "service_p50_ms": float(np.percentile(lat - wait, 50)),
                "batches": self.batches, "launches": self.launches,
                "requests_per_launch": int(lat.size) / max(self.launches, 1),
                "merged_steps": self.merged_steps,
                "requests_per_merged_step": self.merged_requests / max(self.merged_steps, 1),
                "merge_host_ms_per_step": 1e3 * self.merge_host_s / max(self.merged_steps, 1),
                "admissions": self.admissions, "evictions": self.evictions}

    # -------------------------------------------------------------- scheduler
    def _admit(self, name: str):
        ds = self.datasets[name]
        need = self.estimate(ds)
        slab = 0
        if need > self.budget:  # never fits whole: hold its partials in pattern slabs
            slab, need = self.slab_fit(ds, self.budget)
            if not slab:
                exc = MemoryError(f"data set {name!r} does not fit the HBM budget even in pattern slabs")
                for r in self.pending.pop(name, []):
                    r.future.set_exception(exc)
                return None
        while self.used + need > self.budget:
            idle = [(ex.last_used, n) for n, ex in self.executors.items() if not ex.busy and not self.pending.get(n)]
            if not idle:
                return None
            _, victim = min(idle)
            ex = self.executors.pop(victim)
            self.used -= ex.footprint
            ex.close()
            self.evictions += 1
        ex = self.factory(ds, slab) if slab else self.factory(ds)
        self.executors[name] = ex
        self.used += max(ex.footprint, need)
        self.admissions += 1
        return ex

    def step(self) -> bool:
        """One scheduler iteration; True if anything progressed."""
        progressed = False
        for ex in list(self.executors.values()):
            done = ex.poll()
            if done is None:
                continue
            progressed = True
            now = time.perf_counter()
            for r, res, exc in done:
                r.t_done = now
                if exc is None:
                    self.completed.append(r)
                    r.future.set_result(res)
                else:
                    r.future.set_exception(exc)
        while True:
            try:
                r = self._queue.get_nowait()
            except queue.Empty:
                break
            self.pending.setdefault(r.dataset, []).append(r)
        self.merge_inflight = [(i, ev) for i, ev in self.merge_inflight if not ev.query()]
        merge_open = len(self.merge_inflight) < self.merge_depth
        order = sorted((reqs[0].t_submit, n) for n, reqs in self.pending.items() if reqs)
        merged = []
        for _, name in order:
            ex = self.executors.get(name)
            if ex is None:
                ex = self._admit(name)
                if ex is None:
                    continue
            if ex.busy:
                continue
            mergeable = getattr(ex, "mergeable", False)
            if mergeable and not merge_open:
                continue  # waits for a merged step to finish, gathering more requests
            reqs = self.pending[name][: getattr(ex, "slots", self.slots)]
            del self.pending[name][: len(reqs)]
            if mergeable:
                merged.append((ex, reqs))
            else:
                ex.launch(reqs)
                self.launches += 1
            self.batches += 1
            progressed = True
        if merged:  # every ready 4-state data set in one step
            busy = {i for i, _ in self.merge_inflight}
            idx = next(i for i in range(self.merge_depth) if i not in busy)
            while len(self.merge_streams) <= idx:
                self.merge_streams.append(torch.cuda.Stream(self.device))
            t0 = time.perf_counter()
            ev = merged_step(merged, self.merge_streams[idx], self.device)
            self.merge_host_s += time.perf_counter() - t0
            self.merge_inflight.append((idx, ev))
            self.launches += 1
            self.merged_steps += 1
            self.merged_requests += sum(len(r) for _, r in merged)
        return progressed

    def _busy(self) -> bool:
        return any(ex.busy for ex in self.executors.values()) or any(self.pending.values()) or \
            not self._queue.empty()

    def _loop(self) -> None:
        try:
            if self.device.type == "cuda":
                torch.cuda.set_device(self.device)
            while not self._stop.is_set() or self._busy():
                if not self.step():
                    time.sleep(50e-6)
        except Exception as exc:  # surface on stop(); fail every waiting and in-flight request
            self._error = exc
            waiting = [r for reqs in self.pending.values() for r in reqs]
            in_flight = []
            for ex in self.executors.values():
                batch = getattr(ex, "batch", None)
                if batch:  # GraphExecutor: (requests, host inputs)
                    in_flight += list(batch[0] if isinstance(batch, tuple) else batch)
            for r in waiting + in_flight:
                if not r.future.done():
                    r.future.set_exception(exc)
