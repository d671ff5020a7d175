"""Python handle on a C-ABI plan (``include/torchtree_gb300.h``).

A ``LikelihoodEngine`` owns one plan: the topology schedule, the resident
tip codes and pattern weights, and the device workspace for a fixed batch
size.  Every method launches on torch's current CUDA stream and takes
contiguous CUDA float64 tensors.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _native
from ._native import check, ptr


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _dev(t: torch.Tensor, device) -> torch.Tensor:
    return t.detach().to(device=device, dtype=torch.float64).contiguous()


class LikelihoodEngine:
    """Batched pruning likelihood + gradient for one topology and alignment.

    ``postorder``: ``[T-1, 3]`` (node, left, right) triples, root 2T-2 last.
    ``codes [T, N]`` uint8 indexing ``table [C, S]``; ``weights [N]``.
    ``precision``: ``"f32"`` (rescaled FP32 partials) or ``"f64"``.
    """

    def __init__(self, postorder, tip_count: int, state_count: int, category_count: int,
                 codes, table, weights, batch: int = 1, precision: str = "f32", device=None):
        if not torch.cuda.is_available():
            raise RuntimeError("torchtree_gb300 needs a CUDA device; there is no CPU fallback")
        self.lib = _native.load()
        self.device = (torch.device("cuda", torch.cuda.current_device()) if device is None
                       else torch.device(device))
        self.tip_count = int(tip_count)
        self.state_count = int(state_count)
        self.category_count = int(category_count)
        codes = np.ascontiguousarray(np.asarray(codes, dtype=np.uint8))
        self.pattern_count = int(codes.shape[1])
        self.batch = int(batch)
        self.precision = precision
        self.branch_count = 2 * self.tip_count - 2
        post = np.ascontiguousarray(np.asarray(postorder, dtype=np.int32).reshape(-1, 3))
        prec = {"f32": _native.TT_PRECISION_F32, "f64": _native.TT_PRECISION_F64}[precision]
        handle = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            check(self.lib.tt_plan_create(ctypes.byref(handle), self.tip_count,
                                          post.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                          self.state_count, self.category_count, self.pattern_count,
                                          self.batch, prec))
        self._plan = handle
        table = np.ascontiguousarray(np.asarray(table, dtype=np.float64))
        w = np.ascontiguousarray(np.asarray(weights, dtype=np.float64))
        with torch.cuda.device(self.device):
            check(self.lib.tt_plan_set_tips(self._plan, ptr(codes), ptr(table), int(table.shape[0]),
                                            ptr(w)))
        self.token = 0  # bumped by every forward that keeps partials

    # ---------------------------------------------------------------- lifetime
    def close(self):
        if getattr(self, "_plan", None):
            self.lib.tt_plan_destroy(self._plan)
            self._plan = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def workspace_bytes(self) -> int:
        n = ctypes.c_size_t()
        check(self.lib.tt_plan_workspace_bytes(self._plan, ctypes.byref(n)))
        return int(n.value)

    @property
    def launch_count(self) -> int:
        n = ctypes.c_int64()
        check(self.lib.tt_plan_launch_count(self._plan, ctypes.byref(n)))
        return int(n.value)

    def set_option(self, option: int, value: int) -> None:
        """Plan option (``_native.TT_OPT_*``): kernel shapes, which leave results
        unchanged, or ``TT_OPT_SLAB_PATTERNS``, which changes only the grouping
        of the gradient's FP64 sums over pattern slabs."""
        check(self.lib.tt_plan_set_option(self._plan, int(option), int(value)))

    def get_option(self, option: int) -> int:
        v = ctypes.c_int32()
        check(self.lib.tt_plan_get_option(self._plan, int(option), ctypes.byref(v)))
        return int(v.value)

    def selftest_timeout(self, limit_ns: int = 1_000_000) -> None:
        """Launch one bounded wait that nothing completes (failure-path self-test);
        ``device_status()`` then reports ``TT_ERR_DEVICE_TIMEOUT``."""
        check(self.lib.tt_plan_selftest_timeout(self._plan, int(limit_ns), _stream()))

    def device_status(self, reset: bool = True) -> int:
        s = ctypes.c_int32()
        check(self.lib.tt_plan_device_status(self._plan, _stream(), ctypes.byref(s), int(reset)))
        return int(s.value)

    # ------------------------------------------------------------- operations
    def set_eigen(self, lam, u, w, branch_lengths, rates):
        """Transition matrices from ``Q = U diag(lam) W`` (all FP64 device tensors).

        ``lam [b,S]``, ``u``/``w`` ``[b,S,S]``, ``branch_lengths [b,2T-2]``,
        ``rates [b,K]``.
        """
        args = [_dev(x, self.device) for x in (lam, u, w, branch_lengths, rates)]
        self._check_shapes(*args)
        check(self.lib.tt_update_transition_matrices(self._plan, *map(ptr, args), _stream()))
        self._keep = args  # keep alive until the launch has consumed them

    def set_matrices(self, mats):
        """Transition matrices ``[b, 2T-2, K, S, S]`` given directly."""
        m = _dev(mats, self.device)
        exp = (self.batch, self.branch_count, self.category_count, self.state_count, self.state_count)
        if tuple(m.shape) != exp:
            raise ValueError(f"matrices must have shape {exp}, got {tuple(m.shape)}")
        check(self.lib.tt_set_transition_matrices(self._plan, ptr(m), _stream()))
        self._keep = [m]

    def log_likelihood(self, props, freqs, rescale: bool = True, keep_partials: bool = False,
                       site: bool = False):
        """lnL ``[b]`` (and per-pattern site lnL ``[b,N]`` when ``site``)."""
        p = self._per_sample(props, self.category_count)
        f = self._per_sample(freqs, self.state_count)
        out = torch.empty(self.batch, dtype=torch.float64, device=self.device)
        site_out = torch.empty(self.batch, self.pattern_count, dtype=torch.float64,
                               device=self.device) if site else None
        check(self.lib.tt_log_likelihood(self._plan, ptr(p), ptr(f), int(rescale), int(keep_partials),
                                         ptr(out), ptr(site_out), _stream()))
        if keep_partials:
            self.token += 1
        self._root_inputs = (p, f)
        return (out, site_out) if site else out

    def gradient(self, props, freqs, want_matrices: bool = False):
        """``(dlnL/dP [b,B,K,S,S] or None, dlnL/dpi [b,S], dlnL/dc [b,K])``."""
        p = self._per_sample(props, self.category_count)
        f = self._per_sample(freqs, self.state_count)
        dP = torch.empty(self.batch, self.branch_count, self.category_count, self.state_count,
                         self.state_count, dtype=torch.float64, device=self.device) if want_matrices else None
        dpi = torch.empty(self.batch, self.state_count, dtype=torch.float64, device=self.device)
        dc = torch.empty(self.batch, self.category_count, dtype=torch.float64, device=self.device)
        check(self.lib.tt_gradient(self._plan, ptr(p), ptr(f), ptr(dP), ptr(dpi), ptr(dc), _stream()))
        if self.state_count != 4 or self.precision == "f32":  # these adjoints consume the stored partials
            self.token += 1
        return dP, dpi, dc

    def eigen_gradient(self, lam, u, w, branch_lengths, rates):
        """Chain dlnL/dP through the eigen form: ``(dlam, dU, dW, dt, dr)``."""
        args = [_dev(x, self.device) for x in (lam, u, w, branch_lengths, rates)]
        b, S, K, B = self.batch, self.state_count, self.category_count, self.branch_count
        kw = dict(dtype=torch.float64, device=self.device)
        dlam, du, dw = torch.empty(b, S, **kw), torch.empty(b, S, S, **kw), torch.empty(b, S, S, **kw)
        dt, dr = torch.empty(b, B, **kw), torch.empty(b, K, **kw)
        check(self.lib.tt_transition_matrices_gradient(self._plan, *map(ptr, args), ptr(dlam), ptr(du),
                                                       ptr(dw), ptr(dt), ptr(dr), _stream()))
        return dlam, du, dw, dt, dr

    def rate_matrix_gradient(self, lam, u, w, branch_lengths, rates):
        """Chain dlnL/dP to the rate matrix: ``(dQ [b,S,S], dt [b,B], dr [b,K])``."""
        args = [_dev(x, self.device) for x in (lam, u, w, branch_lengths, rates)]
        b, S, K, B = self.batch, self.state_count, self.category_count, self.branch_count
        kw = dict(dtype=torch.float64, device=self.device)
        dq, dt, dr = torch.empty(b, S, S, **kw), torch.empty(b, B, **kw), torch.empty(b, K, **kw)
        check(self.lib.tt_rate_matrix_gradient(self._plan, *map(ptr, args), ptr(dq), ptr(dt), ptr(dr), _stream()))
        return dq, dt, dr

    def expm_matrices(self, q, branch_lengths, rates):
        """``exp(Q t r)`` for every (sample, branch, category) of a normalised,
        possibly non-reversible ``q [b,S,S]`` (FP64, one launch): ``[b,B,K,S,S]``."""
        args = [_dev(x, self.device) for x in (q, branch_lengths, rates)]
        b, S, K, B = self.batch, self.state_count, self.category_count, self.branch_count
        mats = torch.empty(b, B, K, S, S, dtype=torch.float64, device=self.device)
        check(self.lib.tt_transition_matrices_expm(b, S, B, K, *map(ptr, args), ptr(mats), _stream()))
        self._keep_expm = args
        return mats

    def expm_gradient(self, q, branch_lengths, rates, grad_matrices):
        """Chain dlnL/dP through ``P = exp(Q t r)``: ``(dQ [b,S,S], dt [b,B], dr [b,K])``."""
        qd, bl, r, g = (_dev(x, self.device) for x in (q, branch_lengths, rates, grad_matrices))
        b, S, K, B = self.batch, self.state_count, self.category_count, self.branch_count
        parts = torch.empty(b, B, K, S, S, dtype=torch.float64, device=self.device)
        dtau = torch.empty(b, B, K, dtype=torch.float64, device=self.device)
        check(self.lib.tt_transition_matrices_expm_adjoint(b, S, B, K, ptr(qd), ptr(bl), ptr(r), ptr(g),
                                                           ptr(parts), ptr(dtau), _stream()))
        return parts.sum((1, 2)), (dtau * r.unsqueeze(1)).sum(-1), (dtau * bl.unsqueeze(-1)).sum(1)

    def _per_sample(self, x, width):
        """``[..., width]`` (one row or one per sample) -> contiguous ``[batch, width]``."""
        t = _dev(x, self.device).reshape(-1, width)
        if t.shape[0] not in (1, self.batch):
            raise ValueError(f"expected 1 or {self.batch} rows of width {width}, got {tuple(x.shape)}")
        return t.expand(self.batch, width).contiguous()

    def _check_shapes(self, lam, u, w, bl, r):
        b, S, K, B = self.batch, self.state_count, self.category_count, self.branch_count
        for name, t, shp in (("eigenvalues", lam, (b, S)), ("eigenvectors", u, (b, S, S)),
                             ("inverse eigenvectors", w, (b, S, S)), ("branch lengths", bl, (b, B)),
                             ("category rates", r, (b, K))):
            if tuple(t.shape) != shp:
                raise ValueError(f"{name} must have shape {shp}, got {tuple(t.shape)}")


def _ptr_array(values):
    arr = (ctypes.c_void_p * len(values))()
    for i, v in enumerate(values):
        arr[i] = ptr(v).value if v is not None else None
    return arr


def plans_log_likelihood(engines, props, freqs, rescale: bool = True, keep_partials: bool = False):
    """lnL ``[b_i]`` of several engines in one C-ABI call (``tt_plans_log_likelihood``):
    plans on the default FP32 4-state kernels share one post-order launch;
    each result equals that engine's own ``log_likelihood``."""
    if not engines:
        return []
    lib = engines[0].lib
    p = [e._per_sample(x, e.category_count) for e, x in zip(engines, props)]
    f = [e._per_sample(x, e.state_count) for e, x in zip(engines, freqs)]
    outs = [torch.empty(e.batch, dtype=torch.float64, device=e.device) for e in engines]
    plans = (ctypes.c_void_p * len(engines))(*[e._plan for e in engines])
    with torch.cuda.device(engines[0].device):
        check(lib.tt_plans_log_likelihood(len(engines), plans, _ptr_array(p), _ptr_array(f), int(rescale),
                                          int(keep_partials), _ptr_array(outs), _stream()))
    for e, pi, fi in zip(engines, p, f):
        if keep_partials:
            e.token += 1
        e._root_inputs = (pi, fi)
    return outs


def plans_gradient(engines, props, freqs):
    """``[(dlnL/dpi [b,S], dlnL/dc [b,K])]`` of several engines in one call
    (``tt_plans_gradient``); dlnL/dP stays in each plan for
    ``rate_matrix_gradient``."""
    if not engines:
        return []
    lib = engines[0].lib
    p = [e._per_sample(x, e.category_count) for e, x in zip(engines, props)]
    f = [e._per_sample(x, e.state_count) for e, x in zip(engines, freqs)]
    kw = [dict(dtype=torch.float64, device=e.device) for e in engines]
    dpi = [torch.empty(e.batch, e.state_count, **k) for e, k in zip(engines, kw)]
    dc = [torch.empty(e.batch, e.category_count, **k) for e, k in zip(engines, kw)]
    plans = (ctypes.c_void_p * len(engines))(*[e._plan for e in engines])
    with torch.cuda.device(engines[0].device):
        check(lib.tt_plans_gradient(len(engines), plans, _ptr_array(p), _ptr_array(f), _ptr_array(dpi),
                                    _ptr_array(dc), _stream()))
    for e in engines:
        if e.state_count != 4 or e.precision == "f32":
            e.token += 1
    return list(zip(dpi, dc))

