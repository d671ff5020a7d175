"""ctypes binding of the C ABI in ``include/torchtree_gb300.h``.

The library is loaded from the package directory only.  There is no
fallback: when the library is missing or a call fails, a ``RuntimeError``
(or ``ValueError`` for bad arguments) is raised.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_native" / "libtorchtree_gb300.so"

TT_OK = 0
TT_ERR_INVALID_ARGUMENT = 1
TT_ERR_UNSUPPORTED = 2
TT_ERR_OUT_OF_MEMORY = 3
TT_ERR_CUDA = 4
TT_ERR_DEVICE_TIMEOUT = 5
TT_ERR_NOT_READY = 6
TT_PRECISION_F32 = 0
TT_PRECISION_F64 = 1

_P = ctypes.c_void_p
_I32 = ctypes.c_int32
_PI32 = ctypes.POINTER(ctypes.c_int32)

# name -> (restype, argtypes); every symbol the header declares
TT_OPT_FWD_STAGES, TT_OPT_BWD_STAGES, TT_OPT_TENSOR_CORES, TT_OPT_PAIR_THREADS, TT_OPT_PRODUCER_WARP = 1, 2, 3, 4, 5
TT_OPT_INPLACE_ADJOINT = 6
TT_OPT_SLAB_PATTERNS = 7
TT_OPT_PAIR_ADJOINT = 8
TT_OPT_TENSOR_CORE_ADJOINT = 9
TT_OPT_ACTIVE_SAMPLES = 10

SIGNATURES = {
    "tt_version": (ctypes.c_char_p, []),
    "tt_last_error": (ctypes.c_char_p, []),
    "tt_plan_create": (ctypes.c_int, [ctypes.POINTER(_P), _I32, _PI32, _I32, _I32, _I32, _I32, _I32]),
    "tt_plan_destroy": (ctypes.c_int, [_P]),
    "tt_plan_workspace_bytes": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_size_t)]),
    "tt_plan_selftest_timeout": (ctypes.c_int, [_P, ctypes.c_uint64, _P]),
    "tt_plan_set_tips": (ctypes.c_int, [_P, _P, _P, _I32, _P]),
    "tt_update_transition_matrices": (ctypes.c_int, [_P, _P, _P, _P, _P, _P, _P]),
    "tt_set_transition_matrices": (ctypes.c_int, [_P, _P, _P]),
    "tt_log_likelihood": (ctypes.c_int, [_P, _P, _P, _I32, _I32, _P, _P, _P]),
    "tt_gradient": (ctypes.c_int, [_P, _P, _P, _P, _P, _P, _P]),
    "tt_transition_matrices_gradient": (ctypes.c_int, [_P] + [_P] * 10 + [_P]),
    "tt_rate_matrix_gradient": (ctypes.c_int, [_P] + [_P] * 8 + [_P]),
    "tt_plan_device_status": (ctypes.c_int, [_P, _P, _PI32, _I32]),
    "tt_plan_launch_count": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int64)]),
    "tt_schedule": (ctypes.c_int, [_I32, _PI32, _PI32, _PI32]),
    "tt_plan_set_option": (ctypes.c_int, [_P, _I32, _I32]),
    "tt_time_tree_create": (ctypes.c_int, [ctypes.POINTER(_P), _I32, _PI32, _P]),
    "tt_time_tree_destroy": (ctypes.c_int, [_P]),
    "tt_ratio_transform": (ctypes.c_int, [_P, _I32, _P, _P, _P, _P, _P]),
    "tt_ratio_transform_backward": (ctypes.c_int, [_P, _I32, _P, _P, _P, _P, _P, _P, _P]),
    "tt_constant_coalescent": (ctypes.c_int, [_P, _I32, _P, _P, _P, _P, _P, _P]),
    "tt_compress_columns": (ctypes.c_int, [_P, ctypes.c_int64, ctypes.c_int64, _P, _P, _P, _P]),
    "tt_plan_get_option": (ctypes.c_int, [_P, _I32, _PI32]),
    "tt_reversible_eigen": (ctypes.c_int, [_I32, _I32, _P, _P, _P, _P, _P, _P, _P]),
    "tt_gamma_quantiles": (ctypes.c_int, [_I32, _I32, _P, _P, _P, _P]),
    "tt_gamma_quantiles_host": (ctypes.c_int, [_I32, _I32, _P, _P, _P]),
    "tt_transition_matrices_expm": (ctypes.c_int, [_I32, _I32, _I32, _I32, _P, _P, _P, _P, _P]),
    "tt_transition_matrices_expm_adjoint": (ctypes.c_int, [_I32, _I32, _I32, _I32, _P, _P, _P, _P, _P, _P, _P]),
    "tt_plans_log_likelihood": (ctypes.c_int, [_I32, _P, _P, _P, _I32, _I32, _P, _P]),
    "tt_plans_gradient": (ctypes.c_int, [_I32, _P, _P, _P, _P, _P, _P]),
    "tt_log_likelihood_static": (ctypes.c_int, [_I32, _PI32, _I32, _I32, _I32, _I32, _P, _P, _I32, _P, _P, _P,
                                                _P, _I32, _P, _P]),
}

_lib = None


class EngineError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, status: int, message: str):
        super().__init__(f"[tt status {status}] {message}")
        self.status = status


def load():
    """Load the engine library (once) and declare its signatures."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(
            f"torchtree_gb300 native library not found at {LIB_PATH}; run "
            "`python -m torchtree_gb300._build` (or __graft_entry__.build()) first"
        )
    lib = ctypes.CDLL(str(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status: int) -> None:
    if status != TT_OK:
        msg = load().tt_last_error().decode(errors="replace")
        if status == TT_ERR_INVALID_ARGUMENT:
            raise ValueError(msg)
        raise EngineError(status, msg)


def schedule(tip_count: int, postorder):
    """Host-only schedule of a topology: ``(steps [T-1,12], (fwd_slots, bwd_slots))``."""
    import numpy as np

    lib = load()
    post = np.ascontiguousarray(np.asarray(postorder, dtype=np.int32).reshape(-1, 3))
    steps = np.zeros((tip_count - 1, 12), dtype=np.int32)
    slots = np.zeros(2, dtype=np.int32)
    p32 = ctypes.POINTER(ctypes.c_int32)
    check(lib.tt_schedule(int(tip_count), post.ctypes.data_as(p32), steps.ctypes.data_as(p32),
                          slots.ctypes.data_as(p32)))
    return steps, (int(slots[0]), int(slots[1]))


def ptr_value(address: int) -> ctypes.c_void_p:
    """A raw address (e.g. a cudaStream_t from torch) as a C pointer."""
    return ctypes.c_void_p(int(address))


def ptr(t) -> ctypes.c_void_p:
    """Raw pointer of a torch tensor or numpy array (None -> NULL)."""
    if t is None:
        return ctypes.c_void_p(0)
    if hasattr(t, "data_ptr"):
        return ctypes.c_void_p(t.data_ptr())
    return ctypes.c_void_p(t.ctypes.data)
