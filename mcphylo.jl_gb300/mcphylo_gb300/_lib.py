"""ctypes binding of libmcphylo_gpu.so (declared in include/mcphylo_gpu.h).

The library is built in-tree by ``mcphylo.jl_gb300/build.py``.  There is no CPU
fallback: if the shared library is missing, or no CUDA device is visible, the
calls raise instead of computing anything on the host.
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
# MCPHYLO_GPU_LIB selects another build of the library (same ABI)
LIB_PATH = os.environ.get("MCPHYLO_GPU_LIB") or os.path.join(_HERE, "libmcphylo_gpu.so")

OK = 0
ERR_ARG, ERR_SHAPE, ERR_TREE, ERR_OOM, ERR_CUDA, ERR_STATE, ERR_TIMEOUT, ERR_NO_DEVICE, ERR_DATA = (
    -1, -2, -3, -4, -5, -6, -7, -8, -9)
PREC_F32 = 0
PREC_F64 = 1
PREC_TF32 = 2
PREC_BF16 = 3
PREC_TF32X3 = 4

i64 = ctypes.c_int64
c_int = ctypes.c_int
dbl = ctypes.c_double
P = ctypes.POINTER
pdbl = P(dbl)
pi64 = P(i64)
pu32 = P(ctypes.c_uint32)
handle_t = ctypes.c_void_p

# name -> (restype, argtypes); exactly the functions include/mcphylo_gpu.h declares
SIGNATURES = {
    "mcphy_create": (c_int, [i64, i64, c_int, P(handle_t)]),
    "mcphy_destroy": (c_int, [handle_t]),
    "mcphy_set_data": (c_int, [handle_t, pdbl, i64, i64, pi64, i64]),
    "mcphy_set_tree": (c_int, [handle_t, i64, pi64, pdbl]),
    "mcphy_set_branch_lengths": (c_int, [handle_t, pdbl]),
    "mcphy_set_model": (c_int, [handle_t, pdbl, pdbl, pdbl, dbl, pdbl, pdbl]),
    "mcphy_logpdf": (c_int, [handle_t, pdbl]),
    "mcphy_logpdf_grad": (c_int, [handle_t, pdbl, pdbl]),
    "mcphy_batch_create": (c_int, [i64, i64, i64, c_int, P(handle_t)]),
    "mcphy_batch_set_data": (c_int, [handle_t, i64, pdbl, i64, i64, pi64, i64]),
    "mcphy_batch_set_codes": (c_int, [handle_t, i64, pu32, i64, pi64, i64]),
    "mcphy_batch_set_tree": (c_int, [handle_t, i64, i64, pi64, pdbl]),
    "mcphy_batch_set_branch_lengths": (c_int, [handle_t, i64, pdbl]),
    "mcphy_batch_set_all_branch_lengths": (c_int, [handle_t, pdbl]),
    "mcphy_batch_set_model": (c_int, [handle_t, i64, pdbl, pdbl, pdbl, dbl, pdbl, pdbl]),
    "mcphy_batch_logpdf": (c_int, [handle_t, pdbl]),
    "mcphy_batch_logpdf_grad": (c_int, [handle_t, pdbl, pdbl]),
    "mcphy_batch_grad_offsets": (c_int, [handle_t, pi64]),
    "mcphy_set_all_branch_lengths_device": (c_int, [handle_t, ctypes.c_void_p]),
    "mcphy_logpdf_grad_device": (c_int, [handle_t, ctypes.c_void_p, ctypes.c_void_p]),
    "mcphy_logpdf_device": (c_int, [handle_t, ctypes.c_void_p]),
    "mcphy_logpdf_grad_noalloc": (c_int, [handle_t, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_void_p]),
    "mcphy_batch_set_weights": (c_int, [handle_t, i64, pdbl, i64]),
    "mcphy_set_weights": (c_int, [handle_t, pdbl, i64]),
    "mcphy_tc_selftest": (c_int, [ctypes.c_int64, ctypes.c_int64, c_int, P(ctypes.c_float),
                                  P(ctypes.c_float), P(ctypes.c_float)]),
    "mcphy_set_stream": (c_int, [handle_t, ctypes.c_void_p]),
    "mcphy_synchronize": (c_int, [handle_t]),
    "mcphy_set_tiles": (c_int, [handle_t, c_int, c_int]),
    "mcphy_autotune": (c_int, [handle_t, P(c_int)]),
    "mcphy_set_sweep": (c_int, [handle_t, c_int]),
    "mcphy_get_sweep": (c_int, [handle_t, P(c_int)]),
    "mcphy_enable_graph": (c_int, [handle_t, c_int]),
    "mcphy_debug_inject": (c_int, [handle_t, c_int]),
    "mcphy_debug_check_allowance": (c_int, []),
    "mcphy_set_rates_per_warp": (c_int, [handle_t, c_int]),
    "mcphy_get_tiles": (c_int, [handle_t, P(c_int)]),
    "mcphy_enable_timing": (c_int, [handle_t, c_int]),
    "mcphy_get_timing": (c_int, [handle_t, P(ctypes.c_float)]),
    "mcphy_get_counts": (c_int, [handle_t, pi64]),
    "mcphy_last_error": (ctypes.c_char_p, [handle_t]),
    "mcphy_status_string": (ctypes.c_char_p, [c_int]),
    "mcphy_version": (c_int, []),
    "mcphy_schedule_info": (c_int, [i64, pi64, pi64]),
}

_lib = None


class MCPhyError(RuntimeError):
    """A non-zero status from the engine."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{message} (status {status})")
        self.status = status


class DimensionMismatch(MCPhyError, ValueError):
    """Sizes disagree (the reference throws DimensionMismatch, Phylodist.jl:195-217)."""


class NoDeviceError(MCPhyError):
    """No CUDA device: the engine has no CPU fallback."""


class _Raw:
    """Prototypes of the per-evaluation entry points that take addresses as plain
    integers (no ctypes pointer objects to build per call), for hot loops."""

    def __init__(self, L):
        vp = ctypes.c_void_p

        def proto(name, args):
            f = L[name]            # a new function object: its own argtypes
            f.restype = c_int
            f.argtypes = args
            return f

        self.set_branch_lengths = proto("mcphy_set_branch_lengths", [vp, vp])
        self.logpdf_grad = proto("mcphy_logpdf_grad", [vp, vp, vp])
        self.logpdf = proto("mcphy_logpdf", [vp, vp])


_raw = None


def raw() -> _Raw:
    global _raw
    if _raw is None:
        _raw = _Raw(load())
    return _raw


def load():
    """Load the shared library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            f"{LIB_PATH} is missing: build it with `python mcphylo.jl_gb300/build.py` "
            "(there is no CPU fallback)")
    L = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(status: int, h=None, what: str = "") -> None:
    if status == OK:
        return
    L = load()
    msg = ""
    if h is not None:
        msg = (L.mcphy_last_error(h) or b"").decode()
    if not msg:
        msg = (L.mcphy_status_string(status) or b"").decode()
    if what:
        msg = f"{what}: {msg}"
    if status == ERR_SHAPE:
        raise DimensionMismatch(status, msg)
    if status == ERR_NO_DEVICE:
        raise NoDeviceError(status, msg)
    if status in (ERR_ARG, ERR_TREE, ERR_DATA):
        raise ValueError(f"{msg} (status {status})")
    raise MCPhyError(status, msg)
