"""Python side of the engine: a thin owner of one libmcphylo_gpu handle.

``Engine`` is the object a sampler keeps for a whole chain: the data is uploaded
once, and each leapfrog step only sends the branch lengths and reads back the
log-likelihood and gradient.  ``Engine(..., n_instances=M)`` is the batched form
(MultiplePhyloDist): M independent trees, data sets and models in one launch.
"""
from __future__ import annotations

import ctypes
from typing import Optional, Sequence

import numpy as np

from . import _lib
from ._lib import check

_PREC = {"f32": _lib.PREC_F32, "fp32": _lib.PREC_F32, "float32": _lib.PREC_F32,
         "f64": _lib.PREC_F64, "fp64": _lib.PREC_F64, "float64": _lib.PREC_F64,
         "tf32": _lib.PREC_TF32, "bf16": _lib.PREC_BF16, "tf32x3": _lib.PREC_TF32X3}


def _pd(a: np.ndarray):
    return a.ctypes.data_as(_lib.pdbl)


def _pi64(a: np.ndarray):
    return a.ctypes.data_as(_lib.pi64)


def _f64(a, order="C") -> np.ndarray:
    return np.require(np.asarray(a, dtype=np.float64), requirements=[order[0], "A"])


class Engine:
    """Owner of one engine handle (K states, C rate categories, M instances)."""

    def __init__(self, nbase: int, nrates: int, precision: str = "f32", n_instances: int = 1):
        L = _lib.load()
        self._L = L
        self.K = int(nbase)
        self.C = int(nrates)
        self.M = int(n_instances)
        self.precision = precision
        h = _lib.handle_t()
        st = L.mcphy_batch_create(self.K, self.C, self.M, _PREC[precision], ctypes.byref(h))
        if st != _lib.OK:
            check(st, None, "mcphy_batch_create")
        self._h = h
        self._N = [0] * self.M
        self._grad_off = None

    # ------------------------------------------------------------------ lifetime
    def close(self) -> None:
        if getattr(self, "_h", None):
            self._L.mcphy_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ------------------------------------------------------------------ setters
    def set_data(self, x: np.ndarray, leaf_nums: Sequence[int], i: int = 0) -> None:
        """x: the reference's (K, S, N) FP64 tensor; leaf slices at x[:, :, num-1]."""
        x = np.asfortranarray(x, dtype=np.float64)
        if x.ndim != 3 or x.shape[0] != self.K:
            raise _lib.DimensionMismatch(_lib.ERR_SHAPE, f"x must be ({self.K}, S, N), got {x.shape}")
        ln = np.ascontiguousarray(leaf_nums, dtype=np.int64)
        check(self._L.mcphy_batch_set_data(self._h, i, _pd(x), x.shape[1], x.shape[2], _pi64(ln),
                                           len(ln)), self._h, "set_data")

    def set_codes(self, codes: np.ndarray, leaf_nums: Sequence[int], i: int = 0) -> None:
        """codes: (n_leaves, S) uint32 state bitmasks, row l for leaf leaf_nums[l]."""
        c = np.ascontiguousarray(codes, dtype=np.uint32)
        ln = np.ascontiguousarray(leaf_nums, dtype=np.int64)
        if c.ndim != 2 or c.shape[0] != len(ln):
            raise _lib.DimensionMismatch(_lib.ERR_SHAPE, "codes must be (n_leaves, S)")
        check(self._L.mcphy_batch_set_codes(self._h, i, c.ctypes.data_as(_lib.pu32), c.shape[1],
                                            _pi64(ln), len(ln)), self._h, "set_codes")

    def set_weights(self, weights: Optional[Sequence[float]], i: int = 0) -> None:
        """Site-pattern weights (one per site of instance i; None: every site once)."""
        if weights is None:
            check(self._L.mcphy_batch_set_weights(self._h, i, None, 0), self._h, "set_weights")
            return
        w = np.ascontiguousarray(weights, dtype=np.float64)
        check(self._L.mcphy_batch_set_weights(self._h, i, _pd(w), len(w)), self._h, "set_weights")

    def set_tree(self, parent: Sequence[int], blen: Optional[Sequence[float]] = None,
                 i: int = 0) -> None:
        p = np.ascontiguousarray(parent, dtype=np.int64)
        b = None if blen is None else np.ascontiguousarray(blen, dtype=np.float64)
        if b is not None and len(b) != len(p) - 1:
            raise _lib.DimensionMismatch(_lib.ERR_SHAPE, "blen must have N-1 entries")
        check(self._L.mcphy_batch_set_tree(self._h, i, len(p), _pi64(p),
                                           None if b is None else _pd(b)), self._h, "set_tree")
        self._N[i] = len(p)
        self._grad_off = None

    def set_branch_lengths(self, blen, i: int = 0) -> None:
        b = np.ascontiguousarray(blen, dtype=np.float64)
        if len(b) != self._N[i] - 1:
            raise _lib.DimensionMismatch(_lib.ERR_SHAPE, "blen must have N-1 entries")
        check(self._L.mcphy_batch_set_branch_lengths(self._h, i, _pd(b)), self._h,
              "set_branch_lengths")

    def set_all_branch_lengths(self, blen_packed) -> None:
        b = np.ascontiguousarray(blen_packed, dtype=np.float64)
        if len(b) != sum(self._N) - self.M:
            raise _lib.DimensionMismatch(_lib.ERR_SHAPE, "packed blen has the wrong length")
        check(self._L.mcphy_batch_set_all_branch_lengths(self._h, _pd(b)), self._h,
              "set_all_branch_lengths")

    def set_model(self, U, D, Uinv, mu: float, pi, rates, i: int = 0) -> None:
        if np.iscomplexobj(U) or np.iscomplexobj(D) or np.iscomplexobj(Uinv):
            raise ValueError("the likelihood path needs a real eigensystem")
        Uf = np.asfortranarray(U, dtype=np.float64)
        Uif = np.asfortranarray(Uinv, dtype=np.float64)
        Dd = np.ascontiguousarray(D, dtype=np.float64)
        pid = np.ascontiguousarray(pi, dtype=np.float64)
        rd = np.ascontiguousarray(rates, dtype=np.float64)
        if Uf.shape != (self.K, self.K) or Uif.shape != (self.K, self.K) or len(Dd) != self.K \
                or len(pid) != self.K:
            raise _lib.DimensionMismatch(_lib.ERR_SHAPE, "model arrays do not match K")
        if len(rd) != self.C:
            raise _lib.DimensionMismatch(_lib.ERR_SHAPE, "rates do not match C")
        check(self._L.mcphy_batch_set_model(self._h, i, _pd(Uf), _pd(Dd), _pd(Uif), float(mu),
                                            _pd(pid), _pd(rd)), self._h, "set_model")

    def set_tiles(self, sites_per_thread: int = 0, threads_per_block: int = 0) -> None:
        check(self._L.mcphy_set_tiles(self._h, sites_per_thread, threads_per_block), self._h,
              "set_tiles")

    def set_rates_per_warp(self, rates_per_warp: int = 0) -> None:
        """Rate categories per warp of the FP32 tree walk (1, 2 or 4; 0: automatic)."""
        check(self._L.mcphy_set_rates_per_warp(self._h, int(rates_per_warp)), self._h,
              "set_rates_per_warp")

    def tiles(self):
        """(sites_per_thread, threads_per_block, rates_per_warp) of the current layout."""
        out = (ctypes.c_int * 3)()
        check(self._L.mcphy_get_tiles(self._h, out), self._h, "get_tiles")
        return int(out[0]), int(out[1]), int(out[2])

    SWEEPS = {"auto": 0, "walk": 1, "level": 2}

    def set_sweep(self, sweep: str = "auto") -> None:
        """Sweep of the SIMT paths: "walk" (a warp walks the whole tree), "level"
        (a CTA's warps share a small tree level by level) or "auto"."""
        if sweep not in self.SWEEPS:
            raise ValueError(f"sweep must be one of {sorted(self.SWEEPS)}")
        check(self._L.mcphy_set_sweep(self._h, self.SWEEPS[sweep]), self._h, "set_sweep")

    def sweep(self) -> str:
        """The sweep the current layout uses (lays it out first if needed)."""
        out = ctypes.c_int(0)
        check(self._L.mcphy_get_sweep(self._h, ctypes.byref(out)), self._h, "get_sweep")
        return {1: "walk", 2: "level"}[int(out.value)]

    def autotune(self):
        """Time the candidate launch shapes on the current problem; keep the fastest."""
        out = (ctypes.c_int * 2)()
        check(self._L.mcphy_autotune(self._h, out), self._h, "autotune")
        return int(out[0]), int(out[1])

    def enable_graph(self, on: bool = True) -> None:
        check(self._L.mcphy_enable_graph(self._h, 1 if on else 0), self._h)

    def debug_inject(self, kind: int) -> None:
        check(self._L.mcphy_debug_inject(self._h, int(kind)), self._h)

    def set_stream(self, stream_ptr: int) -> None:
        check(self._L.mcphy_set_stream(self._h, ctypes.c_void_p(stream_ptr or None)), self._h)

    def enable_timing(self, on: bool = True) -> None:
        check(self._L.mcphy_enable_timing(self._h, 1 if on else 0), self._h)

    # ------------------------------------------------------------------ evaluation
    def grad_offsets(self) -> np.ndarray:
        if self._grad_off is None:
            off = np.zeros(self.M + 1, dtype=np.int64)
            check(self._L.mcphy_batch_grad_offsets(self._h, _pi64(off)), self._h)
            self._grad_off = off
        return self._grad_off

    def logpdf(self):
        ll = np.zeros(self.M, dtype=np.float64)
        check(self._L.mcphy_batch_logpdf(self._h, _pd(ll)), self._h, "logpdf")
        return float(ll[0]) if self.M == 1 else ll

    def logpdf_grad(self, out_ll: Optional[np.ndarray] = None,
                    out_grad: Optional[np.ndarray] = None):
        """-> (ll, grad) for one instance, (ll[M], packed grad) for a batch."""
        off = self.grad_offsets()
        ll = out_ll if out_ll is not None else np.zeros(self.M, dtype=np.float64)
        g = out_grad if out_grad is not None else np.zeros(int(off[-1]), dtype=np.float64)
        check(self._L.mcphy_batch_logpdf_grad(self._h, _pd(ll), _pd(g)), self._h, "logpdf_grad")
        if self.M == 1:
            return float(ll[0]), g
        return ll, g

    def bind(self, i: int = 0):
        """(grad_fn, logf_fn) for a sampler that evaluates this single-instance
        handle thousands of times at new branch lengths: grad_fn(blen) -> (ll, grad)
        and logf_fn(blen) -> ll.  The input and output buffers are allocated once and
        their addresses passed as plain integers, so a call costs two C calls and a
        copy of blen.  The returned grad array is reused by the next call (copy it to
        keep it).  A new topology on the same nodes (set_tree with N nodes again) keeps
        the binding valid; another node count needs a new bind()."""
        if self.M != 1:
            raise ValueError("bind() is for single-instance handles")
        n = self._N[0] - 1
        buf_b = np.empty(n, dtype=np.float64)
        buf_ll = np.empty(1, dtype=np.float64)
        buf_g = np.empty(n, dtype=np.float64)
        pb, pll, pg = buf_b.ctypes.data, buf_ll.ctypes.data, buf_g.ctypes.data
        raw = _lib.raw()
        setb, lg, lf = raw.set_branch_lengths, raw.logpdf_grad, raw.logpdf
        h = self._h.value

        def fail(st, what):
            check(st, self._h, what)

        def grad_fn(blen):
            np.copyto(buf_b, blen)
            st = setb(h, pb)
            if st:
                fail(st, "set_branch_lengths")
            st = lg(h, pll, pg)
            if st:
                fail(st, "logpdf_grad")
            return float(buf_ll[0]), buf_g

        def logf_fn(blen):
            np.copyto(buf_b, blen)
            st = setb(h, pb)
            if st:
                fail(st, "set_branch_lengths")
            st = lf(h, pll)
            if st:
                fail(st, "logpdf")
            return float(buf_ll[0])

        return grad_fn, logf_fn

    def logpdf_grad_device(self, d_ll_ptr: int, d_grad_ptr: int) -> None:
        check(self._L.mcphy_logpdf_grad_device(self._h, ctypes.c_void_p(d_ll_ptr),
                                               ctypes.c_void_p(d_grad_ptr)), self._h)

    def logpdf_device(self, d_ll_ptr: int) -> None:
        check(self._L.mcphy_logpdf_device(self._h, ctypes.c_void_p(d_ll_ptr)), self._h)

    def set_all_branch_lengths_device(self, d_blen_ptr: int) -> None:
        check(self._L.mcphy_set_all_branch_lengths_device(self._h, ctypes.c_void_p(d_blen_ptr)),
              self._h)

    def synchronize(self) -> None:
        check(self._L.mcphy_synchronize(self._h), self._h)

    def timing(self):
        ms = (ctypes.c_float * 3)()
        check(self._L.mcphy_get_timing(self._h, ms), self._h)
        return {"build_p_ms": ms[0], "prune_ms": ms[1], "reduce_ms": ms[2]}

    def counts(self):
        c = np.zeros(3, dtype=np.int64)
        check(self._L.mcphy_get_counts(self._h, _pi64(c)), self._h)
        return {"launches": int(c[0]), "units": int(c[1]), "scratch_bytes": int(c[2])}


def schedule_info(parent) -> dict:
    """Host-only: validate a parent array and describe its kernel schedule."""
    L = _lib.load()
    p = np.ascontiguousarray(parent, dtype=np.int64)
    out = np.zeros(5, dtype=np.int64)
    st = L.mcphy_schedule_info(len(p), _pi64(p), _pi64(out))
    if st != _lib.OK:
        raise ValueError("invalid tree (parent array)")
    return {"internal": int(out[0]), "virtual": int(out[1]), "leaves": int(out[2]),
            "max_depth": int(out[3]), "pre_slots": int(out[4])}
