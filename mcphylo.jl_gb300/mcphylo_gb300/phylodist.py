"""PhyloDist / MultiplePhyloDist with the reference's logpdf / gradlogpdf
contract (src/distributions/Phylodist.jl:8-300), evaluated by the GB300 engine.

    pd = PhyloDist(tree, base_freq, substitution_rates, rates, JC)
    ll = logpdf(pd, x)                 # x: (K, S, N) FP64, leaves at x[:, :, num-1]
    ll, grad = gradlogpdf(pd, x)       # grad[num-1] = d logL / d blen[num-1]

Each PhyloDist keeps one engine handle.  A call re-sends only what changed
since the previous call: the topology (after an NNI move), the branch lengths,
the model, or the data.  ``precision`` selects the plain FP64 path ("f64", the
default, matching the reference to 1e-12) or the FP32-scaled path ("f32").
"""
from __future__ import annotations

from numbers import Real
from typing import List, Optional

import numpy as np

from . import _lib
from .engine import Engine
from .models import freeK, freeK_equilibrium
from .parse import codes_from_tensor
from .tree import Node, get_leaves, post_order, to_parent


def _vec(v) -> np.ndarray:
    if isinstance(v, Real):
        return np.array([float(v)])
    return np.array(v, dtype=np.float64).ravel()


class PhyloDist:
    """Distribution whose likelihood is computed with Felsenstein's algorithm.

    PhyloDist(tree, base_freq, substitution_rates, rates, substitution_model)
    PhyloDist(tree, substitution_rates, rates, freeK)   # base_freq = freeK equilibrium
    """

    def __init__(self, tree, *args, precision: str = "f64"):
        tree = getattr(tree, "value", tree)          # a Stochastic/TreeVariate wrapper
        if len(args) == 3 and args[2] is freeK:
            substitution_rates, rates, model = args
            base_freq = freeK_equilibrium(_vec(substitution_rates))
        elif len(args) == 4:
            base_freq, substitution_rates, rates, model = args
        else:
            raise TypeError("PhyloDist(tree, base_freq, substitution_rates, rates, model) "
                            "or PhyloDist(tree, substitution_rates, rates, freeK)")
        self.tree: Node = tree
        self.base_freq = _vec(base_freq)
        self.substitution_rates = _vec(substitution_rates)
        self.rates = _vec(rates)
        self.substitution_model = model
        self.nbase = len(self.base_freq)
        self.nnodes = len(post_order(tree))
        self.precision = precision
        self._eng: Optional[Engine] = None
        self._cache = {}

    # Base.size / minimum / maximum (Phylodist.jl:102-105)
    @property
    def size(self):
        return (self.nbase, 1, self.nnodes)

    def minimum(self) -> float:
        return -np.inf

    def maximum(self) -> float:
        return np.inf

    def __eq__(self, other) -> bool:
        if not isinstance(other, PhyloDist):
            return NotImplemented
        return (self.tree is other.tree and np.array_equal(self.base_freq, other.base_freq)
                and np.array_equal(self.substitution_rates, other.substitution_rates)
                and np.array_equal(self.rates, other.rates)
                and self.substitution_model is other.substitution_model
                and self.nbase == other.nbase and self.nnodes == other.nnodes)

    __hash__ = object.__hash__

    # ------------------------------------------------------------------ engine sync
    def _engine(self) -> Engine:
        if self._eng is None:
            self._eng = Engine(self.nbase, len(self.rates), self.precision)
        return self._eng

    def _sync(self, x: np.ndarray) -> Engine:
        eng = self._engine()
        c = self._cache
        x = np.asarray(x)
        if x.ndim != 3 or x.shape[0] != self.nbase:
            raise _lib.DimensionMismatch(_lib.ERR_SHAPE,
                                         f"x must be ({self.nbase}, S, N), got {x.shape}")
        parent, blen = to_parent(self.tree)
        if x.shape[2] != len(parent):
            raise _lib.DimensionMismatch(_lib.ERR_SHAPE, "x has a different number of nodes "
                                         "than the tree")
        leaf_nums = np.array(sorted(n.num for n in get_leaves(self.tree)), dtype=np.int64)
        if "parent" not in c or not np.array_equal(c["parent"], parent):
            eng.set_tree(parent, blen)
            c["parent"] = parent
            c["blen"] = blen
        elif not np.array_equal(c["blen"], blen):
            eng.set_branch_lengths(blen)
            c["blen"] = blen
        leaf = x[:, :, leaf_nums - 1]
        if ("leaf" not in c or c["leaf"].shape != leaf.shape or not np.array_equal(c["leaf"], leaf)
                or not np.array_equal(c["leaf_nums"], leaf_nums)):
            codes, ok = codes_from_tensor(x, leaf_nums)
            if ok:
                eng.set_codes(codes, leaf_nums)
            else:
                eng.set_data(x, leaf_nums)
            c["leaf"] = np.array(leaf, copy=True)
            c["leaf_nums"] = leaf_nums
        key = (self.substitution_model, self.base_freq.tobytes(),
               self.substitution_rates.tobytes(), self.rates.tobytes())
        if c.get("model") != key:
            U, D, Uinv, mu = self.substitution_model(self.base_freq, self.substitution_rates)
            eng.set_model(U, D, Uinv, mu, self.base_freq, self.rates)
            c["model"] = key
        return eng


def logpdf(d, x) -> float:
    """logpdf(d::PhyloDist, x) (Phylodist.jl:107-122) and
    logpdf(d::MultiplePhyloDist, x) (Phylodist.jl:281-288)."""
    if isinstance(d, MultiplePhyloDist):
        return float(np.sum(d._eval(x, want_grad=False)[0]))
    return d._sync(x).logpdf()


def gradlogpdf(d: PhyloDist, x):
    """gradlogpdf(d::PhyloDist, x) (Phylodist.jl:124-138) -> (ll, grad[N-1])."""
    return d._sync(x).logpdf_grad()


class MultiplePhyloDist:
    """A batch of PhyloDists (Phylodist.jl:143-272), evaluated in one launch.

    MultiplePhyloDist(trees, base_freq, substitution_rates, rates, model)
      base_freq / substitution_rates / rates: (k, n_trees) arrays, or one column
      (or vector / scalar) shared by all trees; other widths raise DimensionMismatch.
    MultiplePhyloDist(trees, substitution_rates, rates, freeK)
    """

    def __init__(self, trees: List[Node], *args, precision: str = "f64"):
        n_t = len(trees)

        def widen(a, what):
            a = np.asarray(a, dtype=np.float64)
            if a.ndim <= 1:
                a = a.reshape(-1, 1)
            if a.shape[1] == n_t:
                return a
            if a.shape[1] == 1:
                return np.repeat(a, n_t, axis=1)
            raise _lib.DimensionMismatch(_lib.ERR_SHAPE,
                                         f"Size of {what} and tree_array are incompatible")

        if len(args) == 3 and args[2] is freeK:
            sr, rates, model = args
            sr = widen(sr, "substitution_rates")
            bf = np.stack([freeK_equilibrium(sr[:, i]) for i in range(n_t)], axis=1)
            rates = np.asarray(rates, dtype=np.float64)
            rates = rates.reshape(-1, 1) if rates.ndim <= 1 else rates
        elif len(args) == 4:
            bf, sr, rates, model = args
            bf = widen(bf, "base_freq")
            sr = widen(sr, "substitution_rates")
            rates = widen(rates, "rates")
        else:
            raise TypeError("MultiplePhyloDist(trees, base_freq, substitution_rates, rates, model)")
        rates_w = rates if rates.shape[1] == n_t else np.repeat(rates, n_t, axis=1)
        self.DistCollector = [PhyloDist(t, bf[:, i], sr[:, i], rates_w[:, i], model,
                                        precision=precision) for i, t in enumerate(trees)]
        self.size_array = np.array([d.nnodes for d in self.DistCollector], dtype=np.int64)
        self.precision = precision
        self._eng: Optional[Engine] = None
        self._cache = {}

    @property
    def size(self):
        return (len(self.DistCollector[0].base_freq), 1, int(self.size_array.max()),
                len(self.size_array))

    def minimum(self) -> float:
        return -np.inf

    def maximum(self) -> float:
        return np.inf

    def __eq__(self, other) -> bool:
        if not isinstance(other, MultiplePhyloDist):
            return NotImplemented
        return (len(self.DistCollector) == len(other.DistCollector)
                and all(a == b for a, b in zip(self.DistCollector, other.DistCollector)))

    __hash__ = object.__hash__

    def _eval(self, x, want_grad: bool):
        x = np.asarray(x)
        M = len(self.DistCollector)
        d0 = self.DistCollector[0]
        if x.ndim != 4 or x.shape[3] != M:
            raise _lib.DimensionMismatch(_lib.ERR_SHAPE, "x must be (K, S, Nmax, n_trees)")
        if self._eng is None:
            self._eng = Engine(d0.nbase, len(d0.rates), self.precision, n_instances=M)
        eng = self._eng
        c = self._cache
        for i, d in enumerate(self.DistCollector):
            xi = x[:, :, :self.size_array[i], i]
            parent, blen = to_parent(d.tree)
            leaf_nums = np.array(sorted(n.num for n in get_leaves(d.tree)), dtype=np.int64)
            ci = c.setdefault(i, {})
            if "parent" not in ci or not np.array_equal(ci["parent"], parent):
                eng.set_tree(parent, blen, i)
                ci["parent"], ci["blen"] = parent, blen
            elif not np.array_equal(ci["blen"], blen):
                eng.set_branch_lengths(blen, i)
                ci["blen"] = blen
            leaf = xi[:, :, leaf_nums - 1]
            if "leaf" not in ci or ci["leaf"].shape != leaf.shape or not np.array_equal(ci["leaf"], leaf):
                codes, ok = codes_from_tensor(xi, leaf_nums)
                if ok:
                    eng.set_codes(codes, leaf_nums, i)
                else:
                    eng.set_data(np.asfortranarray(xi), leaf_nums, i)
                ci["leaf"] = np.array(leaf, copy=True)
            key = (d.substitution_model, d.base_freq.tobytes(), d.substitution_rates.tobytes(),
                   d.rates.tobytes())
            if ci.get("model") != key:
                U, D, Uinv, mu = d.substitution_model(d.base_freq, d.substitution_rates)
                eng.set_model(U, D, Uinv, mu, d.base_freq, d.rates, i)
                ci["model"] = key
        if want_grad:
            ll, g = eng.logpdf_grad()
            ll = np.atleast_1d(ll)
            off = eng.grad_offsets()
            return ll, [g[off[i]:off[i + 1]] for i in range(M)]
        return np.atleast_1d(eng.logpdf()), None


def __logpdf(d: MultiplePhyloDist, x):
    """__logpdf(::MultiplePhyloDist, x) (Phylodist.jl:290-297): a list of
    (ll, grad) per tree."""
    ll, grads = d._eval(x, want_grad=True)
    return [(float(ll[i]), grads[i]) for i in range(len(ll))]


multiple_gradlogpdf = __logpdf
