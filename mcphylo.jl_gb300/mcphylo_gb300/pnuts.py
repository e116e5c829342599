"""PNUTS: the No-U-Turn sampler over a tree's branch lengths with refraction and
NNI moves, driving the engine for logL + gradient at every leapfrog step.

Restated from src/samplers/pnuts.jl:103-419 (sample!, dual_averaging, setadapt!,
nuts_sub!, buildtree, nouturn), src/samplers/tree_hamiltonian/refraction.jl:2-91
(refraction!, ref_NNI!), tree_hamiltonian/auxilliary.jl:1-50 and :204-210
(jitter, nutsepsilon, scale_fac, molifier) and tree_hamiltonian/states.jl
(Tree_HMC_State, Extendend_Tree_HMC_State, transfer!, NUTS_StepParams).

The host arithmetic follows the reference step for step in FP64, including its
quirks, which are kept on purpose:
  - both trajectory ends of nuts_sub! start with direction -1 (pnuts.jl:197-198);
  - the gradient at the start of a trajectory is scaled with the lengths before the
    molifier (pnuts.jl:189-195);
  - transfer! between tree states copies every field but att_nni (states.jl), so a
    state taken from an extension reports att_nni = 0.
Random numbers come from numpy's generator, so sample paths differ from Julia's;
their distribution does not.

A tree is (parent, blen): parent[num-1] = the mother's num (0 for the root) and
blen[num-1] = the length of the branch above node num, num = 1..N-1.  Node numbers
stay with nodes through NNI moves, as in MCPhyloTree.  The three MCPhyloTree
operations the sampler uses (NNI!, internal_external, BHV_bounds) are restated here
from their definitions: MCPhyloTree is not part of the reference sources.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field
from typing import Callable, Dict, List, Optional, Tuple

import numpy as np
from scipy.special import gammaln


# ----------------------------------------------------------------------------- helpers
def molifier(x, delta):
    """x if x >= delta else (x^2 + delta^2) / (2 delta)  (auxilliary.jl:208-210)."""
    x = np.asarray(x, dtype=np.float64)
    return np.where(x >= delta, x, (x * x + delta * delta) / (2.0 * delta))


def scale_fac(x, delta):
    """d molifier / dx: x / delta if x < delta else 1  (auxilliary.jl:204-206)."""
    x = np.asarray(x, dtype=np.float64)
    return np.where(x < delta, x / delta, 1.0)


def logaddexp(a: float, b: float) -> float:
    return float(np.logaddexp(a, b))


def internal_external(parent: np.ndarray) -> np.ndarray:
    """MCPhyloTree.internal_external: entry num-1 is 1 when node num has children,
    0 for a leaf (num = 1..N-1)."""
    p = np.asarray(parent, dtype=np.int64)
    N = len(p)
    has_child = np.zeros(N, dtype=bool)
    has_child[p[p > 0] - 1] = True
    return has_child[:N - 1].astype(np.int64)


def nni(parent: np.ndarray, target: int, rng: np.random.Generator) -> Tuple[np.ndarray, int]:
    """MCPhyloTree.NNI!(tree, target): a nearest-neighbour interchange across the
    branch above node `target` -- one of its children (chosen at random) trades
    places with one of its siblings (chosen at random).  Returns (new parent
    array, 1), or (parent, 0) when target is a leaf, the root or has no sibling."""
    p = int(parent[target - 1])
    if p == 0:
        return parent, 0
    children = np.flatnonzero(parent == target) + 1
    if len(children) == 0:
        return parent, 0
    siblings = np.flatnonzero(parent == p) + 1
    siblings = siblings[siblings != target]
    if len(siblings) == 0:
        return parent, 0
    c = int(children[rng.integers(len(children))])
    s = int(siblings[rng.integers(len(siblings))])
    new = parent.copy()
    new[c - 1] = p
    new[s - 1] = target
    return new, 1


class _Clusters:
    """Leaf set below every non-root node as a Python-int bitmask (one bit per leaf,
    bits in leaf-num order), for each topology seen (cached by topology)."""

    def __init__(self, capacity: int = 64):
        self._cache: Dict[bytes, List[int]] = {}
        self._cap = capacity

    def __call__(self, parent: np.ndarray) -> List[int]:
        key = np.ascontiguousarray(parent, dtype=np.int64).tobytes()
        hit = self._cache.get(key)
        if hit is not None:
            return hit
        par = [int(v) for v in parent]
        N = len(par)
        kids: List[List[int]] = [[] for _ in range(N)]
        root = -1
        for n, v in enumerate(par):
            if v > 0:
                kids[v - 1].append(n)
            else:
                root = n
        mask = [0] * N
        bit = 0
        for n in range(N):
            if not kids[n]:
                mask[n] = 1 << bit
                bit += 1
        order = []
        stack = [root]
        while stack:
            n = stack.pop()
            order.append(n)
            stack.extend(kids[n])
        for n in reversed(order):           # children before parents
            if par[n] > 0:
                mask[par[n] - 1] |= mask[n]
        out = mask[:N - 1]
        if len(self._cache) >= self._cap:
            self._cache.clear()
        self._cache[key] = out
        return out


_clusters = _Clusters()


def bhv_bounds(t1, t2) -> Tuple[float, float]:
    """MCPhyloTree.BHV_bounds: lower and upper bounds of the BHV geodesic distance
    between two trees on the same leaves.  Splits in both trees contribute their
    length differences; the splits A of one tree only and B of the other only
    contribute ||A||^2 + ||B||^2 to the lower bound (both in one orthant) and
    (||A|| + ||B||)^2 to the upper bound (the path through the cone point)."""
    p1, b1 = t1
    p2, b2 = t2
    b1 = np.asarray(b1, dtype=np.float64)
    b2 = np.asarray(b2, dtype=np.float64)
    if np.array_equal(p1, p2):
        d = float(np.sqrt(np.sum((b1 - b2) ** 2)))
        return d, d
    c1 = _clusters(p1)
    c2 = _clusters(p2)
    where2 = {c: i for i, c in enumerate(c2)}
    idx1 = np.array([where2.get(c, -1) for c in c1])
    common = idx1 >= 0
    seen = np.zeros(len(c2), dtype=bool)
    seen[idx1[common]] = True
    d_common = float(np.sum((b1[common] - b2[idx1[common]]) ** 2))
    a = float(np.sum(b1[~common] ** 2))
    b = float(np.sum(b2[~seen] ** 2))
    lower = math.sqrt(d_common + a + b)
    upper = math.sqrt(d_common + (math.sqrt(a) + math.sqrt(b)) ** 2)
    return lower, upper


# ----------------------------------------------------------------------------- priors
@dataclass
class ExponentialBL:
    """exponentialBL(scale): i.i.d. Exponential(scale) branch lengths
    (src/distributions/TreeDistribution.jl:8-13, src/Likelihood/Prior.jl:50-57,80-83)."""
    scale: float = 1.0

    def logpdf_grad(self, parent, blen):
        z = self.scale
        v = float(np.sum(-math.log(z) - np.asarray(blen) / z))
        return v, np.full(len(blen), -1.0 / z)


@dataclass
class CompoundDirichlet:
    """CompoundDirichlet(alpha, a, beta, c) tree-length prior
    (src/Likelihood/Prior.jl:1-48); the gradient is the analytic derivative of
    internal_logpdf."""
    alpha: float = 1.0
    a: float = 1.0
    beta: float = 0.1
    c: float = 1.0

    def _topology(self, parent):
        """Per topology (cached): the weight of each log branch length, a - 1 for a
        leaf branch and a c - 1 for an internal one, and the exponent of the tree
        length, alpha - a n_term - a c (n_term - 3)."""
        cache = self.__dict__.setdefault("_cache", {})
        key = np.ascontiguousarray(parent, dtype=np.int64).tobytes()
        hit = cache.get(key)
        if hit is None:
            internal = internal_external(parent) == 1
            a, c = self.a, self.c
            nterm = float(np.sum(~internal))
            w = np.where(internal, a * c - 1.0, a - 1.0)
            coef = self.alpha - a * nterm - a * c * (nterm - 3.0)
            if len(cache) >= 64:
                cache.clear()
            hit = cache[key] = (w, coef)
        return hit

    def logpdf_grad(self, parent, blen):
        blen = np.asarray(blen, dtype=np.float64)
        w, coef = self._topology(parent)
        al, a, be, c = self.alpha, self.a, self.beta, self.c
        t_l = float(np.sum(blen))
        const = al * math.log(be) - gammaln(al) - gammaln(a) - gammaln(c) + gammaln(a + c)
        v = const - t_l * be + float(np.dot(w, np.log(blen))) + coef * math.log(t_l)
        g = w / blen + (coef / t_l - be)
        return float(v), g


class TreePosterior:
    """log posterior of (parent, blen) = engine log-likelihood + tree prior: the
    `logfgrad` / `logf` pair the sampler calls (the model's logpdf of every
    stochastic node that depends on the tree).

    The engine's topology is re-sent only when it changed.  With a second engine
    (`proposal_engine`, same data and model), an NNI proposal is evaluated there,
    so a rejected proposal leaves the main engine's schedule in place and an
    accepted one makes the two engines trade places."""

    def __init__(self, engine, parent, blen, prior=None, proposal_engine=None):
        self.eng = engine
        self.prop = proposal_engine
        self.prior = prior
        self._parent = np.asarray(parent, dtype=np.int64).copy()
        self._prop_parent: Optional[np.ndarray] = None
        engine.set_tree(self._parent, blen)
        self.n_set_tree = 0
        # per engine: (grad_fn, logf_fn) bound to its handle (Engine.bind)
        self._bound = {}

    def _fns(self, e):
        f = self._bound.get(id(e))
        if f is None:
            f = self._bound[id(e)] = e.bind()
        return f

    def _main(self, parent):
        """The engine holding `parent`, its topology updated when needed (the branch
        lengths are sent by the evaluation itself)."""
        if np.array_equal(parent, self._parent):
            pass
        elif self._prop_parent is not None and np.array_equal(parent, self._prop_parent):
            self.eng, self.prop = self.prop, self.eng
            self._parent, self._prop_parent = self._prop_parent, self._parent
        else:
            self.eng.set_tree(parent)
            self._parent = np.asarray(parent, dtype=np.int64).copy()
            self.n_set_tree += 1
        return self.eng

    def _prior(self, parent, blen):
        if self.prior is None:
            return 0.0, 0.0
        return self.prior.logpdf_grad(parent, blen)

    def logfgrad(self, parent, blen):
        ll, g = self._fns(self._main(parent))[0](blen)
        lp, gp = self._prior(parent, blen)
        return ll + lp, g + gp

    def logf(self, parent, blen):
        if self.prop is not None and not np.array_equal(parent, self._parent):
            if self._prop_parent is None or not np.array_equal(parent, self._prop_parent):
                self.prop.set_tree(parent)
                self._prop_parent = np.asarray(parent, dtype=np.int64).copy()
                self.n_set_tree += 1
            ll = self._fns(self.prop)[1](blen)
        else:
            ll = self._fns(self._main(parent))[1](blen)
        return ll + self._prior(parent, blen)[0]


def engine_posterior(parent, blen, codes, leaf_nums, model_out, pi, rates, prior=None,
                     precision: str = "f32", proposals: bool = True,
                     graph: bool = True) -> TreePosterior:
    """A TreePosterior over engines holding one alignment: `codes` is the
    (n_leaves, S) state-bitmask array of leaf_nums' rows, model_out the
    substitution model's (U, D, Uinv, mu)."""
    from .engine import Engine

    U, D, Uinv, mu = model_out
    engines = []
    tiles = sweep = None
    for _ in range(2 if proposals else 1):
        e = Engine(len(pi), len(rates), precision)
        e.set_tree(parent, blen)
        e.set_codes(codes, leaf_nums)
        e.set_model(U, D, Uinv, mu, pi, rates)
        if tiles is None:
            # a chain evaluates the same problem thousands of times: time the launch
            # shapes once, and give the proposal engine the same one
            tiles = e.autotune()
            sweep = e.sweep() if precision in ("f32", "f64") else None
        else:
            e.set_tiles(*tiles)
            if sweep is not None:
                e.set_sweep(sweep)
        if graph:
            e.enable_graph(True)
        engines.append(e)
    return TreePosterior(engines[0], parent, blen, prior,
                         engines[1] if proposals else None)


# ----------------------------------------------------------------------------- states
@dataclass
class TreeState:
    """Tree_HMC_State (states.jl): position (tree), momentum, gradient, log density."""
    parent: np.ndarray
    blen: np.ndarray
    r: np.ndarray
    g: np.ndarray
    lf: float
    extended: bool = False
    nni: int = 0
    att_nni: int = 0

    def copy(self) -> "TreeState":
        return TreeState(self.parent.copy(), self.blen.copy(), self.r.copy(), self.g.copy(),
                         self.lf, self.extended, self.nni, self.att_nni)

    def assign(self, o: "TreeState") -> None:
        """transfer!(self, o): every field but att_nni."""
        self.parent = o.parent.copy()
        self.blen = o.blen.copy()
        self.r = o.r.copy()
        self.g = o.g.copy()
        self.lf = o.lf
        self.extended = o.extended
        self.nni = o.nni

    def tree(self):
        return self.parent, self.blen

    def hamiltonian(self) -> float:
        return self.lf - 0.5 * float(self.r @ self.r)


class ExtState:
    """Extendend_Tree_HMC_State (states.jl): a trajectory end, the state one
    leapfrog step further (computed by nouturn, reused by the next buildtree) and
    the direction."""

    def __init__(self, s: TreeState, direction: int):
        self.curr = s.copy()
        self.ext = s.copy()
        self.extended = False
        self.direction = direction

    def copy(self) -> "ExtState":
        o = ExtState.__new__(ExtState)
        o.curr = self.curr.copy()
        o.ext = self.ext.copy()
        o.extended = self.extended
        o.direction = self.direction
        return o

    def unextend(self) -> None:
        self.curr.assign(self.ext)
        self.extended = False

    def extend(self, s: TreeState) -> None:
        self.ext.assign(s)
        self.extended = True

    def hamiltonian(self) -> float:
        return self.curr.hamiltonian()


@dataclass
class Meta:
    """NUTSMeta (states.jl)."""
    nni: int = 0
    alpha: float = 0.0
    nalpha: float = 0.0
    accnni: int = 0
    att_nni: int = 0
    l_NNI: int = 0


# ----------------------------------------------------------------------------- sampler
class PNUTS:
    """PNUTS(params; target=0.6, tree_depth=10, targetNNI=0.5, delta=0.003,
    jitter=0.0) (pnuts.jl:4-94) over one tree.  `logfgrad(parent, blen) ->
    (logf, grad)` and `logf(parent, blen) -> logf` evaluate the log posterior.
    `sample(adapt)` is one iteration of sample! (pnuts.jl:103-143).

    `plus_end_forward=True` is a variant that is NOT the reference's behaviour: the
    plus end of every trajectory starts with direction +1 instead of -1
    (pnuts.jl:197-198 starts both ends with -1).  It exists to measure what that
    quirk costs in mixing; parity runs leave it off."""

    def __init__(self, parent, blen, logfgrad: Callable, logf: Callable, *, target=0.6,
                 tree_depth=10, targetNNI=0.5, delta=0.003, jitter=0.0, epsilon=-math.inf,
                 rng: Optional[np.random.Generator] = None, max_refractions=1_000_000,
                 plus_end_forward: bool = False):
        if not 0.0 <= jitter <= 1.0:
            raise ValueError("jitter must lie in [0, 1]")
        self.parent = np.asarray(parent, dtype=np.int64).copy()
        self.blen = np.asarray(blen, dtype=np.float64).copy()
        if len(self.blen) != len(self.parent) - 1:
            raise ValueError("blen must have N-1 entries")
        self.logfgrad = logfgrad
        self.logf = logf
        self.tree_depth = int(tree_depth)
        self.delta = float(delta)
        self.jitter_amt = float(jitter)
        self.epsilon = float(epsilon)
        self.rng = rng if rng is not None else np.random.default_rng()
        self.max_refractions = max_refractions
        self.plus_end_forward = bool(plus_end_forward)
        # NUTSstepadapter(0, 0.0, 0.0, NUTS_StepParams(0.5, target, 0.05, 0.75, 10, targetNNI))
        self.m = 0
        self.s_bar = 0.0
        self.x_bar = 0.0
        self.mu_p = 0.5
        self.delta_p = float(target)
        self.gamma_p = 0.05
        self.kappa_p = 0.75
        self.t0_p = 10
        self.delta_nni = float(targetNNI)
        self.metro_acc_prob = 0.0
        self.nni_stat = 0.0
        self.adapt = False
        self.moves: List[int] = []
        self.att_moves: List[int] = []
        self.tree_depth_trace: List[int] = []
        self.acc_p_r: List[int] = []
        self.lf = math.nan
        self.n_grad_evals = 0
        self.n_logf_evals = 0

    # -- checkpoint / resume (the sampler state a Chains file carries in the
    #    reference, output/fileio.jl:15-35 and model/mcmc.jl:17-58)
    _STATE = ("parent", "blen", "tree_depth", "delta", "jitter_amt", "epsilon", "m", "s_bar",
              "x_bar", "mu_p", "delta_p", "gamma_p", "kappa_p", "t0_p", "delta_nni",
              "metro_acc_prob", "nni_stat", "adapt", "moves", "att_moves", "tree_depth_trace",
              "acc_p_r", "lf", "n_grad_evals", "n_logf_evals", "max_refractions",
              "plus_end_forward")

    def state(self) -> dict:
        """Everything needed to continue the chain: tree, step-size adapter, traces
        and the random generator's state (a picklable dict)."""
        out = {k: (v.copy() if isinstance(v, (np.ndarray, list)) else v)
               for k, v in ((k, getattr(self, k)) for k in self._STATE)}
        out["rng"] = self.rng.bit_generator.state
        out["rng_kind"] = type(self.rng.bit_generator).__name__
        return out

    @classmethod
    def from_state(cls, state: dict, logfgrad: Callable, logf: Callable) -> "PNUTS":
        """A sampler that continues exactly where the one `state` came from."""
        bg = getattr(np.random, state["rng_kind"])()
        bg.state = state["rng"]
        s = cls(state["parent"], state["blen"], logfgrad, logf, rng=np.random.Generator(bg))
        for k in cls._STATE:
            if k not in state:   # a state saved before the field existed
                continue
            v = state[k]
            setattr(s, k, v.copy() if isinstance(v, (np.ndarray, list)) else v)
        return s

    # -- evaluation counting
    def _fg(self, parent, blen):
        self.n_grad_evals += 1
        lf, g = self.logfgrad(parent, blen)
        return float(lf), np.asarray(g, dtype=np.float64)

    def _f(self, parent, blen) -> float:
        self.n_logf_evals += 1
        return float(self.logf(parent, blen))

    # -- refraction.jl
    def refraction(self, s: TreeState, eps: float, delta: float) -> Tuple[int, int]:
        """refraction!: half momentum step, position step with reflections at zero
        length (NNI across internal branches), molifier, gradient, half step."""
        blenvec = s.blen.copy()
        s.r = s.r + (eps * 0.5) * s.g
        tmpB = blenvec + eps * s.r
        tmpB, nni_n, att = self.ref_nni(s, tmpB, eps, blenvec, delta)
        blenvec = molifier(tmpB, delta)
        s.blen = blenvec
        lf, grad = self._fg(s.parent, s.blen)
        grad = grad * scale_fac(blenvec, delta)
        s.r = s.r + (eps * 0.5) * grad
        s.g = grad.copy()
        s.lf = lf
        return nni_n, att

    def ref_nni(self, s: TreeState, tmpB, eps, blv, delta):
        """ref_NNI!: while a length is non-positive, reflect the branch with the
        smallest tmpB/|r|; across an internal branch, try an NNI and keep it when
        the momentum pays for the change in log density.  The internal/leaf map is
        taken once, before the loop, as in the reference."""
        intext = internal_external(s.parent)
        t = 0.0
        nni_n = 0
        att = 0
        guard = 0
        while np.min(tmpB) <= 0.0:
            guard += 1
            if guard > self.max_refractions:
                raise RuntimeError("refraction did not terminate")
            with np.errstate(divide="ignore"):      # r_i = 0: time +-inf, as in Julia
                timelist = tmpB / np.abs(s.r)
            ref_index = int(np.argmin(timelist))
            temp = eps - t + timelist[ref_index]
            blv = np.abs(blv + temp * s.r)
            s.r[ref_index] *= -1.0
            if intext[ref_index] == 1:
                s.blen = molifier(blv, delta)
                u_before = self._f(s.parent, s.blen)
                new_parent, made = nni(s.parent, ref_index + 1, self.rng)
                if made != 0:
                    att += 1
                    u_after = self._f(new_parent, s.blen)
                    delta_u = 2.0 * (u_before - u_after)
                    my_v = s.r[ref_index] ** 2
                    if my_v > delta_u:
                        nni_n += made
                        s.r[ref_index] = math.sqrt(my_v - delta_u)
                        s.parent = new_parent
            t = eps + timelist[ref_index]
            tmpB = blv + (eps - t) * s.r
        return tmpB, nni_n, att

    # -- pnuts.jl
    def nouturn(self, xminus: ExtState, xplus: ExtState, eps: float, delta: float) -> bool:
        """True while the BHV distance between the trajectory ends still grows:
        upper bound now <= lower bound one step further."""
        _, curr_h = bhv_bounds(xminus.curr.tree(), xplus.curr.tree())
        for st in (xminus, xplus):
            if not st.extended:
                xt = st.curr.copy()
                n, a = self.refraction(xt, st.direction * eps, delta)
                xt.nni = n
                xt.att_nni = a
                st.extend(xt)
        curr_t_l, _ = bhv_bounds(xminus.ext.tree(), xplus.ext.tree())
        return curr_h <= curr_t_l

    def buildtree(self, x: ExtState, pm: int, j: int, eps: float, logp0: float, lu: float,
                  delta: float, meta: Meta, lsw_subtree: float):
        if j == 0:
            if not x.extended:
                nni_n, att = self.refraction(x.curr, pm * eps, delta)
            else:
                x.unextend()
                nni_n, att = x.curr.nni, x.curr.att_nni
            logpprime = -x.hamiltonian()
            lsw_subtree = logaddexp(lsw_subtree, logp0 - logpprime)
            meta.att_nni += att
            sprime = lu + (logpprime - logp0) < 1000.0
            meta.nni += nni_n
            d = logp0 - logpprime
            if math.isnan(d):
                alphaprime = -math.inf
            else:
                alphaprime = 1.0 if d >= 0.0 else math.exp(d)
            meta.alpha += alphaprime
            nprime = 0
            if logp0 + lu < logpprime:
                nprime = 1
                meta.accnni += nni_n
            meta.nalpha += 1
            meta.l_NNI += att
            return x.curr.copy(), x.copy(), x.copy(), nprime, sprime, lsw_subtree
        lsw_init = -math.inf
        lsw_final = -math.inf
        xprime, xplus, xminus, nprime, sprime, lsw_init = self.buildtree(
            x, pm, j - 1, eps, logp0, lu, delta, meta, lsw_init)
        if sprime:
            if pm == -1:
                worker, _, xminus, nprime2, sprime2, lsw_final = self.buildtree(
                    x, pm, j - 1, eps, logp0, lu, delta, meta, lsw_final)
            else:
                worker, xplus, _, nprime2, sprime2, lsw_final = self.buildtree(
                    x, pm, j - 1, eps, logp0, lu, delta, meta, lsw_final)
            ls_final = logaddexp(lsw_init, lsw_final)
            if lsw_final > ls_final:
                xprime.assign(worker)
            elif self.rng.random() < math.exp(lsw_final - ls_final):
                xprime.assign(worker)
            nprime += nprime2
            lsw_subtree = logaddexp(lsw_subtree, ls_final)
            sprime = sprime2 and self.nouturn(xplus, xminus, eps, delta)
        return xprime, xplus, xminus, nprime, sprime, lsw_subtree

    def nuts_sub(self, eps: float) -> None:
        """nuts_sub!: one trajectory, doubling until a U-turn or tree_depth."""
        delta = self.delta
        blv = self.blen.copy()
        r = self.rng.standard_normal(len(blv))
        bl_m = molifier(blv, delta)
        logf, grad = self._fg(self.parent, bl_m)
        grad = grad * scale_fac(blv, delta)
        s0 = TreeState(self.parent.copy(), bl_m.copy(), r.copy(), grad.copy(), logf)
        if math.isnan(self.lf):
            self.lf = logf
        xminus = ExtState(s0, -1)
        xplus = ExtState(s0, 1 if self.plus_end_forward else -1)
        lu = math.log(self.rng.random())
        logp0 = -xminus.hamiltonian()
        nni_acc = 0
        tnni = 0
        j = 0
        meta = Meta()
        lsw = 0.0
        acc = 0
        ds = 0
        while j < self.tree_depth:
            pm = self.rng.random() > 0.5
            meta.nalpha = 0
            meta.alpha = 0.0
            meta.l_NNI = 0
            lsw_sub = -math.inf
            if pm:
                xprime, _, xminus, nprime, sprime, lsw_sub = self.buildtree(
                    xminus, xminus.direction, j, eps, logp0, lu, delta, meta, lsw_sub)
            else:
                xprime, xplus, _, nprime, sprime, lsw_sub = self.buildtree(
                    xplus, xplus.direction, j, eps, logp0, lu, delta, meta, lsw_sub)
            ds += meta.nalpha
            ratio = meta.alpha / meta.nalpha
            self.metro_acc_prob = 1.0 if ratio > 1 else ratio
            tnni += meta.nni
            if not sprime:
                break
            if lsw_sub > lsw or self.rng.random() < math.exp(lsw_sub - lsw):
                acc += 1
                self.parent = xprime.parent.copy()
                self.blen = xprime.blen.copy()
                self.lf = xprime.lf
                nni_acc += meta.nni
            lsw = logaddexp(lsw, lsw_sub)
            j += 1
            if not self.nouturn(xminus, xplus, eps, delta):
                break
        self.nni_stat = 0.0 if ds == 0 else meta.att_nni / ds
        self.moves.append(nni_acc)
        self.att_moves.append(tnni)
        self.tree_depth_trace.append(j)
        self.acc_p_r.append(acc)

    # -- step size
    def nutsepsilon(self) -> float:
        """auxilliary.jl:6-50: double or halve a trial step from 1.0 until the
        acceptance of one refraction step crosses the target."""
        log_target = math.log(self.delta_p)
        logf0, gr = self._fg(self.parent, self.blen)
        n = len(self.blen)
        x0 = TreeState(self.parent.copy(), self.blen.copy(), self.rng.standard_normal(n),
                       gr.copy(), logf0)
        x1 = x0.copy()
        h0 = -x0.hamiltonian()
        eps = 1.0
        self.refraction(x0, eps, 2 * eps)
        prob = h0 + x0.hamiltonian()
        direction = 1 if prob > log_target else -1
        it = 0
        while (prob > log_target) if direction == 1 else (prob < log_target):
            it += 1
            if it > 200:
                raise RuntimeError("step size search did not converge")
            eps = 2 * eps if direction == 1 else 0.5 * eps
            x1.r = self.rng.standard_normal(n)
            h0 = -x1.hamiltonian()
            x2 = x1.copy()
            self.refraction(x2, eps, 2 * eps)
            prob = h0 + x2.hamiltonian()
        return eps

    def dual_averaging(self) -> float:
        """pnuts.jl:145-161."""
        ht = self.delta_p - self.metro_acc_prob
        eta = 1.0 / (self.m + self.t0_p)
        self.s_bar = (1.0 - eta) * self.s_bar + eta * ht
        x = self.mu_p - self.s_bar * math.sqrt(self.m) / self.gamma_p
        x_eta = self.m ** -self.kappa_p
        self.x_bar = (1.0 - x_eta) * self.x_bar + x_eta * x
        return x

    def set_adapt(self, adapt: bool) -> None:
        """setadapt! (pnuts.jl:164-177)."""
        if adapt and not self.adapt:
            self.m = 0
            self.mu_p = math.log(10.0 * self.epsilon)
        self.adapt = adapt

    def sample(self, adapt: bool = False) -> None:
        """sample! (pnuts.jl:103-143)."""
        if self.m == 0 and math.isinf(self.epsilon):
            self.epsilon = self.nutsepsilon()
        self.set_adapt(adapt)
        if self.adapt:
            self.m += 1
            self.delta = 2 * self.epsilon
            self.nuts_sub(self.epsilon)
            self.epsilon = math.exp(self.dual_averaging())
        else:
            if self.m > 0:
                self.epsilon = math.exp(self.x_bar)
            self.delta = 2 * self.epsilon
            eps = self.epsilon * (1.0 + self.jitter_amt * (2.0 * self.rng.random() - 1.0))
            self.nuts_sub(eps)


# ----------------------------------------------------------------------------- ESS
def mcse_bm(x, size: int = 100) -> float:
    """Batch-means Monte Carlo standard error (src/output/mcse.jl:26-34)."""
    x = np.asarray(x, dtype=np.float64)
    m = len(x) // size
    if m < 2:
        raise ValueError(f"iterations are < {2 * size} and batch size is > {len(x) // 2}")
    mbar = x[:m * size].reshape(m, size).mean(axis=1)
    return float(np.std(mbar, ddof=1) / math.sqrt(m))


def ess(x, size: int = 100) -> float:
    """ESS column of summarystats: min((SD / MCSE_bm)^2, n)
    (src/output/stats.jl:167-172)."""
    x = np.asarray(x, dtype=np.float64)
    se = mcse_bm(x, size)
    sd = float(np.std(x, ddof=1))
    if se == 0.0:
        return float(len(x))
    return float(min((sd / se) ** 2, len(x)))


@dataclass
class Chain:
    """Draws of one PNUTS chain after adaptation, with its wall-clock time."""
    seconds: float
    logf: np.ndarray          # log posterior of each draw
    tree_length: np.ndarray   # sum of branch lengths of each draw
    blen: np.ndarray          # (n_iter, N-1) branch lengths by num
    depth: np.ndarray
    nni_moves: np.ndarray
    grad_evals: int
    logf_evals: int
    epsilon: float
    adapt_seconds: float = 0.0
    extra: dict = field(default_factory=dict)

    def ess(self, size: int = 100) -> dict:
        out = {"logf": ess(self.logf, size), "tree_length": ess(self.tree_length, size)}
        per = [ess(self.blen[:, i], size) for i in range(self.blen.shape[1])]
        out["blen_min"] = float(np.min(per))
        out["blen_median"] = float(np.median(per))
        return out


def run_chain(parent, blen, logfgrad, logf, n_iter: int, n_adapt: int = 0, seed: int = 0,
              **kw) -> Chain:
    """n_adapt adaptation iterations, then n_iter timed sampling iterations."""
    s = PNUTS(parent, blen, logfgrad, logf, rng=np.random.default_rng(seed), **kw)
    t0 = time.perf_counter()
    for _ in range(n_adapt):
        s.sample(True)
    t_adapt = time.perf_counter() - t0
    lf = np.empty(n_iter)
    tl = np.empty(n_iter)
    bl = np.empty((n_iter, len(s.blen)))
    g0, f0 = s.n_grad_evals, s.n_logf_evals
    t0 = time.perf_counter()
    for it in range(n_iter):
        s.sample(False)
        lf[it] = s.lf
        tl[it] = float(np.sum(s.blen))
        bl[it] = s.blen
    secs = time.perf_counter() - t0
    return Chain(secs, lf, tl, bl, np.array(s.tree_depth_trace[-n_iter:]),
                 np.array(s.moves[-n_iter:]), s.n_grad_evals - g0, s.n_logf_evals - f0,
                 s.epsilon, t_adapt)
