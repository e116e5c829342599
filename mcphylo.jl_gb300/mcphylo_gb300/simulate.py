"""Seeded synthetic inputs for tests and benchmarks (the reference ships no tree
or sequence simulator): Yule and birth-death trees, sequences simulated down a
tree under a substitution model with Gamma rate categories, missing cells, and
the workload generators used by the benchmark.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from . import models
from .tree import Node, number_nodes, post_order, pre_order, to_parent


def yule_tree(n_taxa: int, rng: np.random.Generator, mean_blen: float = 0.1) -> Node:
    """Random rooted binary topology by Yule splitting; branch lengths Exp(mean)."""
    root = Node()
    tips = [root]
    while len(tips) < n_taxa:
        k = int(rng.integers(len(tips)))
        t = tips.pop(k)
        a, b = t.add_child(Node()), t.add_child(Node())
        tips.extend([a, b])
    for i, t in enumerate(tips):
        t.name = f"t{i}"
    for n in post_order(root):
        if n.mother is not None:
            n.inc_length = float(rng.exponential(mean_blen))
    number_nodes(root)
    return root


def birth_death_tree(n_taxa: int, rng: np.random.Generator, lam: float = 1.0, mu: float = 0.5,
                     height: float = 1.0) -> Node:
    """Birth-death tree grown forward in time until n_taxa lineages are alive
    (extinct lineages pruned), rescaled to root height ``height``."""
    while True:
        root = Node()
        birth = {id(root): 0.0}
        alive = [root]
        t = 0.0
        while 0 < len(alive) < n_taxa:
            rate = (lam + mu) * len(alive)
            t += rng.exponential(1.0 / rate)
            k = int(rng.integers(len(alive)))
            nd = alive.pop(k)
            nd.inc_length = t - birth[id(nd)]
            if rng.random() < lam / (lam + mu):
                for _ in range(2):
                    c = nd.add_child(Node())
                    birth[id(c)] = t
                    alive.append(c)
            else:
                nd.name = "extinct"
        if len(alive) == n_taxa:
            break
    # observe the tree one waiting time after the last event, so that no tip
    # born in it has length zero
    t += rng.exponential(1.0 / ((lam + mu) * n_taxa))
    for nd in alive:
        nd.inc_length = t - birth[id(nd)]
    # prune extinct tips and suppress unary nodes
    def prune(n: Node) -> Optional[Node]:
        if not n.children:
            return None if n.name == "extinct" else n
        kids = [k for k in (prune(c) for c in n.children) if k is not None]
        n.children = []
        for k in kids:
            n.add_child(k)
        if not kids:
            return None
        if len(kids) == 1:
            only = kids[0]
            only.inc_length += n.inc_length
            only.mother = None
            return only
        return n
    root = prune(root)
    root.mother = None
    # rescale to the requested root height
    depth = {id(root): 0.0}
    h = 0.0
    for n in pre_order(root):
        for c in n.children:
            depth[id(c)] = depth[id(n)] + c.inc_length
            h = max(h, depth[id(c)])
    for n in post_order(root):
        if n.mother is not None:
            n.inc_length *= height / h
    for i, leaf in enumerate(n for n in post_order(root) if not n.children):
        leaf.name = f"t{i}"
    number_nodes(root)
    return root


def transition(U, D, Uinv, mu, t, r) -> np.ndarray:
    P = (U * np.exp(mu * t * np.asarray(D) * r)[None, :]) @ Uinv
    P = np.clip(np.real(P), 0.0, None)
    return P / P.sum(axis=1, keepdims=True)


def simulate_codes(tree: Node, model_out, pi, rates, n_sites: int, rng: np.random.Generator,
                   missing: float = 0.0):
    """Simulate n_sites columns down the tree; each site draws one of the rate
    categories uniformly.  Returns (leaf_nums sorted, codes (n_leaves, S) uint32
    bitmasks); a fraction ``missing`` of cells becomes all-ones."""
    U, D, Uinv, mu = model_out
    K = len(pi)
    pi = np.asarray(pi, dtype=np.float64)
    rates = np.asarray(rates, dtype=np.float64)
    C = len(rates)
    cat = rng.integers(C, size=n_sites)
    root = tree
    cum0 = np.cumsum(pi / pi.sum())
    state = {id(root): np.minimum(np.searchsorted(cum0, rng.random(n_sites), side="right"), K - 1)
             .astype(np.int8)}
    for n in pre_order(root):
        ps = state.pop(id(n)) if n.children else state[id(n)]
        for c in n.children:
            # cumulative transition rows for every rate: (C, K, K), gathered per site
            cum = np.stack([np.cumsum(transition(U, D, Uinv, mu, c.inc_length, r), axis=1)
                            for r in rates]).astype(np.float32)
            rows = cum[cat, ps]                                  # (S, K)
            u = rng.random(n_sites, dtype=np.float32)
            state[id(c)] = np.minimum((u[:, None] > rows).sum(axis=1), K - 1).astype(np.int8)
    leaves = sorted((n for n in post_order(root) if not n.children), key=lambda n: n.num)
    codes = np.empty((len(leaves), n_sites), dtype=np.uint32)
    allm = (1 << K) - 1
    for i, lf in enumerate(leaves):
        codes[i] = np.left_shift(np.uint32(1), state[id(lf)].astype(np.uint32))
        if missing > 0:
            codes[i][rng.random(n_sites) < missing] = allm
    return np.array([lf.num for lf in leaves], dtype=np.int64), codes


def codes_to_tensor(codes: np.ndarray, leaf_nums, K: int, N: int) -> np.ndarray:
    """(n_leaves, S) bitmasks -> the reference's (K, S, N) FP64 tensor (Fortran order)."""
    S = codes.shape[1]
    x = np.zeros((K, S, N), dtype=np.float64, order="F")
    bits = ((codes[:, :, None] >> np.arange(K, dtype=np.uint32)) & 1).astype(np.float64)
    for i, n in enumerate(leaf_nums):
        x[:, :, n - 1] = bits[i].T
    return x


@dataclass
class Instance:
    """One (tree, data, model) problem in engine form."""
    tree: Node
    parent: np.ndarray
    blen: np.ndarray
    leaf_nums: np.ndarray
    codes: np.ndarray
    U: np.ndarray
    D: np.ndarray
    Uinv: np.ndarray
    mu: float
    pi: np.ndarray
    rates: np.ndarray
    weights: Optional[np.ndarray] = None
    meta: dict = field(default_factory=dict)

    @property
    def K(self) -> int:
        return len(self.pi)

    @property
    def S(self) -> int:
        return self.codes.shape[1]

    @property
    def N(self) -> int:
        return len(self.parent)

    def units(self) -> int:
        return (self.N - 1) * self.S * len(self.rates)

    def tensor(self) -> np.ndarray:
        return codes_to_tensor(self.codes, self.leaf_nums, self.K, self.N)


def _instance(tree, model_out, pi, rates, S, rng, missing=0.0, **meta) -> Instance:
    leaf_nums, codes = simulate_codes(tree, model_out, pi, rates, S, rng, missing)
    parent, blen = to_parent(tree)
    U, D, Uinv, mu = model_out
    return Instance(tree, parent, blen, leaf_nums, codes, np.asarray(U, float), np.asarray(D, float),
                    np.asarray(Uinv, float), float(mu), np.asarray(pi, float),
                    np.asarray(rates, float), meta=meta)


# --------------------------------------------------------------------- workloads
def restriction_small(seed: int = 1, S: int = 1000, taxa: int = 32) -> Instance:
    """2-state restriction model, one rate, Yule tree, Exp(0.1) lengths,
    pi = (0.4, 0.6), 5% missing leaf cells."""
    rng = np.random.default_rng(seed)
    tree = yule_tree(taxa, rng, 0.1)
    pi = np.array([0.4, 0.6])
    return _instance(tree, models.Restriction(pi), pi, np.array([1.0]), S, rng, 0.05,
                     name="restriction-k2-c1")


def gtr_gamma(seed: int = 2, S: int = 100_000, taxa: int = 128, alpha: float = 0.5,
              with_weights: bool = True) -> Instance:
    """4-state GTR+G4: exchangeabilities ~ Dir(1^6), pi ~ Dir(5^4), Yule tree with
    Exp(0.05) lengths, Gamma shape 0.5.  Pattern weights Poisson(1)+1 are drawn
    (the reference has no weights: a weight w equals w repeated columns)."""
    rng = np.random.default_rng(seed)
    ex = rng.dirichlet(np.ones(6))
    pi = rng.dirichlet(np.full(4, 5.0))
    tree = yule_tree(taxa, rng, 0.05)
    rates = models.discrete_gamma_rates(alpha, alpha, 4)
    inst = _instance(tree, models.GTR(pi, ex), pi, rates, S, rng, 0.0, name="gtr-g4-k4",
                     exchangeabilities=ex)
    if with_weights:
        inst.weights = rng.poisson(1.0, size=S) + 1
    return inst


def restriction_gamma_bd(seed: int = 3, S: int = 20_000, taxa: int = 512) -> Instance:
    """2-state restriction +G4 (shape 1.0), birth-death tree (lambda=1, mu=0.5)
    rescaled to height 1."""
    rng = np.random.default_rng(seed)
    tree = birth_death_tree(taxa, rng, 1.0, 0.5, 1.0)
    pi = np.array([0.4, 0.6])
    rates = models.discrete_gamma_rates(1.0, 1.0, 4)
    return _instance(tree, models.Restriction(pi), pi, rates, S, rng, 0.0,
                     name="restriction-g4-k2-bd512")


def _hky_one(args) -> Instance:
    seed, i, T, S, kappa, pi, alpha = args
    rng = np.random.default_rng([seed, i])
    tree = yule_tree(T, rng, 0.1)
    rates = models.discrete_gamma_rates(alpha, alpha, 4)
    return _instance(tree, models.HKY(pi, kappa), pi, rates, S, rng, 0.0,
                     name=f"hky-g4-{i}", kappa=kappa)


def hky_batch(seed: int = 4, n: int = 256, taxa=(16, 1024), sites=(500, 50_000),
              alpha: float = 0.5, scale: float = 1.0, workers: int = 0) -> List[Instance]:
    """Uneven batch: per instance T ~ logU[16,1024], S ~ logU[500,50000],
    HKY+G4 (shape ``alpha``) with kappa ~ LogNormal(1, 0.5), pi ~ Dir(5^4), Yule
    tree with Exp(0.1) lengths.  ``scale`` < 1 shrinks the site counts (for
    tests).  ``workers`` > 1 simulates instances in a spawn-started process pool;
    the result does not depend on the worker count."""
    rng = np.random.default_rng(seed)
    jobs = []
    for i in range(n):
        T = int(round(np.exp(rng.uniform(np.log(taxa[0]), np.log(taxa[1])))))
        S = max(1, int(round(np.exp(rng.uniform(np.log(sites[0]), np.log(sites[1]))) * scale)))
        kappa = float(rng.lognormal(1.0, 0.5))
        pi = rng.dirichlet(np.full(4, 5.0))
        jobs.append((seed, i, T, S, kappa, pi, alpha))
    if workers and workers > 1:
        import multiprocessing as mp_
        with mp_.get_context("spawn").Pool(workers) as pool:
            return pool.map(_hky_one, jobs, chunksize=1)
    return [_hky_one(j) for j in jobs]


def protein_gamma(seed: int = 5, S: int = 50_000, taxa: int = 256, alpha: float = 0.5) -> Instance:
    """20-state reversible +G4: exchangeabilities ~ Dir(1^190), pi ~ Dir(2^20),
    Yule tree with Exp(0.1) lengths."""
    rng = np.random.default_rng(seed)
    ex = rng.dirichlet(np.ones(190))
    pi = rng.dirichlet(np.full(20, 2.0))
    tree = yule_tree(taxa, rng, 0.1)
    rates = models.discrete_gamma_rates(alpha, alpha, 4)
    return _instance(tree, models.GTR(pi, ex), pi, rates, S, rng, 0.0, name="gtr20-g4-k20")
