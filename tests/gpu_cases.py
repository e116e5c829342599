"""Shared helpers for the GPU parity tests: random problems and the oracle call."""
import numpy as np

from oracle import pyoracle as O

import mcphylo_gb300 as mp
from mcphylo_gb300 import models, simulate
from mcphylo_gb300.tree import Node, number_nodes, post_order, to_parent


def collapse(tree: Node, rng, p: float) -> Node:
    """Merge a fraction p of internal edges into their parents (multifurcations)."""
    for n in list(post_order(tree)):
        if n.mother is not None and n.children and rng.random() < p:
            m = n.mother
            i = m.children.index(n)
            kids = n.children
            for k in kids:
                k.mother = m
                k.inc_length += 0.0
            m.children[i:i + 1] = kids
    number_nodes(tree)
    return tree


def caterpillar(n_taxa: int, rng, mean=0.1) -> Node:
    root = Node()
    cur = root
    for i in range(n_taxa - 1):
        a = cur.add_child(Node(f"t{i}"))
        a.inc_length = rng.exponential(mean)
        if i < n_taxa - 2:
            nxt = cur.add_child(Node())
        else:
            nxt = cur.add_child(Node(f"t{i + 1}"))
        nxt.inc_length = rng.exponential(mean)
        cur = nxt
    number_nodes(root)
    return root


def balanced(depth: int, rng, mean=0.1) -> Node:
    """A perfectly balanced binary tree of 2**depth leaves (the deepest partial stacks
    a tree of that size can need)."""
    count = [0]

    def grow(d):
        if d == 0:
            count[0] += 1
            return Node(f"t{count[0]}")
        n = Node()
        for _ in range(2):
            c = n.add_child(grow(d - 1))
            c.inc_length = rng.exponential(mean)
        return n

    root = grow(depth)
    number_nodes(root)
    return root


def random_instance(K, C, taxa, S, seed, multifurcate=0.0, missing=0.05, tree=None,
                    model="gtr"):
    rng = np.random.default_rng(seed)
    if tree is None:
        tree = simulate.yule_tree(taxa, rng, 0.15)
        if multifurcate:
            tree = collapse(tree, rng, multifurcate)
    pi = rng.dirichlet(np.full(K, 4.0))
    if model == "restriction" and K == 2:
        m = models.Restriction(pi)
    elif model == "jc":
        pi = np.ones(K) / K
        m = models.JC(pi)
    else:
        m = models.GTR(pi, rng.dirichlet(np.ones(K * (K - 1) // 2)) * K)
    rates = models.discrete_gamma_rates(0.7, 0.7, C) if C > 1 else np.array([1.0])
    return simulate._instance(tree, m, pi, rates, S, rng, missing)


def oracle(inst, blen=None):
    t = O.tree_from_parent(inst.parent, inst.blen if blen is None else blen)
    return O.gradlogpdf(t, inst.tensor(), inst.pi, (inst.U, inst.D, inst.Uinv, inst.mu),
                        inst.rates)


def oracle_ll(inst, blen=None):
    t = O.tree_from_parent(inst.parent, inst.blen if blen is None else blen)
    return O.logpdf(t, inst.tensor(), inst.pi, (inst.U, inst.D, inst.Uinv, inst.mu), inst.rates)


def level_fits(K, n_leaves, precision, warps=4):
    """Whether an item of the level-synchronous sweep fits one CTA's shared memory
    (the library's rule: records, post- and pre-order partials of every step of a
    32-site block, level plan and leaf codes, at most 100 KB)."""
    kp = 2 if K <= 2 else 4 if K <= 4 else 8 if K <= 8 else 0
    if not kp:
        return False
    b = 8 if precision == "f64" else 4
    J = n_leaves - 1
    rec = 48 + 4 * (kp + 1) * kp * b
    plan = (4 * (2 * J + 2) + 15) // 16 * 16
    total = J * rec + 2 * J * 32 * kp * b + warps * 32 * 4 + 32 * b + plan + (J + 1) * 32
    return total <= 100 * 1024


def engine(inst, precision, spt=0, dense=False):
    e = mp.Engine(inst.K, len(inst.rates), precision)
    if spt:
        e.set_tiles(spt, 0)
    e.set_tree(inst.parent, inst.blen)
    if dense:
        e.set_data(inst.tensor(), inst.leaf_nums)
    else:
        e.set_codes(inst.codes, inst.leaf_nums)
    e.set_model(inst.U, inst.D, inst.Uinv, inst.mu, inst.pi, inst.rates)
    return e


# Tolerances.  Plain FP64 path: logL within 1e-12 relative of the oracle; the gradient
# within 1e-10 of the oracle norm-wise, |g_i - go_i| <= 1e-10 * max_j |go_j|.  An entry
# is a sum of thousands of per-site terms that partly cancel, and each term inherits the
# conditioning of the eigenvector matrix U: on the 20-state case the oracle itself is
# ~1e-11 (norm-wise) away from an extended-precision evaluation of the same inputs
# (test_oracle_golden.py::test_fp64_gradient_conditioning), so 1e-12 is below what FP64
# can promise there.  FP32-scaled path: logL within 1e-6 relative; each gradient entry
# within 1e-4 relative to max(|go_i|, 1e-2 * max_j |go_j|).
F64_RTOL, F32_LL_RTOL, F32_G_RTOL = 1e-12, 1e-6, 1e-4
F64_G_RTOL = 1e-10
F64_G_FLOOR, F32_G_FLOOR = 1.0, 1e-2


def assert_grad_close(g, go, rtol, floor):
    g, go = np.asarray(g), np.asarray(go)
    scale = np.maximum(np.abs(go), floor * np.max(np.abs(go)))
    err = np.abs(g - go) / scale
    assert np.all(err <= rtol), (float(err.max()), int(err.argmax()))
    return float(err.max())
