"""Extended-precision (numpy longdouble) evaluation of logL and the branch
gradient, test infrastructure: it measures how far any FP64 evaluation (the
oracle's, the GPU's) is from a more precise one on the same inputs, which is
what the FP64 gradient tolerance has to allow for.

Besides (ll, grad) it can return, per gradient entry, the sum of the absolute
values of the per-(site, rate) terms that make it up.  Entry i is a sum of such
terms that partly cancel; its ratio to |g_i| is the entry's condition number.
"""
import numpy as np

from mcphylo_gb300.tree import nodes_by_num, post_order

LD = np.longdouble


def ext_grad(inst, with_scale=False):
    """(ll, grad[, scale]) in longdouble, the reference's recursion
    (LikelihoodCalculator_Node.jl:3-114) without rescaling of the post-order
    partials; pre-order partials are rescaled by their maximum (the gradient
    ratios are scale-free)."""
    K, C, S = inst.K, len(inst.rates), inst.S
    U, D, Ui = inst.U.astype(LD), inst.D.astype(LD), inst.Uinv.astype(LD)
    mu, r = LD(inst.mu), inst.rates.astype(LD)
    by = nodes_by_num(inst.tree)
    N = len(by)
    blen = inst.blen.astype(LD)
    P, dP = {}, {}
    for n in by[:-1]:
        for c in range(C):
            e = np.exp(mu * blen[n.num - 1] * D * r[c])
            P[n.num, c] = (U * e[None, :]) @ Ui
            dP[n.num, c] = (U * (D * r[c] * mu * e)[None, :]) @ Ui
    x = inst.tensor()
    L, Dn = {}, {}
    for n in post_order(inst.tree):
        if not n.children:
            L[n.num] = [x[:, :, n.num - 1].astype(LD) for _ in range(C)]   # (K, S) per rate
            continue
        L[n.num] = []
        for c in range(C):
            prod = np.ones((K, S), dtype=LD)
            for ch in n.children:
                d = P[ch.num, c] @ L[ch.num][c]
                Dn[ch.num, c] = d
                prod *= d
            L[n.num].append(prod)
    root = post_order(inst.tree)[-1]
    pi = inst.pi.astype(LD)
    ll = LD(0)
    for c in range(C):
        ll += np.sum(np.log(pi @ L[root.num][c]))
    pre = {}
    g = np.zeros(N - 1, dtype=LD)
    scale = np.zeros(N - 1, dtype=LD)
    for c in range(C):
        pre[root.num, c] = np.tile(pi[:, None], (1, S))
    for n in list(reversed(post_order(inst.tree)))[1:]:
        m = n.mother
        for c in range(C):
            pt = pre[m.num, c].copy()
            for s in m.children:
                if s is not n:
                    pt *= Dn[s.num, c]
            num = np.sum(pt * (dP[n.num, c] @ L[n.num][c]), axis=0)
            den = np.sum(pt * (P[n.num, c] @ L[n.num][c]), axis=0)
            g[n.num - 1] += np.sum(num / den)
            scale[n.num - 1] += np.sum(np.abs(num / den))
            pb = P[n.num, c].T @ pt
            pb /= pb.max(axis=0, keepdims=True)
            pre[n.num, c] = pb
    return (ll, g, scale) if with_scale else (ll, g)
