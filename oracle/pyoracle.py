"""CPU FP64 oracle for the MCPhylo likelihood / branch-gradient path.

TEST INFRASTRUCTURE ONLY.  Only the tests, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` import this module,
and only as the checker or the timed CPU baseline.  The product package never
imports it.

Pieces restated from the reference (MCPhylo.jl v0.9.5; paths relative to the
reference project) and from its un-vendored tree dependency:

* Newick parsing and node numbering (MCPhyloTree 1.1, not vendored; its
  ``ParseNewick``/``post_order``/``get_branchlength_vector`` are restated from
  their documented behaviour: nodes are numbered 1..N in post-order, the root is
  N, and the branch-length vector is indexed by ``node.num``).  The rule is
  pinned by the gradient golden of test/likelihood/felsenstein.jl:37.
* ``ParseNexus`` / ``get_alphabet`` / ``extract_meta_info`` / ``create_nexusdf``
  (src/Parser/ParseNexus.jl:10-130) and ``datafortree`` (src/Parser/Parser.jl:48-85).
* Substitution models ``Restriction``/``JC``/``GTR``/``freeK``/``setmatrix``
  (src/Likelihood/SubstitutionModels.jl:13-113); LAPACK ``eigen``/``inv`` are
  numpy's ``eig``/``inv`` (P(t) is invariant to eigenvector sign and order).
* ``discrete_gamma_rates`` / ``mean_boundaries`` / ``median_boundaries``
  (src/Likelihood/Rates.jl:11-58); Distributions' ``Chisq`` quantile and
  SpecialFunctions' ``gamma_inc`` are scipy's ``chi2.ppf`` and ``gammainc``.
* The pruning loops themselves live in ``oracle.c`` (FP64, OpenMP), called via
  ctypes: ``logpdf``/``gradlogpdf`` follow src/distributions/Phylodist.jl:107-138.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None


# --------------------------------------------------------------------------- build/load
def build(force: bool = False) -> str:
    """Compile oracle.c into oracle/_build/liboracle.so with gcc + OpenMP."""
    src = os.path.join(_HERE, "oracle.c")
    if (not force and os.path.exists(_LIB_PATH)
            and os.path.getmtime(_LIB_PATH) >= os.path.getmtime(src)):
        return _LIB_PATH
    subprocess.check_call(["make", "-s", "-C", _HERE])
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        i64, dbl = ctypes.c_int64, ctypes.c_double
        P = ctypes.POINTER
        pi64, pd = P(i64), P(dbl)
        L.orc_logpdf.restype = dbl
        L.orc_logpdf.argtypes = [i64, pi64, pi64, pi64, pi64, i64, pd, pd, pd, pd, dbl,
                                 pd, pd, pd, i64, i64, i64]
        L.orc_gradlogpdf.restype = dbl
        L.orc_gradlogpdf.argtypes = [i64, pi64, pi64, pi64, pi64, pi64, i64, pd, pd, pd, pd,
                                     dbl, pd, pd, pd, i64, i64, i64, pd, pd]
        L.orc_parallel_transition_prob.restype = None
        L.orc_parallel_transition_prob.argtypes = [pd, pd, pd, pd, i64, dbl, pd, i64, i64, pd]
        L.orc_transition_grad.restype = None
        L.orc_transition_grad.argtypes = [pd, pd, pd, pd, i64, dbl, pd, i64, i64, pd]
        L.orc_num_threads.restype = ctypes.c_int
        L.orc_set_threads.argtypes = [ctypes.c_int]
        _lib = L
    return _lib


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


def num_threads() -> int:
    return int(lib().orc_num_threads())


def _p64(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))


def _pd(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


# --------------------------------------------------------------------------- trees
@dataclass(eq=False)
class ONode:
    name: str = ""
    inc_length: float = 0.0
    children: List["ONode"] = field(default_factory=list)
    mother: Optional["ONode"] = None
    num: int = 0

    @property
    def nchild(self) -> int:
        return len(self.children)


def post_order(root: ONode) -> List[ONode]:
    out: List[ONode] = []
    stack = [(root, False)]
    while stack:
        node, done = stack.pop()
        if done:
            out.append(node)
        else:
            stack.append((node, True))
            for c in reversed(node.children):
                stack.append((c, False))
    return out


def parse_newick(text: str) -> ONode:
    """Newick string -> tree, numbered by ``number_nodes``."""
    s = "".join(text.split())
    if not s.endswith(";"):
        raise ValueError("Newick string must end with ';'")
    pos = 0

    def label():
        nonlocal pos
        start = pos
        while pos < len(s) and s[pos] not in "(),:;":
            pos += 1
        return s[start:pos]

    def length():
        nonlocal pos
        if pos < len(s) and s[pos] == ":":
            pos += 1
            start = pos
            while pos < len(s) and s[pos] not in "(),;":
                pos += 1
            return float(s[start:pos])
        return 0.0

    def subtree():
        nonlocal pos
        node = ONode()
        if s[pos] == "(":
            pos += 1
            while True:
                c = subtree()
                c.mother = node
                node.children.append(c)
                if s[pos] == ",":
                    pos += 1
                    continue
                if s[pos] == ")":
                    pos += 1
                    break
                raise ValueError(f"bad Newick at {pos}")
        node.name = label()
        node.inc_length = length()
        return node

    root = subtree()
    if s[pos] != ";":
        raise ValueError("trailing characters in Newick string")
    number_nodes(root)
    return root


def number_nodes(root: ONode) -> None:
    """Leaves get 1..n in post-order, then internal nodes n+1..N in post-order
    (root = N).  This is the numbering the gradient golden of
    test/likelihood/felsenstein.jl:37 is indexed by."""
    po = post_order(root)
    k = 1
    for n in po:
        if n.nchild == 0:
            n.num = k
            k += 1
    for n in po:
        if n.nchild != 0:
            n.num = k
            k += 1


def flatten(root: ONode):
    """Tree -> (N, post, cptr, cidx, mother, leaf_nums, blv) as int64/float64 arrays."""
    po = post_order(root)
    N = len(po)
    by_num = sorted(po, key=lambda n: n.num)
    post = np.array([n.num for n in po], dtype=np.int64)
    cptr = np.zeros(N + 1, dtype=np.int64)
    cidx = []
    for i, n in enumerate(by_num):
        cidx.extend(c.num for c in n.children)
        cptr[i + 1] = len(cidx)
    mother = np.array([n.mother.num if n.mother is not None else 0 for n in by_num],
                      dtype=np.int64)
    leaf_nums = np.array([n.num for n in po if n.nchild == 0], dtype=np.int64)
    blv = np.array([n.inc_length for n in by_num if n.mother is not None], dtype=np.float64)
    return (N, post, cptr, np.asarray(cidx, dtype=np.int64), mother, leaf_nums, blv)


def tree_from_parent(parent: np.ndarray, blen: np.ndarray) -> ONode:
    """Build a tree from a 1-based parent array (root has parent 0) and a branch
    vector indexed by num-1.  Children are ordered by num."""
    N = len(parent)
    nodes = [ONode(name=str(i + 1), num=i + 1) for i in range(N)]
    root = None
    for i in range(N):
        p = int(parent[i])
        if p == 0:
            root = nodes[i]
        else:
            nodes[i].mother = nodes[p - 1]
            nodes[p - 1].children.append(nodes[i])
            nodes[i].inc_length = float(blen[i])
    return root


# --------------------------------------------------------------------------- NEXUS
def parse_nexus(path: str):
    """ParseNexus (src/Parser/ParseNexus.jl:10-35): returns
    (ntax, nchar, gap, missing, symbols, df (list of str rows), langs)."""
    with open(path) as f:
        content = [ln.rstrip("\n") for ln in f]
    if content[0].lower() != "#nexus":
        raise ValueError(f"{path} is not a Nexus file")
    while True:
        line = content.pop(0)
        if line.lower() == "begin data;":
            break
    ntax = nchar = 0
    gap, miss, symbols = "-", "?", "NOSYMBOLS"
    while True:
        line = content.pop(0)
        if "matrix" in line.lower():
            break
        for entry in line.split():
            info = [t.lower() for t in entry.split("=")]
            if len(info) != 1:
                v = info[1][:-1] if info[1].endswith(";") else info[1]
                if info[0] == "ntax":
                    ntax = int(v)
                elif info[0] == "nchar":
                    nchar = int(v)
                elif info[0] == "gap":
                    gap = v
                elif info[0] == "missing":
                    miss = v
                elif info[0] == "symbols":
                    symbols = v.strip('"')
    langs, rows = [], []
    while True:
        line = content.pop(0)
        if line == "":
            continue
        if line[-1] == ";":
            break
        lang, raw = line.split(None, 1)
        langs.append(lang)
        rows.append("".join(raw.strip()))
    if symbols == "NOSYMBOLS":
        alpha = set()
        for r in rows:
            for ch in r:
                if ch != gap and ch != miss:
                    alpha.add(ch)
        out_symbols = sorted(alpha)
    else:
        out_symbols = [c for c in symbols]
    return ntax, nchar, gap, miss, out_symbols, rows, langs


def datafortree(rows, langs, tree: ONode, symbols, gap, miss) -> np.ndarray:
    """datafortree (src/Parser/Parser.jl:48-85) with log_space=false.
    Returns x of shape (K, S, N), Fortran order; non-leaf slices are zero."""
    po = post_order(tree)
    N = len(po)
    K = len(symbols)
    S = len(rows[0])
    x = np.zeros((K, S, N), dtype=np.float64, order="F")
    by_name = {n.name: n for n in po}
    sym_index = {s: i for i, s in enumerate(symbols)}
    for ind, row in enumerate(rows):
        mind = by_name[langs[ind]].num - 1
        for j, ch in enumerate(row):
            idx = sym_index.get(ch)
            if idx is None:
                if ch == gap or ch == miss:
                    x[:, j, mind] = 1.0
                else:
                    raise ValueError(f"unknown symbol {ch}")
            else:
                x[:, j, mind] = 0.0
                x[idx, j, mind] = 1.0
    return x


# --------------------------------------------------------------------------- models
def setmatrix(vec_vals):
    """setmatrix (SubstitutionModels.jl:106-113)."""
    vec_vals = np.asarray(vec_vals, dtype=np.float64)
    n = len(vec_vals)
    s = int(round((np.sqrt(8 * n + 1) + 1) / 2))
    if s * (s - 1) // 2 != n:
        raise ValueError("setmatrix: length of vector is not triangular")
    Q = np.zeros((s, s))
    k = 0
    for j in range(s):          # column-major comprehension order: i fastest
        for i in range(s):
            if i < j:
                Q[i, j] = vec_vals[k]
                k += 1
    return Q + Q.T


def _eig(Q):
    D, U = np.linalg.eig(Q)
    order = np.lexsort((D.imag, D.real))
    D, U = D[order], U[:, order]
    if np.max(np.abs(D.imag)) == 0 and np.max(np.abs(U.imag)) == 0:
        D, U = D.real, U.real
    return U, D, np.linalg.inv(U)


def Restriction(base_freq, _rates=None):
    """SubstitutionModels.jl:13-24."""
    bf = np.asarray(base_freq, dtype=np.float64)
    if len(bf) != 2:
        raise AssertionError("Restriction needs 2 base frequencies")
    D = np.array([-1.0, 0.0])
    U = np.array([[bf[1], bf[1]], [-1.0 + bf[1], 0.0 + bf[1]]])
    return U, D, np.linalg.inv(U), 1.0 / (2.0 * np.prod(bf))


def JC(base_freq, _rates=None):
    """SubstitutionModels.jl:36-50 (mu = 1/((K-1)/K))."""
    K = len(base_freq)
    off = 1.0 / K
    dg = off * (K - 1)
    Q = np.full((K, K), off)
    np.fill_diagonal(Q, -dg)
    U, D, Uinv = _eig(Q)
    return U, D, Uinv, 1.0 / dg


def GTR(base_freq, rates):
    """SubstitutionModels.jl:62-74: Q_ij = x_ij * pi_j, mu = 1/sum(row sums)."""
    bf = np.asarray(base_freq, dtype=np.float64)
    Q = setmatrix(rates) * bf[None, :]
    dia = Q.sum(axis=1)
    np.fill_diagonal(Q, -dia)
    U, D, Uinv = _eig(Q)
    return U, D, Uinv, 1.0 / dia.sum()


def freeK(_base_freq, rates):
    """SubstitutionModels.jl:83-102: Q[j, i] filled column by column."""
    rates = np.asarray(rates, dtype=np.float64).ravel()
    nb = int(np.ceil(np.sqrt(len(rates))))
    Q = np.zeros((nb, nb))
    c = 0
    for i in range(nb):
        for j in range(nb):
            if i != j:
                Q[j, i] = rates[c]
                c += 1
    dia = Q.sum(axis=1)
    np.fill_diagonal(Q, -dia)
    U, D, Uinv = _eig(Q)
    return U, D, Uinv, 1.0 / dia.sum()


# --------------------------------------------------------------------------- rates
def mean_boundaries(alpha, beta, k):
    from scipy.stats import chi2
    return np.array([chi2.ppf(i / k, (2 * alpha) / (2 * beta)) / (2 * beta)
                     for i in range(1, k)] + [0.0])


def median_boundaries(alpha, beta, k):
    from scipy.stats import chi2
    return np.array([chi2.ppf(((i - 1) * 2 + 1) / (2 * k), (2 * alpha) / (2 * beta))
                     for i in range(1, k + 1)])


def discrete_gamma_rates(alpha, beta, k, method="mean"):
    """Rates.jl:11-38 (Yang 1994 discretisation as the reference writes it)."""
    from scipy.special import gammainc
    factor = alpha / beta * k
    if method == "median":
        m = median_boundaries(alpha, beta, k)
        return m * (factor / m.sum())
    m = mean_boundaries(alpha, beta, k)
    for i in range(k - 1):
        m[i] = gammainc(alpha + 1, m[i] * beta)
    m[k - 1] = 1.0
    for i in range(k - 1, 0, -1):
        m[i] -= m[i - 1]
        m[i] *= factor
    m[0] *= factor
    return m


# --------------------------------------------------------------------------- likelihood
def _prep(root, x, model_out, rates, blv=None):
    N, post, cptr, cidx, mother, leaf_nums, tblv = flatten(root)
    if blv is None:
        blv = tblv
    U, D, Uinv, mu = model_out
    if np.iscomplexobj(U) or np.iscomplexobj(D):
        raise ValueError("complex eigensystem: the reference's P(t) path needs a real one")
    K, S = x.shape[0], x.shape[1]
    xf = np.asfortranarray(x, dtype=np.float64)
    Uf = np.asfortranarray(U, dtype=np.float64)
    Uif = np.asfortranarray(Uinv, dtype=np.float64)
    Dd = np.ascontiguousarray(D, dtype=np.float64)
    rates = np.ascontiguousarray(rates, dtype=np.float64)
    blv = np.ascontiguousarray(blv, dtype=np.float64)
    return (N, post, cptr, cidx, mother, leaf_nums, xf, Uf, Dd, Uif, float(mu), rates, blv,
            K, S, len(rates))


def logpdf(root, x, pi, model_out, rates, blv=None) -> float:
    """logpdf(d::PhyloDist, x) (Phylodist.jl:107-122); model_out = (U, D, Uinv, mu)."""
    (N, post, cptr, cidx, mother, leaf_nums, xf, Uf, Dd, Uif, mu, rates, blv, K, S,
     C) = _prep(root, x, model_out, rates, blv)
    pi = np.ascontiguousarray(pi, dtype=np.float64)
    return lib().orc_logpdf(N, _p64(post), _p64(cptr), _p64(cidx), _p64(leaf_nums),
                            len(leaf_nums), _pd(xf), _pd(Uf), _pd(Dd), _pd(Uif), mu,
                            _pd(pi), _pd(rates), _pd(blv), K, S, C)


def gradlogpdf(root, x, pi, model_out, rates, blv=None, with_scale=False):
    """gradlogpdf(d::PhyloDist, x) (Phylodist.jl:124-138) -> (ll, grad[N-1]).

    with_scale=True also returns, per entry, the sum over sites and rates of the
    absolute values of the terms the entry adds up (the entry's condition number is
    scale / |grad|)."""
    (N, post, cptr, cidx, mother, leaf_nums, xf, Uf, Dd, Uif, mu, rates, blv, K, S,
     C) = _prep(root, x, model_out, rates, blv)
    pi = np.ascontiguousarray(pi, dtype=np.float64)
    grad = np.zeros(N - 1, dtype=np.float64)
    scale = np.zeros(N - 1, dtype=np.float64) if with_scale else None
    ll = lib().orc_gradlogpdf(N, _p64(post), _p64(cptr), _p64(cidx), _p64(mother),
                              _p64(leaf_nums), len(leaf_nums), _pd(xf), _pd(Uf), _pd(Dd),
                              _pd(Uif), mu, _pd(pi), _pd(rates), _pd(blv), K, S, C,
                              _pd(grad), _pd(scale) if with_scale else None)
    return (ll, grad, scale) if with_scale else (ll, grad)


def transition_matrices(model_out, rates, blv):
    """P (K,K,C,B) and dP/dt (K,K,C,B) in the reference layout, Fortran order."""
    U, D, Uinv, mu = model_out
    K = len(D)
    C = len(rates)
    B = len(blv)
    P = np.zeros((K, K, C, B), order="F")
    dP = np.zeros((K, K, C, B), order="F")
    Uf = np.asfortranarray(U, dtype=np.float64)
    Uif = np.asfortranarray(Uinv, dtype=np.float64)
    Dd = np.ascontiguousarray(D, dtype=np.float64)
    r = np.ascontiguousarray(rates, dtype=np.float64)
    b = np.ascontiguousarray(blv, dtype=np.float64)
    lib().orc_parallel_transition_prob(_pd(Uf), _pd(Dd), _pd(Uif), _pd(r), C, float(mu),
                                       _pd(b), B, K, _pd(P))
    lib().orc_transition_grad(_pd(Uf), _pd(Dd), _pd(Uif), _pd(r), C, float(mu), _pd(b), B,
                              K, _pd(dP))
    return P, dP
