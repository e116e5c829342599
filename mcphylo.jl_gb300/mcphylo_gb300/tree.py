"""Rooted trees as MCPhylo uses them (the subset of MCPhyloTree 1.1 the
likelihood path needs; MCPhyloTree is a dependency of the reference, not part
of it).

Node numbering is MCPhyloTree's: leaves 1..n in post-order, then internal nodes
n+1..N in post-order, the root is N (the gradient vector of gradlogpdf is
indexed this way, test/likelihood/felsenstein.jl:37).  ``to_parent`` flattens a
tree into the (parent, blen) arrays the engine's C ABI takes.
"""
from __future__ import annotations

from typing import Iterator, List, Optional

import numpy as np


class Node:
    __slots__ = ("name", "inc_length", "children", "mother", "num")

    def __init__(self, name: str = "", inc_length: float = 0.0):
        self.name = name
        self.inc_length = float(inc_length)
        self.children: List["Node"] = []
        self.mother: Optional["Node"] = None
        self.num = 0

    @property
    def nchild(self) -> int:
        return len(self.children)

    @property
    def root(self) -> bool:
        return self.mother is None

    def add_child(self, c: "Node") -> "Node":
        c.mother = self
        self.children.append(c)
        return c

    def __repr__(self) -> str:
        return f"Node(num={self.num}, name={self.name!r}, nchild={self.nchild})"


def post_order(root: Node) -> List[Node]:
    out: List[Node] = []
    stack = [(root, False)]
    while stack:
        n, done = stack.pop()
        if done:
            out.append(n)
            continue
        stack.append((n, True))
        for c in reversed(n.children):
            stack.append((c, False))
    return out


def pre_order(root: Node) -> Iterator[Node]:
    stack = [root]
    while stack:
        n = stack.pop()
        yield n
        stack.extend(reversed(n.children))


def get_leaves(root: Node) -> List[Node]:
    return [n for n in post_order(root) if n.nchild == 0]


def number_nodes(root: Node) -> None:
    """Leaves first (post-order), then internal nodes (post-order); root = N."""
    po = post_order(root)
    k = 1
    for n in po:
        if n.nchild == 0:
            n.num = k
            k += 1
    for n in po:
        if n.nchild:
            n.num = k
            k += 1


def parse_newick(text: str) -> Node:
    """ParseNewick: whitespace is ignored, labels and ':length' are optional."""
    s = "".join(text.split())
    if not s.endswith(";"):
        raise ValueError("Newick string must end with ';'")
    n = len(s)
    stack: List[Node] = []
    cur: Optional[Node] = None
    root: Optional[Node] = None
    i = 0

    def read_label_length(node: Node, i: int) -> int:
        j = i
        while j < n and s[j] not in "(),:;":
            j += 1
        node.name = s[i:j]
        if j < n and s[j] == ":":
            k = j + 1
            while k < n and s[k] not in "(),;":
                k += 1
            node.inc_length = float(s[j + 1:k])
            j = k
        return j

    while i < n:
        ch = s[i]
        if ch == "(":
            node = Node()
            if stack:
                stack[-1].add_child(node)
            stack.append(node)
            i += 1
            if i < n and s[i] not in "(":
                leaf = Node()
                stack[-1].add_child(leaf)
                i = read_label_length(leaf, i)
            continue
        if ch == ",":
            i += 1
            if i < n and s[i] != "(":
                leaf = Node()
                stack[-1].add_child(leaf)
                i = read_label_length(leaf, i)
            continue
        if ch == ")":
            cur = stack.pop()
            i = read_label_length(cur, i + 1)
            if not stack:
                root = cur
            continue
        if ch == ";":
            break
        if root is None and not stack:      # a single-node tree "A;"
            root = Node()
            i = read_label_length(root, i)
            continue
        raise ValueError(f"bad Newick at position {i}")
    if root is None or stack:
        raise ValueError("unbalanced parentheses in Newick string")
    number_nodes(root)
    return root


ParseNewick = parse_newick


def newick(root: Node, digits: int = 17) -> str:
    def rec(n: Node) -> str:
        lab = n.name
        if n.children:
            lab = "(" + ",".join(rec(c) for c in n.children) + ")" + n.name
        if n.mother is not None:
            lab += ":" + repr(float(n.inc_length)) if digits >= 17 else f":{n.inc_length:.{digits}g}"
        return lab
    return rec(root) + ";"


def nodes_by_num(root: Node) -> List[Node]:
    po = post_order(root)
    out: List[Optional[Node]] = [None] * len(po)
    for n in po:
        out[n.num - 1] = n
    return out  # type: ignore[return-value]


def get_branchlength_vector(root: Node) -> np.ndarray:
    """blen[num-1] = inc_length of node num, for num = 1..N-1."""
    by = nodes_by_num(root)
    return np.array([n.inc_length for n in by[:-1]], dtype=np.float64)


def set_branchlength_vector(root: Node, blen) -> None:
    by = nodes_by_num(root)
    blen = np.asarray(blen, dtype=np.float64)
    if len(blen) != len(by) - 1:
        raise ValueError("branch-length vector must have N-1 entries")
    for n, b in zip(by[:-1], blen):
        n.inc_length = float(b)


def to_parent(root: Node):
    """(parent, blen) int64/float64 arrays: parent[num-1] = mother's num (0 = root)."""
    by = nodes_by_num(root)
    if by[-1].mother is not None:
        raise ValueError("the root must carry the largest num")
    parent = np.array([n.mother.num if n.mother is not None else 0 for n in by], dtype=np.int64)
    return parent, get_branchlength_vector(root)


def from_parent(parent, blen, names=None) -> Node:
    """Tree from a 1-based parent array (root = N, parent 0); children ordered by num."""
    parent = np.asarray(parent, dtype=np.int64)
    N = len(parent)
    nodes = [Node(name=(names[i] if names is not None else str(i + 1))) for i in range(N)]
    for i, nd in enumerate(nodes):
        nd.num = i + 1
    root = None
    for i in range(N):
        p = int(parent[i])
        if p == 0:
            root = nodes[i]
        else:
            nodes[p - 1].add_child(nodes[i])
            nodes[i].inc_length = float(blen[i])
    if root is None:
        raise ValueError("no root in parent array")
    return root


def find_by_name(root: Node, name: str) -> Node:
    for n in post_order(root):
        if n.name == name:
            return n
    raise KeyError(name)
