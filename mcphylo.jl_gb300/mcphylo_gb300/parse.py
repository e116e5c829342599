"""Input formats feeding the likelihood path: NEXUS character matrices and the
(K, S, N) leaf tensor (src/Parser/ParseNexus.jl:10-130, src/Parser/Parser.jl:48-85),
plus state-bitmask codes, the compact leaf form the engine stores on the device.
"""
from __future__ import annotations

from typing import List, Sequence, Tuple

import numpy as np

from .tree import Node, post_order


class FileSyntaxError(ValueError):
    pass


def ParseNexus(filename: str):
    """-> (ntax, nchar, gap, missing, symbols, rows, langs).  rows[i] is taxon
    langs[i]'s character string; symbols are sorted unless the file lists them."""
    with open(filename) as f:
        content = [ln.rstrip("\r\n") for ln in f]
    if not content or content[0].lower() != "#nexus":
        raise FileSyntaxError(f"{filename} is not a Nexus file!")
    pos = 0
    while True:
        if pos >= len(content):
            raise FileSyntaxError("no 'begin data;' block")
        line = content[pos]
        pos += 1
        if line.lower() == "begin data;":
            break
    ntax = nchar = 0
    gap, miss, symbols = "-", "?", "NOSYMBOLS"
    while True:
        line = content[pos]
        pos += 1
        if "matrix" in line.lower():
            break
        for entry in line.split():
            kv = [t.lower() for t in entry.split("=")]
            if len(kv) == 1:
                continue
            val = kv[1][:-1] if kv[1].endswith(";") else kv[1]
            if kv[0] == "ntax":
                ntax = int(val)
            elif kv[0] == "nchar":
                nchar = int(val)
            elif kv[0] == "gap":
                gap = val
            elif kv[0] == "missing":
                miss = val
            elif kv[0] == "symbols":
                symbols = val.strip('"')
    langs: List[str] = []
    rows: List[str] = []
    while pos < len(content):
        line = content[pos]
        pos += 1
        if line == "":
            continue
        if line[-1] == ";":
            break
        name, raw = line.split(None, 1)
        langs.append(name)
        rows.append(raw.strip())
    if symbols == "NOSYMBOLS":
        out_symbols = get_alphabet(rows, gap, miss)
    else:
        out_symbols = [c for c in symbols]
    return ntax, nchar, gap, miss, out_symbols, rows, langs


def get_alphabet(rows: Sequence[str], gap: str, miss: str) -> List[str]:
    return sorted({ch for r in rows for ch in r if ch != gap and ch != miss})


def leaf_codes(rows: Sequence[str], symbols: Sequence[str], gap: str, miss: str) -> np.ndarray:
    """(ntaxa, S) uint32 state bitmasks: one bit for a symbol, all K bits for gap
    or missing (datafortree's all-ones column)."""
    K = len(symbols)
    allm = (1 << K) - 1
    lut = {s: 1 << i for i, s in enumerate(symbols)}
    lut[gap] = allm
    lut[miss] = allm
    out = np.empty((len(rows), len(rows[0])), dtype=np.uint32)
    for i, r in enumerate(rows):
        try:
            out[i] = [lut[ch] for ch in r]
        except KeyError as e:
            raise ValueError(f"unknown symbol {e.args[0]}, {list(symbols)}") from None
    return out


def datafortree(rows, langs, tree: Node, symbols, gap, miss, log_space: bool = False) -> np.ndarray:
    """The reference's (K, S, N) data tensor, Fortran order, leaves at x[:, :, num-1].
    Non-leaf slices are zero (the reference leaves them uninitialised; they are
    never read)."""
    po = post_order(tree)
    N = len(po)
    K = len(symbols)
    codes = leaf_codes(rows, symbols, gap, miss)
    S = codes.shape[1]
    x = np.zeros((K, S, N), dtype=np.float64, order="F")
    by_name = {n.name: n for n in po}
    bits = ((codes[:, :, None] >> np.arange(K, dtype=np.uint32)) & 1).astype(np.float64)
    for i, name in enumerate(langs):
        x[:, :, by_name[name].num - 1] = bits[i].T
    if log_space:
        with np.errstate(divide="ignore"):
            x = np.log(x)
    return x


def codes_from_tensor(x: np.ndarray, leaf_nums) -> Tuple[np.ndarray, bool]:
    """(K, S, N) tensor -> ((n_leaves, S) uint32 bitmasks, True) when every leaf
    entry is 0 or 1, else (None, False)."""
    K = x.shape[0]
    sl = np.stack([x[:, :, n - 1] for n in leaf_nums])          # (L, K, S)
    if not np.all((sl == 0.0) | (sl == 1.0)):
        return None, False
    w = (1 << np.arange(K, dtype=np.uint64))[None, :, None]
    return (sl.astype(np.uint64) * w).sum(axis=1).astype(np.uint32), True


def compress_patterns(codes: np.ndarray) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Site-pattern compression of an (n_leaves, S) code matrix: the distinct
    columns, in order of first appearance, how often each occurs (the weights
    Engine.set_weights takes) and, for every original site, its pattern's index.
    logL and the gradient over the weighted patterns equal those over all sites.
    (The reference evaluates every column; this is an input-side saving.)"""
    c = np.ascontiguousarray(np.asarray(codes).T)
    if c.shape[0] == 0:
        return np.asarray(codes)[:, :0], np.zeros(0), np.zeros(0, dtype=np.int64)
    view = c.view(np.dtype((np.void, c.dtype.itemsize * c.shape[1])))[:, 0]
    _, first, inverse, counts = np.unique(view, return_index=True, return_inverse=True,
                                          return_counts=True)
    order = np.argsort(first, kind="stable")          # patterns by first appearance
    rank = np.empty_like(order)
    rank[order] = np.arange(len(order))
    patterns = np.asarray(codes)[:, first[order]]
    return patterns, counts[order].astype(np.float64), rank[inverse.ravel()].astype(np.int64)
