"""Site-sharded evaluation across ranks: one tree, its sites split in contiguous
blocks, one all-reduce per evaluation.

logL and its branch-length gradient are sums over sites (and the reference's
product over rate categories is a sum of logs per site), so rank r evaluating
sites [s0_r, s1_r) and an all-reduce (sum) of the FP64 vector [ll | grad] gives
the whole-alignment result.  The exchange is 8 (1 + N-1) bytes per evaluation,
never partials.  Branch lengths and topology must be identical on every rank
(the sampler runs on every rank with the same seed, or on rank 0 with a
broadcast of the proposal).

On GPUs each rank owns an Engine on its own device over its shard and the
process group is NCCL; the same code runs over gloo with any per-rank evaluator.
"""
from __future__ import annotations

from typing import Callable, Optional, Tuple

import numpy as np


def site_range(n_sites: int, rank: int, world: int) -> Tuple[int, int]:
    """Balanced contiguous block of sites for `rank` (sizes differ by at most one)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank / world")
    base, extra = divmod(n_sites, world)
    s0 = rank * base + min(rank, extra)
    return s0, s0 + base + (1 if rank < extra else 0)


class ShardedEval:
    """`evaluate(blen) -> (ll, grad)` on this rank's sites, summed over the group.

    local: callable(parent, blen) -> (ll, grad) over the local shard (an Engine
    wrapper on a GPU rank); local_ll: optional callable(parent, blen) -> ll."""

    def __init__(self, local: Callable, local_ll: Optional[Callable] = None, group=None):
        import torch.distributed as dist
        self._dist = dist
        self.local = local
        self.local_ll = local_ll
        self.group = group

    def _sum(self, vec: np.ndarray) -> np.ndarray:
        import torch
        t = torch.from_numpy(np.ascontiguousarray(vec, dtype=np.float64))
        if self._dist.get_backend(self.group) == "nccl":
            t = t.cuda()
        self._dist.all_reduce(t, op=self._dist.ReduceOp.SUM, group=self.group)
        return t.cpu().numpy()

    def logfgrad(self, parent, blen):
        ll, g = self.local(parent, blen)
        out = self._sum(np.concatenate([[ll], np.asarray(g, dtype=np.float64)]))
        return float(out[0]), out[1:]

    def logf(self, parent, blen) -> float:
        if self.local_ll is None:
            return self.logfgrad(parent, blen)[0]
        return float(self._sum(np.array([self.local_ll(parent, blen)]))[0])


def engine_shard(parent, blen, codes, leaf_nums, model_out, pi, rates, rank: int, world: int,
                 precision: str = "f32"):
    """An Engine over this rank's block of sites (codes[:, s0:s1]) with the
    (logfgrad, logf) callables ShardedEval expects."""
    from .engine import Engine

    s0, s1 = site_range(codes.shape[1], rank, world)
    U, D, Uinv, mu = model_out
    e = Engine(len(pi), len(rates), precision)
    e.set_tree(parent, blen)
    e.set_codes(np.ascontiguousarray(codes[:, s0:s1]), leaf_nums)
    e.set_model(U, D, Uinv, mu, pi, rates)
    state = {"parent": np.asarray(parent, dtype=np.int64).copy()}

    def sync(p, b):
        if not np.array_equal(p, state["parent"]):
            e.set_tree(p, b)
            state["parent"] = np.asarray(p, dtype=np.int64).copy()
        else:
            e.set_branch_lengths(b)

    def lfg(p, b):
        sync(p, b)
        return e.logpdf_grad()

    def lf(p, b):
        sync(p, b)
        return e.logpdf()

    return e, lfg, lf
