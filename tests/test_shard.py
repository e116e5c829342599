"""Site-sharded evaluation over a world_size-2 gloo group on CPU: each rank
evaluates its block of sites (with the oracle standing in for the rank's engine),
one all-reduce completes logL and the gradient, and a PNUTS chain driven through
the sharded evaluation makes the same decisions on both ranks as a single-process
chain."""
import os
import socket

import numpy as np
import pytest

from mcphylo_gb300 import shard
from mcphylo_gb300.simulate import restriction_small


def test_site_range_partitions():
    for S in (1, 7, 1000, 1001):
        for W in (1, 2, 3, 8):
            if W > S:
                continue
            rs = [shard.site_range(S, r, W) for r in range(W)]
            assert rs[0][0] == 0 and rs[-1][1] == S
            assert all(a[1] == b[0] for a, b in zip(rs, rs[1:]))
            sizes = [b - a for a, b in rs]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard.site_range(10, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _oracle_local(inst, rank, world):
    from oracle import pyoracle as O
    s0, s1 = shard.site_range(inst.S, rank, world)
    x = np.asfortranarray(inst.tensor()[:, s0:s1, :])
    model = (inst.U, inst.D, inst.Uinv, inst.mu)

    def lfg(p, b):
        return O.gradlogpdf(O.tree_from_parent(p, b), x, inst.pi, model, inst.rates)

    def lf(p, b):
        return O.logpdf(O.tree_from_parent(p, b), x, inst.pi, model, inst.rates)

    return lfg, lf


def _worker(rank, world, port, out_dir):
    import torch.distributed as dist
    from mcphylo_gb300 import pnuts as P
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        inst = restriction_small(seed=21, S=301, taxa=14)
        lfg, lf = _oracle_local(inst, rank, world)
        ev = shard.ShardedEval(lfg, lf)
        rng = np.random.default_rng(3)
        b = inst.blen * rng.uniform(0.5, 1.5, len(inst.blen))
        ll, g = ev.logfgrad(inst.parent, b)
        llf = ev.logf(inst.parent, b)
        s = P.PNUTS(inst.parent, inst.blen, ev.logfgrad, ev.logf,
                    rng=np.random.default_rng(5), target=0.8)
        for it in range(6):
            s.sample(it < 3)
        np.savez(os.path.join(out_dir, f"rank{rank}.npz"), ll=ll, g=g, llf=llf, b=b,
                 parent=s.parent, blen=s.blen, depth=np.array(s.tree_depth_trace))
    finally:
        dist.destroy_process_group()


def test_sharded_eval_gloo_world2(tmp_path):
    import torch.multiprocessing as mp
    from oracle import pyoracle as O
    from mcphylo_gb300 import pnuts as P
    O.lib()
    mp.spawn(_worker, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    r0 = np.load(tmp_path / "rank0.npz")
    r1 = np.load(tmp_path / "rank1.npz")
    inst = restriction_small(seed=21, S=301, taxa=14)
    lfg, lf = _oracle_local(inst, 0, 1)
    llo, go = lfg(inst.parent, r0["b"])
    for r in (r0, r1):
        assert float(r["ll"]) == pytest.approx(llo, rel=1e-13)
        assert float(r["llf"]) == pytest.approx(llo, rel=1e-13)
        np.testing.assert_allclose(r["g"], go, rtol=1e-11, atol=1e-11 * np.abs(go).max())
    # both ranks hold the same chain, and it is the single-process chain
    np.testing.assert_array_equal(r0["parent"], r1["parent"])
    np.testing.assert_array_equal(r0["blen"], r1["blen"])
    s = P.PNUTS(inst.parent, inst.blen, lfg, lf, rng=np.random.default_rng(5), target=0.8)
    for it in range(6):
        s.sample(it < 3)
    np.testing.assert_array_equal(s.parent, r0["parent"])
    np.testing.assert_allclose(s.blen, r0["blen"], rtol=1e-9)
    assert list(r0["depth"]) == s.tree_depth_trace
