"""PNUTS driven by the engine: the log posterior the sampler sees matches the
oracle's across NNI moves, and a chain run on the FP64 engine retraces the chain
run on the oracle with the same random numbers."""
import numpy as np
import pytest

from oracle import pyoracle as O

from mcphylo_gb300 import pnuts as P
from mcphylo_gb300.simulate import restriction_small

pytestmark = pytest.mark.gpu

PRIOR = P.CompoundDirichlet(1.0, 1.0, 0.1, 1.0)


def _oracle_posterior(inst):
    x = np.asfortranarray(inst.tensor())
    model = (inst.U, inst.D, inst.Uinv, inst.mu)

    def lfg(p, b):
        ll, g = O.gradlogpdf(O.tree_from_parent(p, b), x, inst.pi, model, inst.rates)
        lp, gp = PRIOR.logpdf_grad(p, b)
        return ll + lp, g + gp

    def lf(p, b):
        ll = O.logpdf(O.tree_from_parent(p, b), x, inst.pi, model, inst.rates)
        return ll + PRIOR.logpdf_grad(p, b)[0]

    return lfg, lf


def _engine_posterior(inst, precision):
    return P.engine_posterior(inst.parent, inst.blen, inst.codes, inst.leaf_nums,
                              (inst.U, inst.D, inst.Uinv, inst.mu), inst.pi, inst.rates,
                              PRIOR, precision=precision)


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_posterior_matches_oracle_across_nni(built_lib, precision):
    inst = restriction_small(seed=11, S=600, taxa=24)
    post = _engine_posterior(inst, precision)
    lfg, lf = _oracle_posterior(inst)
    rng = np.random.default_rng(0)
    parent = inst.parent.copy()
    rtol = 1e-12 if precision == "f64" else 1e-6
    for step in range(12):
        blen = inst.blen * rng.uniform(0.5, 1.5, len(inst.blen))
        if step % 3 == 1:
            # an NNI proposal that is evaluated, then kept or dropped
            q, made = P.nni(parent, int(rng.integers(1, len(parent))), rng)
            assert post.logf(q, blen) == pytest.approx(lf(q, blen), rel=rtol)
            if rng.random() < 0.5:
                parent = q
        v, g = post.logfgrad(parent, blen)
        rv, rg = lfg(parent, blen)
        assert v == pytest.approx(rv, rel=rtol)
        gtol = 1e-10 if precision == "f64" else 1e-4
        assert np.linalg.norm(g - rg) <= gtol * max(np.linalg.norm(rg), 1.0)
        assert post.logf(parent, blen) == pytest.approx(rv, rel=rtol)


def test_fp64_chain_retraces_oracle_chain(built_lib):
    """Same seed, same decisions: the FP64 engine and the oracle agree to ~1e-12,
    so every accept/reject and NNI choice of a short chain comes out the same."""
    inst = restriction_small(seed=12, S=400, taxa=16)
    post = _engine_posterior(inst, "f64")
    lfg, lf = _oracle_posterior(inst)
    a = P.PNUTS(inst.parent, inst.blen, post.logfgrad, post.logf,
                rng=np.random.default_rng(9), target=0.8)
    b = P.PNUTS(inst.parent, inst.blen, lfg, lf, rng=np.random.default_rng(9), target=0.8)
    for it in range(12):
        a.sample(it < 6)
        b.sample(it < 6)
        np.testing.assert_array_equal(a.parent, b.parent)
        np.testing.assert_allclose(a.blen, b.blen, rtol=1e-8)
        assert a.epsilon == pytest.approx(b.epsilon, rel=1e-8)
    assert a.tree_depth_trace == b.tree_depth_trace
    assert a.n_grad_evals == b.n_grad_evals


def test_fp32_chain(built_lib):
    inst = restriction_small(seed=13, S=1000, taxa=32)
    post = _engine_posterior(inst, "f32")
    ch = P.run_chain(inst.parent, inst.blen, post.logfgrad, post.logf, n_iter=30, n_adapt=20,
                     seed=4, target=0.8)
    assert np.all(np.isfinite(ch.logf)) and np.all(ch.blen > 0)
    # the log posterior of the last draw, re-evaluated by the oracle
    lfg, lf = _oracle_posterior(inst)
    post64 = _engine_posterior(inst, "f64")
    s = P.PNUTS(inst.parent, inst.blen, post.logfgrad, post.logf,
                rng=np.random.default_rng(4), target=0.8)
    for it in range(8):
        s.sample(True)
        ref = lf(s.parent, s.blen)
        assert post64.logf(s.parent, s.blen) == pytest.approx(ref, rel=1e-12)
        assert post.logf(s.parent, s.blen) == pytest.approx(ref, rel=1e-6)


def test_engine_shards_sum_to_whole(built_lib):
    """Site shards on separate engines add up to the whole alignment (what the
    all-reduce of a site-sharded evaluation relies on)."""
    from mcphylo_gb300 import shard
    inst = restriction_small(seed=14, S=1001, taxa=20)
    model = (inst.U, inst.D, inst.Uinv, inst.mu)
    whole, lfg, _ = shard.engine_shard(inst.parent, inst.blen, inst.codes, inst.leaf_nums, model,
                                       inst.pi, inst.rates, 0, 1, precision="f64")
    ll, g = lfg(inst.parent, inst.blen)
    parts = [shard.engine_shard(inst.parent, inst.blen, inst.codes, inst.leaf_nums, model,
                                inst.pi, inst.rates, r, 3, precision="f64") for r in range(3)]
    res = [p[1](inst.parent, inst.blen) for p in parts]
    assert sum(r[0] for r in res) == pytest.approx(ll, rel=1e-13)
    np.testing.assert_allclose(sum(r[1] for r in res), g, rtol=1e-11, atol=1e-11 * np.abs(g).max())
