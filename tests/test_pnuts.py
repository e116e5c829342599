"""PNUTS host driver: helpers, tree moves, BHV bounds, priors, ESS and the
sampler's leapfrog with refraction, on CPU (the likelihood from the oracle or a
closed-form target)."""
import math

import numpy as np
import pytest

from mcphylo_gb300 import pnuts as P
from mcphylo_gb300.simulate import restriction_small, yule_tree
from mcphylo_gb300.tree import to_parent

# ---------------------------------------------------------------- helpers


def test_molifier_and_scale_fac():
    d = 0.01
    x = np.array([-0.02, 0.0, 0.003, 0.01, 0.5])
    m = P.molifier(x, d)
    np.testing.assert_allclose(m, [(4e-4 + 1e-4) / 0.02, 1e-4 / 0.02, (9e-6 + 1e-4) / 0.02,
                                   0.01, 0.5], rtol=1e-15)
    # continuous at delta, and scale_fac is its derivative
    assert P.molifier(d - 1e-12, d) == pytest.approx(d, abs=1e-11)
    h = 1e-7
    for v in (0.002, 0.007, 0.3):
        fd = (P.molifier(v + h, d) - P.molifier(v - h, d)) / (2 * h)
        assert P.scale_fac(v, d) == pytest.approx(fd, rel=1e-6)


# ((1,2)5,(3,4)6)7 and the NNI across branch 5 that moves leaf 1 to the root
PARENT_A = np.array([5, 5, 6, 6, 7, 7, 0])
PARENT_B = np.array([7, 5, 6, 6, 5, 7, 0])


def test_internal_external():
    np.testing.assert_array_equal(P.internal_external(PARENT_A), [0, 0, 0, 0, 1, 1])
    np.testing.assert_array_equal(P.internal_external(PARENT_B), [0, 0, 0, 0, 1, 1])


def _valid_tree(parent, leaves):
    N = len(parent)
    assert parent[N - 1] == 0 and np.count_nonzero(parent == 0) == 1
    for n in range(1, N + 1):
        seen, m = 0, n
        while parent[m - 1] != 0:
            m = parent[m - 1]
            seen += 1
            assert seen <= N, "cycle"
        assert m == N
    has_child = np.zeros(N, dtype=bool)
    has_child[parent[parent > 0] - 1] = True
    assert set(np.flatnonzero(~has_child) + 1) == leaves


def test_nni_moves():
    rng = np.random.default_rng(3)
    new, made = P.nni(PARENT_A, 5, rng)
    assert made == 1
    # one child of 5 and the sibling 6 traded places
    moved = [i + 1 for i in range(7) if new[i] != PARENT_A[i]]
    assert len(moved) == 2 and 6 in moved
    assert new[5] == 5 and (new[0] == 7 or new[1] == 7)
    # leaves and the root have no NNI
    assert P.nni(PARENT_A, 1, rng)[1] == 0
    assert P.nni(PARENT_A, 7, rng)[1] == 0
    # random walks of NNIs keep a valid tree on the same leaves
    tree = yule_tree(20, np.random.default_rng(1), 0.1)
    parent, _ = to_parent(tree)
    leaves = set(np.flatnonzero(P.internal_external(parent) == 0) + 1)
    p = parent.copy()
    for _ in range(300):
        p, _ = P.nni(p, int(rng.integers(1, len(p))), rng)
        _valid_tree(p, leaves)


def test_bhv_bounds():
    b1 = np.array([1.0, 1.0, 1.0, 1.0, 0.5, 0.3])
    b2 = np.array([1.2, 1.0, 1.0, 1.0, 0.4, 0.3])
    # same topology: the Euclidean distance, both bounds
    lo, up = P.bhv_bounds((PARENT_A, b1), (PARENT_A, b2))
    assert lo == up == pytest.approx(math.sqrt(0.04 + 0.01))
    # {1,2} only in A (0.5), {2,3,4} only in B (0.4), common leaf 1 differs by 0.2
    lo, up = P.bhv_bounds((PARENT_A, b1), (PARENT_B, b2))
    assert lo == pytest.approx(math.sqrt(0.04 + 0.25 + 0.16), rel=1e-14)
    assert up == pytest.approx(math.sqrt(0.04 + 0.9 ** 2), rel=1e-14)
    lo2, up2 = P.bhv_bounds((PARENT_B, b2), (PARENT_A, b1))
    assert (lo2, up2) == pytest.approx((lo, up), rel=1e-15)
    # random NNI neighbours: lower <= upper
    rng = np.random.default_rng(5)
    tree = yule_tree(30, rng, 0.1)
    parent, blen = to_parent(tree)
    for _ in range(30):
        q, _ = P.nni(parent, int(rng.integers(1, len(parent))), rng)
        lo, up = P.bhv_bounds((parent, blen), (q, blen * rng.uniform(0.5, 2, len(blen))))
        assert 0 <= lo <= up + 1e-15


# ---------------------------------------------------------------- priors


def _fd_grad(f, x, h=1e-6):
    g = np.zeros_like(x)
    for i in range(len(x)):
        e = np.zeros_like(x)
        e[i] = h
        g[i] = (f(x + e) - f(x - e)) / (2 * h)
    return g


def test_compound_dirichlet():
    tree = yule_tree(12, np.random.default_rng(2), 0.1)
    parent, blen = to_parent(tree)
    d = P.CompoundDirichlet(1.5, 1.0, 0.1, 2.0)
    v, g = d.logpdf_grad(parent, blen)
    ie = P.internal_external(parent)
    # internal_logpdf (Prior.jl:1-36), term by term
    t_l = blen.sum()
    nterm = float(np.sum(ie == 0))
    n_int = nterm - 3.0
    ref = (1.5 * math.log(0.1) - math.lgamma(1.5) - t_l * 0.1
           - math.lgamma(1.0) - math.lgamma(2.0) + math.lgamma(3.0)
           + np.sum(np.log(blen[ie == 0])) * 0.0 + np.sum(np.log(blen[ie == 1])) * 1.0
           + (1.5 - nterm - 2.0 * n_int) * math.log(t_l))
    assert v == pytest.approx(ref, rel=1e-14)
    fd = _fd_grad(lambda b: d.logpdf_grad(parent, b)[0], blen)
    np.testing.assert_allclose(g, fd, rtol=1e-6, atol=1e-6)


def test_exponential_bl():
    from scipy.stats import expon
    b = np.array([0.1, 0.2, 0.05])
    v, g = P.ExponentialBL(0.1).logpdf_grad(None, b)
    assert v == pytest.approx(np.sum(expon(scale=0.1).logpdf(b)), rel=1e-14)
    np.testing.assert_allclose(g, -10.0)


# ---------------------------------------------------------------- ESS


def test_ess_batch_means():
    x = np.arange(400, dtype=float)
    # batch means 49.5 .. 349.5: var 50000/3, MCSE^2 = var/4; sample var(x) = 400*401/12
    assert P.mcse_bm(x) == pytest.approx(math.sqrt(50000 / 3 / 4), rel=1e-14)
    assert P.ess(x) == pytest.approx((400 * 401 / 12) / (50000 / 12), rel=1e-13)
    iid = np.random.default_rng(0).standard_normal(2000)
    assert P.ess(iid) <= 2000
    assert P.ess(iid) > 800
    with pytest.raises(ValueError):
        P.mcse_bm(np.zeros(150))


# ---------------------------------------------------------------- leapfrog with refraction

SHAPE, SCALE = 20.0, 0.05


def _gamma_target(p, b):
    b = np.asarray(b)
    return float(np.sum((SHAPE - 1) * np.log(b) - b / SCALE)), (SHAPE - 1) / b - 1 / SCALE


def _flat(p, b):
    return 0.0, np.zeros(len(b))


def _sampler(parent, blen, fg, seed=0):
    return P.PNUTS(parent, blen, fg, lambda p, b: fg(p, b)[0], rng=np.random.default_rng(seed))


def test_refraction_reversible_and_energy():
    tree = yule_tree(10, np.random.default_rng(4), 0.1)
    parent, _ = to_parent(tree)
    rng = np.random.default_rng(7)
    blen = rng.uniform(0.8, 1.2, len(parent) - 1)
    s = _sampler(parent, blen, _gamma_target)
    lf, g = _gamma_target(parent, blen)
    st = P.TreeState(parent.copy(), blen.copy(), rng.standard_normal(len(blen)), g, lf)
    h0 = st.hamiltonian()
    eps = 1e-3
    x = st.copy()
    for _ in range(10):
        s.refraction(x, eps, 1e-9)
    assert abs(x.hamiltonian() - h0) < 1e-4
    x.r = -x.r
    for _ in range(10):
        s.refraction(x, eps, 1e-9)
    np.testing.assert_allclose(x.blen, st.blen, rtol=0, atol=1e-12)
    np.testing.assert_allclose(-x.r, st.r, rtol=0, atol=1e-10)


def test_refraction_reflects_leaf_branch():
    s = _sampler(PARENT_A, np.full(6, 0.5), _flat)
    r = np.zeros(6)
    r[0] = -1.0
    st = P.TreeState(PARENT_A.copy(), np.array([0.001, 0.5, 0.5, 0.5, 0.5, 0.5]), r,
                     np.zeros(6), 0.0)
    nni_n, att = s.refraction(st, 0.01, 1e-9)
    assert (nni_n, att) == (0, 0)
    assert st.blen[0] == pytest.approx(0.009, rel=1e-12)
    assert st.r[0] == 1.0
    np.testing.assert_array_equal(st.parent, PARENT_A)


def test_refraction_nni_across_internal_branch():
    # a flat density makes every NNI free: the momentum keeps its size
    s = _sampler(PARENT_A, np.full(6, 0.5), _flat)
    r = np.zeros(6)
    r[4] = -1.0
    st = P.TreeState(PARENT_A.copy(), np.array([0.5, 0.5, 0.5, 0.5, 0.001, 0.5]), r,
                     np.zeros(6), 0.0)
    nni_n, att = s.refraction(st, 0.01, 1e-9)
    assert (nni_n, att) == (1, 1)
    assert st.r[4] == pytest.approx(1.0)
    assert st.blen[4] == pytest.approx(0.009, rel=1e-12)
    assert not np.array_equal(st.parent, PARENT_A)
    assert s.n_logf_evals == 2


def test_sampler_on_closed_form_target():
    """Gamma(20, 0.05) branch lengths (mean 1): far from zero the molifier and
    reflections are idle; the draws' mean matches within a few percent."""
    tree = yule_tree(8, np.random.default_rng(0), 0.1)
    parent, blen = to_parent(tree)
    ch = P.run_chain(parent, np.full(len(blen), 1.0), _gamma_target,
                     lambda p, b: _gamma_target(p, b)[0], n_iter=1500, n_adapt=300, seed=3,
                     target=0.8)
    assert abs(ch.blen.mean() - SHAPE * SCALE) < 0.03
    assert 0.05 < ch.epsilon < 1.0
    assert np.all(ch.depth >= 1)
    e = ch.ess()
    assert e["tree_length"] > 50


def test_dual_averaging_moves_step_size():
    tree = yule_tree(8, np.random.default_rng(0), 0.1)
    parent, blen = to_parent(tree)
    s = P.PNUTS(parent, np.full(len(blen), 1.0), _gamma_target,
                lambda p, b: _gamma_target(p, b)[0], rng=np.random.default_rng(1), target=0.8)
    s.sample(True)
    assert s.m == 1 and s.mu_p == pytest.approx(math.log(10 * s.delta / 2))
    for _ in range(50):
        s.sample(True)
    x_bar = s.x_bar
    s.sample(False)
    assert s.epsilon == pytest.approx(math.exp(x_bar))
    assert s.delta == pytest.approx(2 * s.epsilon)


# ---------------------------------------------------------------- posterior wrapper


class _FakeEngine:
    """Records the calls a TreePosterior makes: topology updates and evaluations
    (each bound evaluation sends its branch lengths)."""

    def __init__(self, tag, log):
        self.tag, self.log = tag, log

    def set_tree(self, parent, blen=None):
        self.log.append((self.tag, "tree", tuple(parent)))

    def bind(self):
        def grad_fn(blen):
            self.log.append((self.tag, "blen"))
            return -1.0, np.zeros(6)

        def logf_fn(blen):
            self.log.append((self.tag, "blen"))
            return -1.0

        return grad_fn, logf_fn


def test_tree_posterior_routes_proposals():
    log = []
    a, b =_FakeEngine("a", log), _FakeEngine("b", log)
    post = P.TreePosterior(a, PARENT_A, np.ones(6), P.ExponentialBL(1.0), proposal_engine=b)
    assert log == [("a", "tree", tuple(PARENT_A))]
    log.clear()
    post.logfgrad(PARENT_A, np.ones(6))
    post.logf(PARENT_B, np.ones(6))            # proposal goes to b
    post.logf(PARENT_A, np.ones(6))            # rejected: a still holds A
    assert log == [("a", "blen"), ("b", "tree", tuple(PARENT_B)), ("b", "blen"), ("a", "blen")]
    log.clear()
    post.logf(PARENT_B, np.ones(6))            # proposed again: b already holds B
    post.logfgrad(PARENT_B, np.ones(6))        # accepted: the engines trade places
    assert log == [("b", "blen"), ("b", "blen")]
    assert post.eng is b and post.prop is a
    v, g = post.logfgrad(PARENT_B, np.full(6, 2.0))
    assert v == pytest.approx(-1.0 - 12.0)
    np.testing.assert_allclose(g, -1.0)


# ---------------------------------------------------------------- with the oracle


def test_chain_with_oracle_likelihood():
    from oracle import pyoracle as O
    inst = restriction_small(S=200, taxa=12)
    x = np.asfortranarray(inst.tensor())
    model = (inst.U, inst.D, inst.Uinv, inst.mu)
    prior = P.CompoundDirichlet(1.0, 1.0, 0.1, 1.0)

    def lfg(p, b):
        ll, g = O.gradlogpdf(O.tree_from_parent(p, b), x, inst.pi, model, inst.rates)
        lp, gp = prior.logpdf_grad(p, b)
        return ll + lp, g + gp

    def lf(p, b):
        return lfg(p, b)[0]

    ch = P.run_chain(inst.parent, inst.blen, lfg, lf, n_iter=15, n_adapt=10, seed=2, target=0.8)
    assert np.all(np.isfinite(ch.logf)) and np.all(ch.blen > 0)
    assert ch.grad_evals >= 15


def test_checkpoint_resume_continues_the_chain():
    """state() / from_state(): a restored sampler draws exactly what the original
    would have drawn (tree, step size, adapter and random stream)."""
    import pickle
    tree = yule_tree(8, np.random.default_rng(0), 0.1)
    parent, blen = to_parent(tree)
    lf = lambda p, b: _gamma_target(p, b)[0]
    a = P.PNUTS(parent, np.full(len(blen), 1.0), _gamma_target, lf,
                rng=np.random.default_rng(11), target=0.8)
    for it in range(15):
        a.sample(it < 10)
    saved = pickle.loads(pickle.dumps(a.state()))
    for _ in range(6):
        a.sample(False)
    b = P.PNUTS.from_state(saved, _gamma_target, lf)
    for _ in range(6):
        b.sample(False)
    np.testing.assert_array_equal(a.parent, b.parent)
    np.testing.assert_array_equal(a.blen, b.blen)
    assert a.epsilon == b.epsilon and a.tree_depth_trace == b.tree_depth_trace
    assert a.n_grad_evals == b.n_grad_evals


def test_plus_end_forward_variant():
    """The non-parity variant (plus end starts with direction +1) still samples the
    target; the default keeps the reference's -1 for both ends, so the two chains
    differ from the first trajectory on."""
    tree = yule_tree(8, np.random.default_rng(0), 0.1)
    parent, blen = to_parent(tree)
    runs = {}
    for fwd in (False, True):
        runs[fwd] = P.run_chain(parent, np.full(len(blen), 1.0), _gamma_target,
                                lambda p, b: _gamma_target(p, b)[0], n_iter=1500, n_adapt=300,
                                seed=3, target=0.8, plus_end_forward=fwd)
    assert abs(runs[True].blen.mean() - SHAPE * SCALE) < 0.03
    assert not np.array_equal(runs[True].blen, runs[False].blen)
    s = _sampler(parent, blen, _gamma_target)
    assert s.plus_end_forward is False
    assert P.PNUTS.from_state(s.state(), _gamma_target, _flat).plus_end_forward is False
