"""The tensor-core building block of the dense-state path: a 128 x N x KD TF32
product through the library's operand tiles, smem descriptors and TMEM loads,
against the host product."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _tc(kd, n, a, b, bf16=0):
    from mcphylo_gb300 import _lib
    L = _lib.load()
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = np.ascontiguousarray(b, dtype=np.float32)
    d = np.zeros((128, n), dtype=np.float32)
    fp = ctypes.POINTER(ctypes.c_float)
    st = L.mcphy_tc_selftest(kd, n, bf16, a.ctypes.data_as(fp), b.ctypes.data_as(fp),
                             d.ctypes.data_as(fp))
    assert st == 0, st
    return d


def _tf32(x):
    """Round FP32 to TF32 (10 explicit mantissa bits), nearest."""
    u = np.asarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x1000) & 0xFFFFE000
    return u.astype(np.uint32).view(np.float32)


@pytest.mark.parametrize("kd,n", [(8, 16), (16, 32), (24, 32), (32, 32), (32, 64)])
def test_exact_small_integers(built_lib, kd, n):
    """Small integers are exact in TF32 and their sums exact in FP32: the product
    must match bit for bit, which pins the operand and accumulator layouts."""
    rng = np.random.default_rng(kd * 100 + n)
    a = rng.integers(-3, 4, size=(128, kd)).astype(np.float32)
    b = rng.integers(-3, 4, size=(n, kd)).astype(np.float32)
    d = _tc(kd, n, a, b)
    np.testing.assert_array_equal(d, a.astype(np.float64) @ b.astype(np.float64).T)


@pytest.mark.parametrize("kd,n", [(16, 16), (32, 32), (48, 32), (64, 64)])
def test_exact_small_integers_bf16(built_lib, kd, n):
    rng = np.random.default_rng(kd * 10 + n)
    a = rng.integers(-3, 4, size=(128, kd)).astype(np.float32)
    b = rng.integers(-3, 4, size=(n, kd)).astype(np.float32)
    d = _tc(kd, n, a, b, bf16=1)
    np.testing.assert_array_equal(d, a.astype(np.float64) @ b.astype(np.float64).T)


def test_random_tf32_accuracy(built_lib):
    rng = np.random.default_rng(1)
    kd, n = 24, 32
    a = rng.random((128, kd)).astype(np.float32)
    b = rng.random((n, kd)).astype(np.float32)
    d = _tc(kd, n, a, b)
    want = _tf32(a).astype(np.float64) @ _tf32(b).astype(np.float64).T
    # inputs used at TF32 (rounded or truncated by the hardware), FP32 accumulation
    np.testing.assert_allclose(d, want, rtol=2e-3)
    exact = a.astype(np.float64) @ b.astype(np.float64).T
    assert np.max(np.abs(d - exact) / exact) < 2e-3


# ---------------------------------------------------------------- the TF32 likelihood path
from gpu_cases import caterpillar, oracle, random_instance  # noqa: E402

# TF32 keeps 10 mantissa bits of each operand: a relative error of up to 2^-11 per
# rounded operand and node, which accumulates with tree depth (measured: 4e-5 to
# 1.5e-4 on total logL, the larger on a 60-deep caterpillar; gradient entries within
# 5e-4 of max|g|).  Stated tolerances of the tensor-core path against the FP64
# oracle: total logL 5e-4 relative, gradient 5e-3 of max|g|.
TF32_LL_RTOL = 5e-4
TF32_G_RTOL = 5e-3


def _tf32_engine(inst, precision="tf32"):
    import mcphylo_gb300 as mp
    e = mp.Engine(inst.K, len(inst.rates), precision)
    e.set_tree(inst.parent, inst.blen)
    e.set_codes(inst.codes, inst.leaf_nums)
    e.set_model(inst.U, inst.D, inst.Uinv, inst.mu, inst.pi, inst.rates)
    return e


def _check(inst, e=None):
    llo, go = oracle(inst)
    e = e or _tf32_engine(inst)
    ll, g = e.logpdf_grad()
    rel = abs(ll - llo) / abs(llo)
    gerr = np.max(np.abs(g - go)) / np.max(np.abs(go))
    print(f"K={inst.K} N={inst.N} S={inst.S}: logL rel {rel:.2e}, grad {gerr:.2e}")
    assert rel <= TF32_LL_RTOL, (ll, llo)
    assert gerr <= TF32_G_RTOL
    assert e.logpdf() == pytest.approx(ll, rel=1e-12)
    return ll, g


@pytest.mark.parametrize("K,C,taxa,S,mf", [(20, 4, 24, 300, 0.0), (20, 1, 40, 128, 0.3),
                                         (9, 2, 17, 77, 0.0), (12, 3, 30, 257, 0.2),
                                         (32, 2, 12, 140, 0.0), (25, 1, 9, 33, 0.0)])
def test_tf32_vs_oracle(built_lib, K, C, taxa, S, mf):
    inst = random_instance(K, C, taxa, S, seed=K * 7 + taxa, multifurcate=mf)
    _check(inst)


def test_tf32_deep_caterpillar(built_lib):
    rng = np.random.default_rng(3)
    inst = random_instance(20, 2, 0, 200, seed=3, tree=caterpillar(60, rng))
    _check(inst)


def test_tf32_partially_ambiguous_codes(built_lib):
    inst = random_instance(20, 2, 20, 150, seed=9)
    rng = np.random.default_rng(4)
    codes = inst.codes.copy()
    mask = rng.random(codes.shape) < 0.1
    codes[mask] |= np.uint32(1) << rng.integers(0, 20, size=mask.sum()).astype(np.uint32)
    inst.codes = codes
    _check(inst)


def test_tf32_topology_change_and_graph(built_lib):
    from mcphylo_gb300 import simulate, tree as T
    inst = random_instance(20, 4, 30, 300, seed=12)
    e = _tf32_engine(inst)
    e.enable_graph(True)
    _check(inst, e)
    ll_a, g_a = e.logpdf_grad()
    ll_b, g_b = e.logpdf_grad()
    assert ll_a == ll_b and np.array_equal(g_a, g_b)
    # an NNI on the live engine
    p = inst.parent.copy()
    rng = np.random.default_rng(2)
    while True:
        t = int(rng.integers(1, len(p)))
        kids = np.flatnonzero(p == t) + 1
        sibs = [s for s in np.flatnonzero(p == p[t - 1]) + 1 if s != t]
        if len(kids) and p[t - 1] and sibs:
            c, s = int(kids[0]), int(sibs[0])
            p[c - 1], p[s - 1] = p[t - 1], t
            break
    e.set_tree(p, inst.blen)
    inst2 = simulate.Instance(T.from_parent(p, inst.blen), p, inst.blen, inst.leaf_nums,
                              inst.codes, inst.U, inst.D, inst.Uinv, inst.mu, inst.pi, inst.rates)
    _check(inst2, e)


def test_tf32_timeout_is_reported(built_lib):
    import mcphylo_gb300 as mp
    inst = random_instance(20, 2, 20, 200, seed=5)
    e = _tf32_engine(inst)
    ll0, g0 = e.logpdf_grad()
    e.debug_inject(1)
    with pytest.raises(mp.MCPhyError) as ei:
        e.logpdf_grad()
    assert ei.value.status == -7
    ll1, g1 = e.logpdf_grad()
    assert ll1 == ll0 and np.array_equal(g1, g0)


def test_tf32_batched(built_lib):
    import mcphylo_gb300 as mp
    insts = [random_instance(20, 4, t, s, seed=60 + t) for t, s in ((8, 50), (35, 400), (17, 129))]
    e = mp.Engine(20, 4, "tf32", n_instances=3)
    for i, b in enumerate(insts):
        e.set_tree(b.parent, b.blen, i)
        e.set_codes(b.codes, b.leaf_nums, i)
        e.set_model(b.U, b.D, b.Uinv, b.mu, b.pi, b.rates, i)
    ll, g = e.logpdf_grad()
    off = e.grad_offsets()
    for i, b in enumerate(insts):
        llo, go = oracle(b)
        assert abs(ll[i] - llo) <= TF32_LL_RTOL * abs(llo)
        assert np.max(np.abs(g[off[i]:off[i + 1]] - go)) <= TF32_G_RTOL * np.max(np.abs(go))


def test_tf32_rejects_small_state_spaces(built_lib):
    import mcphylo_gb300 as mp
    with pytest.raises(Exception):
        mp.Engine(4, 4, "tf32")


# BF16 keeps 8 significant bits: a relative error of up to 2^-9 per rounded operand
# and node.  Stated tolerances of the BF16 tensor-core path against the FP64 oracle
# (measured values in the test output): total logL 5e-3 relative, gradient 5e-2 of
# max|g|.
BF16_LL_RTOL = 5e-3
BF16_G_RTOL = 5e-2


@pytest.mark.parametrize("K,C,taxa,S,mf", [(20, 4, 24, 300, 0.0), (12, 2, 30, 200, 0.2),
                                         (32, 1, 10, 70, 0.0)])
def test_bf16_vs_oracle(built_lib, K, C, taxa, S, mf):
    inst = random_instance(K, C, taxa, S, seed=K * 11 + taxa, multifurcate=mf)
    llo, go = oracle(inst)
    e = _tf32_engine(inst, "bf16")
    ll, g = e.logpdf_grad()
    rel = abs(ll - llo) / abs(llo)
    gerr = np.max(np.abs(g - go)) / np.max(np.abs(go))
    print(f"bf16 K={K} N={inst.N} S={S}: logL rel {rel:.2e}, grad {gerr:.2e}")
    assert rel <= BF16_LL_RTOL
    assert gerr <= BF16_G_RTOL
    assert e.logpdf() == pytest.approx(ll, rel=1e-12)


# ---------------------------------------------------------------- split TF32 (3xTF32)
# Every operand is a TF32 value plus a TF32 residual and each product is three MMAs
# (lo*hi + hi*lo + hi*hi), about 21 bits per operand: held to the FP32 path's own
# tolerances against the FP64 oracle (logL 1e-6 relative; gradient entries 1e-4
# relative to max(|g_i|, 1e-2 max|g|)).
@pytest.mark.parametrize("K,C,taxa,S,mf", [(20, 4, 24, 300, 0.0), (20, 1, 40, 128, 0.3),
                                         (9, 2, 17, 77, 0.0), (12, 3, 30, 257, 0.2),
                                         (24, 2, 12, 140, 0.0)])
def test_tf32x3_vs_oracle(built_lib, K, C, taxa, S, mf):
    from gpu_cases import F32_G_FLOOR, F32_G_RTOL, F32_LL_RTOL, assert_grad_close
    inst = random_instance(K, C, taxa, S, seed=K * 13 + taxa, multifurcate=mf)
    llo, go = oracle(inst)
    e = _tf32_engine(inst, "tf32x3")
    ll, g = e.logpdf_grad()
    rel = abs(ll - llo) / abs(llo)
    gerr = assert_grad_close(g, go, F32_G_RTOL, F32_G_FLOOR)
    print(f"tf32x3 K={K} N={inst.N} S={S}: logL rel {rel:.2e}, grad {gerr:.2e}")
    assert rel <= F32_LL_RTOL, (ll, llo)
    assert e.logpdf() == pytest.approx(ll, rel=1e-12)


def test_tf32x3_deep_caterpillar(built_lib):
    from gpu_cases import F32_G_FLOOR, F32_G_RTOL, F32_LL_RTOL, assert_grad_close
    rng = np.random.default_rng(3)
    inst = random_instance(20, 2, 0, 200, seed=3, tree=caterpillar(60, rng))
    llo, go = oracle(inst)
    ll, g = _tf32_engine(inst, "tf32x3").logpdf_grad()
    assert abs(ll - llo) <= F32_LL_RTOL * abs(llo), (ll, llo)
    assert_grad_close(g, go, F32_G_RTOL, F32_G_FLOOR)


def test_tf32x3_rejects_unsupported_state_spaces(built_lib):
    import mcphylo_gb300 as mp
    for K in (4, 25, 32):
        with pytest.raises(Exception):
            mp.Engine(K, 2, "tf32x3")
