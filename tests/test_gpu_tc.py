"""The tensor-core building block of the dense-state path: a 128 x N x KD TF32
product through the library's operand tiles, smem descriptors and TMEM loads,
against the host product."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _tc(kd, n, a, b):
    from mcphylo_gb300 import _lib
    L = _lib.load()
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = np.ascontiguousarray(b, dtype=np.float32)
    d = np.zeros((128, n), dtype=np.float32)
    fp = ctypes.POINTER(ctypes.c_float)
    st = L.mcphy_tc_selftest(kd, n, a.ctypes.data_as(fp), b.ctypes.data_as(fp),
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
