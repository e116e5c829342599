"""mcphy_logpdf_grad_noalloc: the evaluation for callers that cannot allocate
device memory while they run (a sampler loop where cudaMalloc's implicit device
synchronisation or any allocation is not allowed).  It must give the same
results as the regular entry point while taking its scratch from the library's
fixed 64 MiB device array.

This file is collected last on purpose: the entry point shares one fixed device
array across the process, and the test must pass both alone and after every
other test has run in the same process.
"""
import ctypes

import numpy as np
import pytest

from gpu_cases import (F32_G_FLOOR, F32_G_RTOL, F32_LL_RTOL, F64_G_FLOOR, F64_G_RTOL, F64_RTOL,
                       assert_grad_close, random_instance)

pytestmark = pytest.mark.gpu


def _handle(L, _lib, inst, precision):
    h = _lib.handle_t()
    assert L.mcphy_batch_create(inst.K, len(inst.rates), 1, precision, ctypes.byref(h)) == 0
    p = np.ascontiguousarray(inst.parent, dtype=np.int64)
    b = np.ascontiguousarray(inst.blen)
    assert L.mcphy_set_tree(h, len(p), p.ctypes.data_as(_lib.pi64), b.ctypes.data_as(_lib.pdbl)) == 0
    c = np.ascontiguousarray(inst.codes, dtype=np.uint32)
    ln = np.ascontiguousarray(inst.leaf_nums, dtype=np.int64)
    assert L.mcphy_batch_set_codes(h, 0, c.ctypes.data_as(_lib.pu32), c.shape[1],
                                   ln.ctypes.data_as(_lib.pi64), len(ln)) == 0
    U = np.asfortranarray(inst.U)
    Ui = np.asfortranarray(inst.Uinv)
    D = np.ascontiguousarray(inst.D)
    pi = np.ascontiguousarray(inst.pi)
    r = np.ascontiguousarray(inst.rates)
    assert L.mcphy_set_model(h, U.ctypes.data_as(_lib.pdbl), D.ctypes.data_as(_lib.pdbl),
                             Ui.ctypes.data_as(_lib.pdbl), inst.mu, pi.ctypes.data_as(_lib.pdbl),
                             r.ctypes.data_as(_lib.pdbl)) == 0
    return h


def _regular(L, _lib, h, blen, G):
    ll = np.zeros(1)
    g = np.zeros(G)
    assert L.mcphy_set_branch_lengths(h, blen.ctypes.data_as(_lib.pdbl)) == 0
    st = L.mcphy_logpdf_grad(h, ll.ctypes.data_as(_lib.pdbl), g.ctypes.data_as(_lib.pdbl))
    assert st == 0, L.mcphy_last_error(h)
    return ll[0], g


@pytest.mark.parametrize("sweep", [1, 2])      # MCPHY_SWEEP_WALK, MCPHY_SWEEP_LEVEL
@pytest.mark.parametrize("precision", [1, 0])   # MCPHY_PREC_F64, MCPHY_PREC_F32
def test_noalloc_matches_regular_entry_point(built_lib, precision, sweep):
    import torch
    from mcphylo_gb300 import _lib
    L = _lib.load()
    if sweep == 1:
        inst = random_instance(4, 4, 60, 4000, seed=31, multifurcate=0.1)
    else:   # a tree whose items fit one CTA's shared memory
        inst = random_instance(4, 4, 30, 500, seed=32, multifurcate=0.1)
    h = _handle(L, _lib, inst, precision)
    assert L.mcphy_set_sweep(h, sweep) == 0
    try:
        G = inst.N - 1
        rng = np.random.default_rng(5)
        blens = [inst.blen * rng.uniform(0.7, 1.3, size=G) for _ in range(2)]
        # a regular call first: it uploads the tree, data and model (and allocates)
        _regular(L, _lib, h, inst.blen.copy(), G)
        got = ctypes.c_int(0)
        assert L.mcphy_get_sweep(h, ctypes.byref(got)) == 0 and got.value == sweep
        d_ll = torch.zeros(1, dtype=torch.float64, device="cuda")
        d_g = torch.zeros(G, dtype=torch.float64, device="cuda")
        for blen in blens:                       # two allocation-free calls in a row
            d_b = torch.tensor(blen, dtype=torch.float64, device="cuda")
            st = L.mcphy_logpdf_grad_noalloc(h, ctypes.c_void_p(d_b.data_ptr()),
                                             ctypes.c_void_p(d_ll.data_ptr()),
                                             ctypes.c_void_p(d_g.data_ptr()))
            assert st == 0, L.mcphy_last_error(h)
            assert L.mcphy_synchronize(h) == 0
            ll_na = float(d_ll.cpu()[0])
            g_na = d_g.cpu().numpy()
            ll_ref, g_ref = _regular(L, _lib, h, blen, G)
            if precision == 1:
                assert abs(ll_na - ll_ref) <= F64_RTOL * abs(ll_ref)
                assert_grad_close(g_na, g_ref, F64_G_RTOL, F64_G_FLOOR)
            else:
                assert abs(ll_na - ll_ref) <= F32_LL_RTOL * abs(ll_ref)
                assert_grad_close(g_na, g_ref, F32_G_RTOL, F32_G_FLOOR)
    finally:
        L.mcphy_destroy(h)


def test_noalloc_rejects_what_it_cannot_hold(built_lib):
    """A problem whose per-item partial sums exceed the fixed array is refused
    with MCPHY_ERR_ARG (-1) and a message, and a handle whose tree changed since
    the last regular call is refused with MCPHY_ERR_STATE (-6)."""
    import torch
    from mcphylo_gb300 import _lib, simulate
    L = _lib.load()
    rng = np.random.default_rng(2)
    tree = simulate.yule_tree(512, rng, 0.1)
    from mcphylo_gb300.tree import to_parent
    parent, blen = to_parent(tree)
    N, S, C = len(parent), 40_000, 64
    h = _lib.handle_t()
    assert L.mcphy_batch_create(4, C, 1, 0, ctypes.byref(h)) == 0
    try:
        p = np.ascontiguousarray(parent, dtype=np.int64)
        assert L.mcphy_set_tree(h, N, p.ctypes.data_as(_lib.pi64), blen.ctypes.data_as(_lib.pdbl)) == 0
        leaves = np.array(sorted(set(range(1, N + 1)) - set(parent.tolist())), dtype=np.int64)
        codes = np.full((len(leaves), S), 15, dtype=np.uint32)
        assert L.mcphy_batch_set_codes(h, 0, codes.ctypes.data_as(_lib.pu32), S,
                                       leaves.ctypes.data_as(_lib.pi64), len(leaves)) == 0
        from mcphylo_gb300 import models
        pi = np.full(4, 0.25)
        U, D, Ui, mu = models.JC(pi)
        U, Ui, D = np.asfortranarray(U), np.asfortranarray(Ui), np.ascontiguousarray(D)
        rates = np.ones(C)
        assert L.mcphy_set_model(h, U.ctypes.data_as(_lib.pdbl), D.ctypes.data_as(_lib.pdbl),
                                 Ui.ctypes.data_as(_lib.pdbl), mu, pi.ctypes.data_as(_lib.pdbl),
                                 rates.ctypes.data_as(_lib.pdbl)) == 0
        d_b = torch.tensor(blen, dtype=torch.float64, device="cuda")
        d_ll = torch.zeros(1, dtype=torch.float64, device="cuda")
        d_g = torch.zeros(N - 1, dtype=torch.float64, device="cuda")
        args = (ctypes.c_void_p(d_b.data_ptr()), ctypes.c_void_p(d_ll.data_ptr()),
                ctypes.c_void_p(d_g.data_ptr()))
        assert L.mcphy_logpdf_grad_noalloc(h, *args) == -6          # nothing uploaded yet
        ll = np.zeros(1)
        g = np.zeros(N - 1)
        assert L.mcphy_logpdf_grad(h, ll.ctypes.data_as(_lib.pdbl), g.ctypes.data_as(_lib.pdbl)) == 0
        st = L.mcphy_logpdf_grad_noalloc(h, *args)
        assert st == -1
        assert b"allocation-free scratch" in L.mcphy_last_error(h)
    finally:
        L.mcphy_destroy(h)
