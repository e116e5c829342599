"""mcphy_logpdf_grad_noalloc: the evaluation for callers that cannot allocate
device memory while they run (a sampler loop where cudaMalloc's implicit device
synchronisation or any allocation is not allowed).  It runs the same kernels and
the same fixed-order reduction as the regular entry point, taking its scratch from
the library's fixed 64 MiB device array, so its results must equal the regular
entry point's bit for bit -- also when the array holds fewer resident blocks than
the regular launch uses.

This file is collected last on purpose: the entry point shares one fixed device
array across the process, and the tests must pass both alone and after every other
test has run in the same process.
"""
import ctypes

import numpy as np
import pytest

from gpu_cases import random_instance

pytestmark = pytest.mark.gpu

NOALLOC_BYTES = 64 << 20


def _handle(L, _lib, insts, precision):
    """A handle over the instances (one PhyloDist each), through the C ABI."""
    h = _lib.handle_t()
    assert L.mcphy_batch_create(insts[0].K, len(insts[0].rates), len(insts), precision,
                                ctypes.byref(h)) == 0
    for i, inst in enumerate(insts):
        p = np.ascontiguousarray(inst.parent, dtype=np.int64)
        b = np.ascontiguousarray(inst.blen)
        assert L.mcphy_batch_set_tree(h, i, len(p), p.ctypes.data_as(_lib.pi64),
                                      b.ctypes.data_as(_lib.pdbl)) == 0
        c = np.ascontiguousarray(inst.codes, dtype=np.uint32)
        ln = np.ascontiguousarray(inst.leaf_nums, dtype=np.int64)
        assert L.mcphy_batch_set_codes(h, i, c.ctypes.data_as(_lib.pu32), c.shape[1],
                                       ln.ctypes.data_as(_lib.pi64), len(ln)) == 0
        U = np.asfortranarray(inst.U)
        Ui = np.asfortranarray(inst.Uinv)
        D = np.ascontiguousarray(inst.D)
        pi = np.ascontiguousarray(inst.pi)
        r = np.ascontiguousarray(inst.rates)
        assert L.mcphy_batch_set_model(h, i, U.ctypes.data_as(_lib.pdbl), D.ctypes.data_as(_lib.pdbl),
                                       Ui.ctypes.data_as(_lib.pdbl), inst.mu,
                                       pi.ctypes.data_as(_lib.pdbl), r.ctypes.data_as(_lib.pdbl)) == 0
    return h


def _regular(L, _lib, h, blen, M, G):
    """The regular (allocating) entry point for packed branch lengths."""
    ll = np.zeros(M)
    g = np.zeros(G)
    assert L.mcphy_batch_set_all_branch_lengths(h, blen.ctypes.data_as(_lib.pdbl)) == 0
    st = L.mcphy_batch_logpdf_grad(h, ll.ctypes.data_as(_lib.pdbl), g.ctypes.data_as(_lib.pdbl))
    assert st == 0, L.mcphy_last_error(h)
    return ll, g


def _noalloc(L, h, torch, blen, M, G):
    d_b = torch.tensor(blen, dtype=torch.float64, device="cuda")
    d_ll = torch.full((M,), -1.0, dtype=torch.float64, device="cuda")
    d_g = torch.full((G,), -1.0, dtype=torch.float64, device="cuda")
    st = L.mcphy_logpdf_grad_noalloc(h, ctypes.c_void_p(d_b.data_ptr()),
                                     ctypes.c_void_p(d_ll.data_ptr()),
                                     ctypes.c_void_p(d_g.data_ptr()))
    assert st == 0, L.mcphy_last_error(h)
    assert L.mcphy_synchronize(h) == 0
    return d_ll.cpu().numpy(), d_g.cpu().numpy()


def _compare_two_calls(L, _lib, h, insts, torch):
    """Two allocation-free calls in a row, each against the regular entry point on
    the same branch lengths: identical bits."""
    M = len(insts)
    blen0 = np.concatenate([inst.blen for inst in insts])
    G = len(blen0)
    rng = np.random.default_rng(5)
    # a regular call first: it uploads the trees, data and models (and allocates)
    _regular(L, _lib, h, blen0.copy(), M, G)
    for _ in range(2):
        blen = blen0 * rng.uniform(0.7, 1.3, size=G)
        ll_na, g_na = _noalloc(L, h, torch, blen, M, G)
        ll_ref, g_ref = _regular(L, _lib, h, blen, M, G)
        assert np.all(np.isfinite(ll_na)) and np.all(np.isfinite(g_na))
        assert np.array_equal(ll_na, ll_ref), (ll_na, ll_ref)
        assert np.array_equal(g_na, g_ref), float(np.max(np.abs(g_na - g_ref)))


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
    h = _handle(L, _lib, [inst], precision)
    assert L.mcphy_set_sweep(h, sweep) == 0
    try:
        _compare_two_calls(L, _lib, h, [inst], torch)
        got = ctypes.c_int(0)
        assert L.mcphy_get_sweep(h, ctypes.byref(got)) == 0 and got.value == sweep
    finally:
        L.mcphy_destroy(h)


@pytest.mark.parametrize("precision", [1, 0])   # MCPHY_PREC_F64, MCPHY_PREC_F32
def test_noalloc_batch_with_fewer_resident_blocks(built_lib, precision):
    """Three instances whose regular launch keeps more per-warp partials than the
    fixed array holds: the allocation-free call runs fewer resident blocks (packed
    per-instance offsets, reduced grid) and still gives the same bits."""
    import torch
    from mcphylo_gb300 import _lib
    L = _lib.load()
    insts = [random_instance(4, 4, t, s, seed=40 + t, multifurcate=0.05)
             for t, s in ((250, 3000), (200, 2500), (150, 2000))]
    h = _handle(L, _lib, insts, precision)
    assert L.mcphy_set_sweep(h, 1) == 0
    try:
        _compare_two_calls(L, _lib, h, insts, torch)
        counts = (ctypes.c_int64 * 3)()
        assert L.mcphy_get_counts(h, counts) == 0
        assert counts[2] > NOALLOC_BYTES   # the regular launch's partials exceed the array
    finally:
        L.mcphy_destroy(h)


def test_noalloc_timeout_writes_nan(built_lib):
    """A bounded wait that gives up cannot be reported in the status of an
    asynchronous call, so every output entry becomes NaN; the next call is
    unaffected.  The wait is made to run out on the host side (the first staging
    copy is never issued, mcphy_debug_inject kind 1), with no device fault."""
    import torch
    from mcphylo_gb300 import _lib
    L = _lib.load()
    insts = [random_instance(4, 4, 40, 3000, seed=51), random_instance(4, 4, 25, 1000, seed=52)]
    h = _handle(L, _lib, insts, 0)
    assert L.mcphy_set_sweep(h, 1) == 0
    try:
        M = len(insts)
        blen = np.concatenate([inst.blen for inst in insts])
        G = len(blen)
        ll_ref, g_ref = _regular(L, _lib, h, blen.copy(), M, G)
        assert L.mcphy_debug_inject(h, 1) == 0
        ll_na, g_na = _noalloc(L, h, torch, blen, M, G)
        assert np.all(np.isnan(ll_na)) and np.all(np.isnan(g_na))
        ll_na, g_na = _noalloc(L, h, torch, blen, M, G)
        assert np.array_equal(ll_na, ll_ref) and np.array_equal(g_na, g_ref)
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
