"""Host-side tests that need no GPU: the C ABI exports, schedule validation,
parsers, substitution models, rates and the PhyloDist constructors."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT, load_alignment
from oracle import pyoracle as O

import mcphylo_gb300 as mp
from mcphylo_gb300 import _lib, models, parse, tree as T

HEADER = os.path.join(ROOT, "include", "mcphylo_gpu.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(mcphy_\w+)\s*\(", src)))


def test_library_exports_every_declared_symbol(built_lib):
    L = ctypes.CDLL(built_lib)
    names = declared_functions()
    assert len(names) >= 25
    for n in names:
        assert hasattr(L, n), n
    assert sorted(_lib.SIGNATURES) == names


def test_smem_allowance_is_per_device_and_thread_safe(built_lib):
    """The record of each kernel's dynamic shared-memory allowance is kept per
    device and behind a mutex (a kernel attribute is set on the current device
    only), checked against a fake setter from several threads: no GPU needed."""
    L = _lib.load()
    assert L.mcphy_debug_check_allowance() == 0


def test_version_and_status_strings(built_lib):
    L = _lib.load()
    assert L.mcphy_version() >= 100
    assert L.mcphy_status_string(-2) == b"dimension mismatch"


SIMU = ("(((0:0.110833,1:0.0137979)10:0.146124,(2:0.197891,(3:0.132967,(4:0.0378759,"
        "5:0.089252)11:0.101833)12:0.184301)13:0.0450774)14:0.335725,6:0.153197,(7:0.0216218,"
        "(8:0.0781687,9:0.120419)15:0.0209114)16:0.0209771);")


def test_schedule_info_binarises_multifurcations(built_lib):
    t = T.parse_newick(SIMU)
    parent, blen = T.to_parent(t)
    info = mp.schedule_info(parent)
    # 8 internal nodes (root trifurcating) -> 9 binary steps, 1 virtual branch
    assert info == {"internal": 9, "virtual": 1, "leaves": 10, "max_depth": 5, "pre_slots": 1}


@pytest.mark.parametrize("bad", [
    [0, 3, 0],            # two roots
    [3, 3, 1],            # root not at N
    [2, 3, 2, 0][:3],     # cycle / no root at N
    [4, 4, 4, 5, 0][:4],  # wrong length: root missing
])
def test_schedule_rejects_bad_trees(built_lib, bad):
    with pytest.raises(ValueError):
        mp.schedule_info(np.array(bad))


def test_schedule_rejects_unary_node(built_lib):
    # 1 -> 3, 2 -> 3, 3 -> 4 (unary), 4 root
    with pytest.raises(ValueError):
        mp.schedule_info(np.array([3, 3, 4, 0]))


def test_newick_numbering_matches_oracle():
    for nwk in (SIMU, "((A:1,B:2):0.5,(C:1,(D:1,E:1):1):0.25,F:3);", "(a,b);"):
        a = T.parse_newick(nwk)
        b = O.parse_newick(nwk)
        pa, ba = T.to_parent(a)
        fb = O.flatten(b)
        mother = fb[4]
        np.testing.assert_array_equal(pa, mother)
        np.testing.assert_array_equal(ba, fb[6])
        assert [n.name for n in T.post_order(a)] == [n.name for n in O.post_order(b)]


def test_newick_roundtrip():
    t = T.parse_newick(SIMU)
    t2 = T.parse_newick(T.newick(t))
    np.testing.assert_array_equal(T.to_parent(t)[0], T.to_parent(t2)[0])
    np.testing.assert_array_equal(T.to_parent(t)[1], T.to_parent(t2)[1])


def test_models_against_golden(golden):
    sm = golden["substitution_models"]
    r = sm["restriction"]
    U, D, Uinv, mu = models.Restriction(r["base_freq"])
    np.testing.assert_allclose(U, r["U"], rtol=1e-12)
    np.testing.assert_allclose(Uinv, r["Uinv"], rtol=1e-8)
    assert mu == pytest.approx(r["mu"], rel=1e-12)
    with pytest.raises(AssertionError):
        models.Restriction(np.ones(3) / 3)
    for key, fn, args in (("gtr", models.GTR, lambda m: (m["base_freq"], m["rates"])),
                          ("freek", models.freeK, lambda m: ([0.0], m["rates"]))):
        m = sm[key]
        U, D, Uinv, mu = fn(*args(m))
        Ug, Dg, Uig = np.array(m["U"]), np.array(m["D"]), np.array(m["Uinv"])
        for t in (0.05, 1.0):
            np.testing.assert_allclose(U @ np.diag(np.exp(D * t)) @ Uinv,
                                       Ug @ np.diag(np.exp(Dg * t)) @ Uig, atol=1e-12)
        assert mu == pytest.approx(m["mu"], rel=1e-12)
    j = sm["jc"]
    U, D, Uinv, mu = models.JC(j["base_freq"])
    np.testing.assert_allclose(U @ np.diag(D) @ Uinv, j["Q"], atol=1e-12)
    assert mu == pytest.approx(1.5)
    s = sm["setmatrix"]
    np.testing.assert_array_equal(models.setmatrix(s["input"]), np.array(s["output"]))


def test_calculate_transition_clipping():
    """test/likelihood/substitutionmodels.jl:16-47."""
    U, D, Uinv, mu = models.Restriction([0.3, 0.7])
    from scipy.linalg import expm
    P = expm(U @ np.diag(D) @ Uinv * mu)
    np.testing.assert_allclose(models.calculate_transition(models.Restriction, 1.0, mu, 1.0, U, Uinv, D, []), P, rtol=1e-10)
    assert np.array_equal(models.calculate_transition(models.Restriction, 1.0, mu, 1e-12, U, Uinv, D, []), np.eye(2))
    assert np.array_equal(models.calculate_transition(models.Restriction, 1.0, mu, 110.0, U, Uinv, D, [2.0, 1.0]),
                          np.array([[1.0, 1.0], [2.0, 2.0]]))
    cu = np.array([[1j, 2j], [0j, 3j]])
    assert np.array_equal(models.calculate_transition(models.Restriction, 1.0, mu, 110.0, cu, cu, D, [1.0, 2.0]),
                          np.array([[2.0, 2.0], [1.0, 1.0]]))
    U, D, Uinv, mu = models.JC([0.15, 0.45, 0.4])
    assert np.array_equal(models.calculate_transition(models.JC, 1.0, mu, 101.1, U, Uinv, D, [0.15, 0.45, 0.4]),
                          np.ones((3, 3)) / 3)


def test_rates_against_golden(golden):
    r = golden["rates"]
    rt = float(np.sqrt(np.finfo(float).eps))   # gamma_inc(..., sig=1) in the reference
    np.testing.assert_allclose(models.discrete_gamma_rates(0.5, 0.5, 4), r["mean"], rtol=rt)
    np.testing.assert_allclose(models.discrete_gamma_rates(0.5, 0.5, 4, "median"), r["median"],
                               rtol=1e-12)
    np.testing.assert_allclose(models.median_boundaries(0.5, 0.5, 4), r["median_boundaries"],
                               rtol=1e-12)
    np.testing.assert_allclose(models.mean_boundaries(0.5, 0.5, 4)[:3], r["mean_boundaries"],
                               rtol=1e-12)


def test_datafortree_matches_oracle(golden):
    g = golden["felsenstein"]["primates"]
    a = load_alignment("primates")
    t = T.parse_newick(g["newick"])
    syms = parse.get_alphabet(a["rows"], "-", "?")
    x = parse.datafortree(a["rows"], a["taxa"], t, syms, "-", "?")
    xo = O.datafortree(a["rows"], a["taxa"], O.parse_newick(g["newick"]), syms, "-", "?")
    np.testing.assert_array_equal(x, xo)
    leaf_nums = np.array(sorted(n.num for n in T.get_leaves(t)))
    codes, ok = parse.codes_from_tensor(x, leaf_nums)
    assert ok and codes.shape == (12, 898)
    back = mp.simulate.codes_to_tensor(codes, leaf_nums, 4, x.shape[2])
    np.testing.assert_array_equal(back[:, :, leaf_nums - 1], x[:, :, leaf_nums - 1])
    x2 = x.copy()
    x2[0, 0, leaf_nums[0] - 1] = 0.5
    assert parse.codes_from_tensor(x2, leaf_nums)[1] is False


def test_parse_nexus(tmp_path):
    a = load_alignment("simudata")
    f = tmp_path / "d.nex"
    lines = ["#NEXUS", "begin data;", "    dimensions ntax=10 nchar=100;",
             "    format datatype=dna interleave=no gap=-;", "    matrix"]
    lines += [f"{n}    {r}" for n, r in zip(a["taxa"], a["rows"])] + ["    ;", "end;"]
    f.write_text("\n".join(lines) + "\n")
    ntax, nchar, gap, miss, syms, rows, langs = mp.ParseNexus(str(f))
    assert (ntax, nchar, gap, miss) == (10, 100, "-", "?")
    assert syms == ["A", "C", "G", "T"] and langs == a["taxa"] and rows == a["rows"]


def test_phylodist_constructors(golden):
    """test/distributions/phylodist.jl:17-42 and :79-88 (size, equality, DimensionMismatch)."""
    g = golden["felsenstein"]["primates"]
    t = T.parse_newick(g["newick"])
    pden = np.ones(4) / 4
    pd = mp.PhyloDist(t, pden, [1.0], [1.0], mp.JC)
    assert pd.size == (4, 1, 22)
    assert pd.minimum() == -np.inf and pd.maximum() == np.inf
    for other in (mp.PhyloDist(t, pden, 1.0, 1.0, mp.JC),
                  mp.PhyloDist(t, [0.25, 0.25, 0.25, 0.25], [1.0], [1.0], mp.JC)):
        assert other == pd
    pd5 = mp.PhyloDist(t, [1.0], [1.0], mp.freeK)
    assert pd5.substitution_model is mp.freeK and pd5.nbase == 1
    trees = [t, t]
    freqs = np.full((4, 2), 0.25)
    rates = np.ones((1, 2))
    mpd = mp.MultiplePhyloDist(trees, freqs, rates, rates, mp.JC)
    assert mpd.size == (4, 1, 22, 2)
    assert mp.MultiplePhyloDist(trees, [1.0], [1.0], mp.freeK) == mp.MultiplePhyloDist(trees, rates, [1.0], mp.freeK)
    bad = np.array([[1.0, 2.0, 3.0]])
    with pytest.raises(mp.DimensionMismatch):
        mp.MultiplePhyloDist(trees, np.full((2, 3), 0.25), [1.0], [1.0], mp.JC)
    with pytest.raises(mp.DimensionMismatch):
        mp.MultiplePhyloDist(trees, freqs, bad, [1.0], mp.JC)
    with pytest.raises(mp.DimensionMismatch):
        mp.MultiplePhyloDist(trees, freqs, [1.0], bad, mp.JC)
    with pytest.raises(mp.DimensionMismatch):
        mp.MultiplePhyloDist(trees, bad, [1.0], mp.freeK)


def test_no_cpu_fallback_without_device(built_lib):
    """Without a GPU the engine fails loudly instead of computing on the host."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(mp.NoDeviceError):
        mp.Engine(4, 1)


def test_simulators_make_valid_instances(built_lib):
    inst = mp.simulate.restriction_small(S=50)
    assert inst.codes.shape == (32, 50) and inst.N == 63
    assert mp.schedule_info(inst.parent)["leaves"] == 32
    bd = mp.simulate.restriction_gamma_bd(S=10, taxa=40)
    assert mp.schedule_info(bd.parent)["leaves"] == 40
    batch = mp.simulate.hky_batch(n=3, scale=0.01)
    assert len(batch) == 3 and all(b.K == 4 and len(b.rates) == 4 for b in batch)


def test_compress_patterns():
    from mcphylo_gb300.parse import compress_patterns
    codes = np.array([[1, 2, 1, 1, 2], [2, 2, 2, 1, 2]], dtype=np.uint32)
    pat, w, idx = compress_patterns(codes)
    np.testing.assert_array_equal(pat, [[1, 2, 1], [2, 2, 1]])
    np.testing.assert_array_equal(w, [2, 2, 1])
    np.testing.assert_array_equal(idx, [0, 1, 0, 2, 1])
    np.testing.assert_array_equal(pat[:, idx], codes)
