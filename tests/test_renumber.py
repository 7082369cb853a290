"""Mesh renumbering on the host: the Hilbert renumbering, the degree
partition that the reference's ball tables expect (low degrees first,
Documentation/GMlib3_en.tex:401) and GmlEvaluateNumbering
(sources/gmlib3.c:4409-4442).  CPU only."""
import ctypes

import numpy as np
import pytest

from conftest import PARAMS


def raw_cube(G, n, split):
    nv, nt = ctypes.c_int(), ctypes.c_int()
    G.lib.GmlxCubeSizes(n, ctypes.byref(nv), ctypes.byref(nt))
    crd = np.zeros((nv.value, 4), np.float32)
    tet = np.zeros((nt.value, 4), np.int32)
    ref = np.zeros(nv.value, np.int32)
    G.lib.GmlxCubeMesh(n, split, 0.3, 77, G.as_ptr(crd), G.as_ptr(tet), G.as_ptr(ref))
    return crd, tet, ref


def same_mesh(crd0, tet0, crd1, tet1, prm):
    """prm maps old vertex indices to new ones: coordinates moved with their
    vertex, and every tet still joins the same points (tets may be reordered)."""
    assert np.array_equal(np.sort(prm), np.arange(len(crd0)))
    assert np.array_equal(crd1[prm], crd0)
    a = np.sort(np.sort(prm[tet0], axis=1), axis=0)
    b = np.sort(np.sort(tet1, axis=1), axis=0)
    assert np.array_equal(np.unique(a, axis=0), np.unique(b, axis=0))


def evaluate_numbering(tet):
    """The reference's measure: a 16-entry direct-mapped cache of 1 K vertex
    blocks indexed by bits 4..7, walked over the element table.  Element
    data hold one item per line (NmbItm = 1, sources/gmlib3.c:589), so the
    walk reads the first vertex of each element only."""
    tab = [0] * 16
    hit = mis = 0
    for v in tet[:, 0].tolist():
        pos, adr = (v >> 4) & 0xf, v >> 10
        if tab[pos] == adr:
            hit += 1
        else:
            mis += 1
            tab[pos] = adr
    return np.float32(100) * np.float32(hit) / np.float32(hit + mis)


def offline_score(G, crd, tet, ref):
    g = G.lib.GmlxInitOffline()
    G.lib.GmlNewParameters(g, 8, PARAMS)
    G.upload_mesh(g, crd, tet, ref)
    G.lib.GmlEvaluateNumbering.restype = ctypes.c_float
    s = G.lib.GmlEvaluateNumbering(g)
    G.lib.GmlStop(g)
    return s


@pytest.mark.parametrize("split", [0, 1])
def test_hilbert_renumber_is_a_consistent_permutation(G, split):
    crd0, tet0, ref0 = raw_cube(G, 9, split)
    crd, tet, ref = crd0.copy(), tet0.copy(), ref0.copy()
    prm = np.zeros(len(crd), np.int32)
    assert G.lib.GmlxHilbertRenumber(len(crd), G.as_ptr(crd), G.as_ptr(ref), len(tet),
                                     G.as_ptr(tet), G.as_ptr(prm)) == 1
    same_mesh(crd0, tet0, crd, tet, prm)
    assert np.array_equal(ref[prm], ref0)


def test_evaluate_numbering_matches_its_definition_and_rewards_locality(G):
    crd, tet, ref = G.cube_mesh(12, split=1, jitter=0.3, seed=5)
    score = offline_score(G, crd, tet, ref)
    assert score == evaluate_numbering(tet)
    # the same mesh under a random vertex numbering scores lower
    rng = np.random.default_rng(1)
    prm = rng.permutation(len(crd)).astype(np.int32)
    crd_r = np.empty_like(crd)
    crd_r[prm] = crd
    ref_r = np.empty_like(ref)
    ref_r[prm] = ref
    tet_r = prm[tet]
    worse = offline_score(G, crd_r, tet_r, ref_r)
    assert worse == evaluate_numbering(tet_r) and worse < score


@pytest.mark.parametrize("n,split,bal", [(8, 1, 32), (7, 0, 20), (6, 1, 16)])
def test_degree_sort_partitions_stably(G, O, n, split, bal):
    crd0, tet0, ref0 = G.cube_mesh(n, split=split, jitter=0.3, seed=n)
    crd, tet, ref = crd0.copy(), tet0.copy(), ref0.copy()
    prm = np.zeros(len(crd), np.int32)
    low = G.lib.GmlxDegreeSort(len(crd), G.as_ptr(crd), G.as_ptr(ref), len(tet), G.as_ptr(tet),
                               bal, G.as_ptr(prm))
    deg0 = np.bincount(tet0.ravel(), minlength=len(crd0))
    assert low == int((deg0 <= bal).sum())
    same_mesh(crd0, tet0, crd, tet, prm)
    assert np.array_equal(ref[prm], ref0)
    assert np.array_equal(tet, prm[tet0])                 # tets keep their order
    deg = np.bincount(tet.ravel(), minlength=len(crd))
    assert np.all(deg[:low] <= bal) and np.all(deg[low:] > bal)
    # stable: each group keeps the previous order
    lo_old = np.nonzero(deg0 <= bal)[0]
    hi_old = np.nonzero(deg0 > bal)[0]
    assert np.array_equal(prm[lo_old], np.arange(low))
    assert np.array_equal(prm[hi_old], np.arange(low, len(crd)))
    if bal == 32 and low < len(crd):
        # the ball tables' wide part now starts after every low-degree vertex
        d, mp, hs, base, high = O.ver_tet_ball(len(crd), tet, 32, 64)
        assert mp == low and hs == 64


def test_degree_sort_rejects_bad_input(G):
    crd, tet, ref = G.cube_mesh(3, split=0, jitter=0.2, seed=1)
    bad = tet.copy()
    bad[5, 2] = len(crd)
    c = crd.copy()
    assert G.lib.GmlxDegreeSort(len(crd), G.as_ptr(c), G.as_ptr(ref), len(bad), G.as_ptr(bad),
                                32, None) == -1
    assert np.array_equal(c, crd)                        # nothing moved
    assert G.lib.GmlxDegreeSort(len(crd), G.as_ptr(c), None, len(tet), G.as_ptr(tet.copy()),
                                0, None) == -1
