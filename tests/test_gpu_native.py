"""Native mesh kernels on the GPU against the oracle: ball of points,
boundary detection, Laplacian sweeps, mean-ratio quality statistics,
histogram, argmin and FP64-decided inverted-element flags."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def make(G, g, n, split, jitter, seed, fix):
    crd, tet, ref = G.cube_mesh(n, split=split, jitter=jitter, seed=seed)
    v, t = G.upload_mesh(g, crd, tet, ref)
    assert G.lib.GmlxMeshSetup(g, fix) == 1
    return crd, tet, ref, v, t


@pytest.mark.parametrize("split", [0, 1])
def test_ball_of_points_and_boundary(G, O, gpu, split):
    crd, tet, ref, v, t = make(G, gpu, 10, split, 0.3, 11, 2)
    fixed = O.boundary_vertices(len(crd), tet)
    assert np.array_equal(fixed, (ref != 0).astype(np.int32))   # cube boundary
    ptr, col = O.point_ball(len(crd), tet, fixed)
    stored, used, mx = ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_int()
    G.lib.GmlxMeshBallInfo(gpu, ctypes.byref(stored), ctypes.byref(used), ctypes.byref(mx))
    assert used.value == len(col)
    assert mx.value == int(np.diff(ptr).max())


@pytest.mark.parametrize("split,fix", [(0, 2), (1, 1), (1, 0)])
def test_laplacian_sweeps_match_oracle(G, O, gpu, split, fix):
    crd, tet, ref, v, t = make(G, gpu, 12, split, 0.3, 21, fix)
    fixed = {0: np.zeros(len(crd), np.int32), 1: (ref != 0).astype(np.int32),
             2: O.boundary_vertices(len(crd), tet)}[fix]
    ptr, col = O.point_ball(len(crd), tet, fixed)
    assert G.lib.GmlxSmooth(gpu, 3, ctypes.c_float(0.7)) == 1
    got = G.get_data(gpu, v, np.float32, (len(crd), 4))
    exp = O.laplace(crd, ptr, col, 0.7, 3)
    assert np.max(np.abs(got - exp)) <= 2e-6
    if fix:
        assert np.array_equal(got[fixed == 1], crd[fixed == 1])


def check_stats(O, crd, tet, res, h):
    q, hist, flags, ninv = O.quality_stats(crd, tet)
    assert res.NmbInv == ninv
    # histogram: bins can only differ for tets within 1e-5 of a bin edge
    edge = np.abs(q * 64 - np.round(q * 64)) < 1e-4 * 64
    got = np.array(res.Hist[:], np.int64)
    assert abs(int(got.sum()) - len(tet)) == 0
    assert np.abs(got - hist.astype(np.int64)).sum() <= 2 * int(edge.sum())
    # extrema: exact index unless the runner-up is within FP32 error
    srt = np.sort(q)
    if srt[1] - srt[0] > 1e-5 * abs(srt[0]) + 1e-7:
        assert res.MinIdx == int(np.argmin(q))
    assert abs(res.MinQal - q.min()) <= 2e-5
    assert abs(res.MaxQal - q.max()) <= 2e-5
    assert res.SumQal == pytest.approx(q.sum(), rel=2e-6)
    return q, flags


@pytest.mark.parametrize("n,split,jitter", [(16, 0, 0.25), (14, 1, 0.45), (45, 1, 0.3)])
def test_quality_stats_match_oracle(G, O, gpu, n, split, jitter):
    crd, tet, ref, v, t = make(G, gpu, n, split, jitter, 5, 1)
    qidx = G.lib.GmlNewSolutionData(gpu, G.GmlTetrahedra, 1, G.GmlFlt, b"q")
    res = G.GmlxQuality()
    assert G.lib.GmlxQualityStats(gpu, 1.0 / n, qidx, ctypes.byref(res)) == 1
    q, flags = check_stats(O, crd, tet, res, 1.0 / n)
    qg = G.get_data(gpu, qidx, np.float32, len(tet))
    assert np.max(np.abs(qg - q)) <= 2e-5
    fl = np.zeros((len(tet) + 31) // 32, np.uint32)
    assert G.lib.GmlxInvertedFlags(gpu, G.as_ptr(fl), len(fl)) == 1
    assert np.array_equal(fl, flags)                     # bit-exact


def test_inverted_elements_exact(G, O, gpu):
    """Large jitter inverts tets; flipped and near-flat tets are decided by
    the FP64 determinant and must match the oracle bit for bit."""
    crd, tet, ref, v, t = make(G, gpu, 12, 0, 0.49, 77, 1)
    res = G.GmlxQuality()
    assert G.lib.GmlxQualityStats(gpu, 1.0 / 12, 0, ctypes.byref(res)) == 1
    q, hist, flags, ninv = O.quality_stats(crd, tet)
    assert ninv > 0 and res.NmbInv == ninv
    fl = np.zeros(len(flags), np.uint32)
    G.lib.GmlxInvertedFlags(gpu, G.as_ptr(fl), len(fl))
    assert np.array_equal(fl, flags)


def test_smoothing_loop_graph_matches_oracle(G, O, gpu):
    n = 16
    crd, tet, ref, v, t = make(G, gpu, n, 1, 0.3, 3, 1)
    fixed = (ref != 0).astype(np.int32)
    ptr, col = O.point_ball(len(crd), tet, fixed)
    res = (G.GmlxQuality * 10)()
    assert G.lib.GmlxSmoothQualityLoop(gpu, 10, ctypes.c_float(1.0), 1.0 / n, res) == 1
    got = G.get_data(gpu, v, np.float32, (len(crd), 4))
    exp = O.laplace(crd, ptr, col, 1.0, 10)
    assert np.max(np.abs(got - exp)) <= 1e-5
    # the quality after the last sweep, on the GPU's own coordinates
    check_stats(O, got, tet, res[9], 1.0 / n)
    # quality improves under smoothing
    assert res[9].MinQal > res[0].MinQal
    # replay: the graph runs again from the smoothed state
    assert G.lib.GmlxSmoothQualityLoop(gpu, 10, ctypes.c_float(1.0), 1.0 / n, res) == 1
    got2 = G.get_data(gpu, v, np.float32, (len(crd), 4))
    exp2 = O.laplace(got.astype(np.float64), ptr, col, 1.0, 10)
    assert np.max(np.abs(got2 - exp2)) <= 1e-5


def test_ball_window_tuning_keeps_results(G, O, gpu):
    """The sorting window of the ball-of-points layout changes the padding,
    not the results: sweeps with windows 64 and 256 are bit-identical, and
    GmlxMeshTune picks a window, leaves the coordinates untouched and
    records the window in use."""
    n = 24
    crd, tet, ref = G.cube_mesh(n, split=1, jitter=0.3, seed=9)
    v, t = G.upload_mesh(gpu, crd, tet, ref)
    out = {}
    for w in (64, 256):
        assert G.lib.GmlxSetBallWindow(gpu, w) == 1
        assert G.lib.GmlxMeshSetup(gpu, 1) == 1
        assert G.lib.GmlxBallWindow(gpu) == w
        G.set_data(gpu, v, crd)
        assert G.lib.GmlxSmooth(gpu, 3, ctypes.c_float(0.7)) == 1
        out[w] = G.get_data(gpu, v, np.float32, (len(crd), 4))
    assert np.array_equal(out[64], out[256])
    ptr, col = O.point_ball(len(crd), tet, (ref != 0).astype(np.int32))
    assert np.max(np.abs(out[64] - O.laplace(crd, ptr, col, 0.7, 3))) <= 2e-6
    G.set_data(gpu, v, crd)
    w = G.lib.GmlxMeshTune(gpu, 3, ctypes.c_float(0.7))
    assert w in (64, 128, 256) and G.lib.GmlxBallWindow(gpu) == w
    assert np.array_equal(G.get_data(gpu, v, np.float32, (len(crd), 4)), crd)
    assert G.lib.GmlxSetBallWindow(gpu, 100) == 0
