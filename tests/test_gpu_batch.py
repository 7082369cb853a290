"""Batched meshes through the C ABI: the persistent tile-queue launch and the
per-mesh launch loop give every mesh the same coordinates, quality
statistics and inverted flags as processing that mesh alone in its own
instance (bit-exact; the quality sum to 1e-7 relative: both are
compensated FP32 sums folded in FP64, grouped differently)."""
import ctypes

import numpy as np
import pytest

import gmlib_gb300 as G

MESHES = [(3, 0, 0.3), (7, 1, 0.3), (4, 1, 0.25), (9, 0, 0.35), (2, 0, 0.2), (6, 1, 0.3)]
OMEGA = ctypes.c_float(0.8)


def meshes():
    out = []
    for i, (n, split, jit) in enumerate(MESHES):
        crd, tet, ref = G.cube_mesh(n, split=split, jitter=jit, seed=40 + i)
        out.append((n, crd, tet, ref))
    return out


def make_batch(ms, fix=1):
    g = G.lib.GmlInit(0)
    assert g
    nm = len(ms)
    nv = np.array([len(m[1]) for m in ms], np.int32)
    nt = np.array([len(m[2]) for m in ms], np.int32)
    h = np.array([1.0 / m[0] for m in ms], np.float64)
    assert G.lib.GmlxBatchCreate(g, nm, G.as_ptr(nv), G.as_ptr(nt), G.as_ptr(h)) == 1
    for i, (n, crd, tet, ref) in enumerate(ms):
        assert G.lib.GmlxBatchSetMesh(g, i, G.as_ptr(crd), G.as_ptr(ref), G.as_ptr(tet)) == 1
    assert G.lib.GmlxBatchSetup(g, fix) == 1
    return g


def alone(n, crd, tet, ref, sweeps, rounds=1, fix=1):
    g = G.lib.GmlInit(0)
    try:
        v, t = G.upload_mesh(g, crd, tet, ref)
        assert G.lib.GmlxMeshSetup(g, fix) == 1
        q = G.GmlxQuality()
        for _ in range(rounds):
            assert G.lib.GmlxSmooth(g, sweeps, OMEGA) == 1
            assert G.lib.GmlxQualityStats(g, 1.0 / n, 0, ctypes.byref(q)) == 1
        c = G.get_data(g, v, np.float32, crd.shape)
        nw = (len(tet) + 31) // 32
        fl = np.zeros(nw, np.uint32)
        assert G.lib.GmlxInvertedFlags(g, G.as_ptr(fl), nw) == 1
        return c, q, fl
    finally:
        G.lib.GmlStop(g)


def batch_results(g, ms):
    out = []
    for i, (n, crd, tet, ref) in enumerate(ms):
        c = np.zeros_like(crd)
        assert G.lib.GmlxBatchGetMesh(g, i, G.as_ptr(c)) == 1
        nw = (len(tet) + 31) // 32
        fl = np.zeros(nw, np.uint32)
        assert G.lib.GmlxBatchFlags(g, i, G.as_ptr(fl), nw) == 1
        out.append((c, fl))
    return out


def same_quality(a, b):
    assert (a.MinQal, a.MinIdx, a.MaxQal, a.MaxIdx) == (b.MinQal, b.MinIdx, b.MaxQal, b.MaxIdx)
    assert (a.NmbInv, a.NmbF64) == (b.NmbInv, b.NmbF64)
    assert list(a.Hist) == list(b.Hist)
    # both sums are compensated FP32 sums folded in FP64, grouped differently
    assert a.SumQal == pytest.approx(b.SumQal, rel=1e-7)


@pytest.mark.gpu
@pytest.mark.parametrize("mode,warp", [(G.GmlxBatchQueue, 0), (G.GmlxBatchQueue, 1),
                                       (G.GmlxBatchLoop, 0)])
@pytest.mark.parametrize("sweeps", [0, 3])
def test_batch_matches_each_mesh_alone(mode, warp, sweeps):
    ms = meshes()
    g = make_batch(ms)
    try:
        if warp:
            assert G.lib.GmlxBatchSetTiles(g, 1, 4, 1024, 0) == 1
        res = (G.GmlxQuality * len(ms))()
        assert G.lib.GmlxBatchRun(g, sweeps, OMEGA, mode, res) == 1
        got = batch_results(g, ms)
    finally:
        G.lib.GmlStop(g)
    for i, m in enumerate(ms):
        c, q, fl = alone(*m, sweeps)
        assert np.array_equal(got[i][0], c), i
        assert np.array_equal(got[i][1], fl), i
        same_quality(res[i], q)


@pytest.mark.gpu
def test_batch_replay_and_tuning_keep_results():
    """Graph replays continue from the smoothed coordinates; tuning leaves
    the coordinates untouched and picks a configuration that gives the same
    results."""
    ms = meshes()
    g = make_batch(ms)
    try:
        before = batch_results(g, ms)
        assert G.lib.GmlxBatchTune(g, 2, OMEGA) == 1
        after = batch_results(g, ms)
        for a, b in zip(before, after):
            assert np.array_equal(a[0], b[0])
        ts, tt, grid, nt, wt = (ctypes.c_int() for _ in range(5))
        assert G.lib.GmlxBatchInfo(g, ctypes.byref(ts), ctypes.byref(tt), ctypes.byref(grid),
                                   ctypes.byref(nt), ctypes.byref(wt)) == 1
        assert ts.value in (2, 4, 8, 16, 32, 128) and grid.value > 0 and wt.value in (0, 1)
        res = (G.GmlxQuality * len(ms))()
        for _ in range(2):
            assert G.lib.GmlxBatchRun(g, 2, OMEGA, G.GmlxBatchQueue, res) == 1
        got = batch_results(g, ms)
    finally:
        G.lib.GmlStop(g)
    for i, m in enumerate(ms):
        c, q, fl = alone(*m, 2, rounds=2)
        assert np.array_equal(got[i][0], c), i
        same_quality(res[i], q)


@pytest.mark.gpu
def test_batch_against_oracle(O):
    """One mesh of the batch against the FP64 oracle: Laplacian sweeps over
    the ball of points with fixed boundary (|dx| <= 1e-5 h) and the quality
    histogram / inverted count of the result."""
    ms = meshes()
    g = make_batch(ms)
    try:
        res = (G.GmlxQuality * len(ms))()
        assert G.lib.GmlxBatchRun(g, 3, OMEGA, G.GmlxBatchQueue, res) == 1
        got = batch_results(g, ms)
    finally:
        G.lib.GmlStop(g)
    k = 3
    n, crd, tet, ref = ms[k]
    ptr, col = O.point_ball(len(crd), tet, (ref != 0).astype(np.int32))
    want = O.laplace(crd, ptr, col, OMEGA.value, 3)
    assert np.max(np.abs(got[k][0][:, :3] - want[:, :3])) <= 1e-5 / n
    q, hist, flags, ninv = O.quality_stats(got[k][0], tet)
    assert res[k].NmbInv == ninv
    assert np.sum(np.abs(np.array(list(res[k].Hist), np.int64) - hist.astype(np.int64))) <= 2


@pytest.mark.gpu
def test_batch_rejects_bad_input():
    g = G.lib.GmlInit(0)
    try:
        nv = np.array([8], np.int32)
        nt = np.array([1], np.int32)
        h = np.array([1.0])
        assert G.lib.GmlxBatchCreate(g, 1, G.as_ptr(nv), G.as_ptr(nt), G.as_ptr(h)) == 1
        crd = np.zeros((8, 4), np.float32)
        bad = np.array([[0, 1, 2, 8]], np.int32)
        assert G.lib.GmlxBatchSetMesh(g, 0, G.as_ptr(crd), None, G.as_ptr(bad)) == 0
        assert G.lib.GmlxBatchRun(g, 1, OMEGA, G.GmlxBatchQueue, None) == 0   # not set up
        assert G.lib.GmlxBatchCreate(g, 1, G.as_ptr(nv), G.as_ptr(nt), G.as_ptr(h)) == 0
    finally:
        G.lib.GmlStop(g)


@pytest.mark.gpu
@pytest.mark.parametrize("warp", [0, 1])
def test_batch_dependency_wait_times_out_and_recovers(capfd, warp):
    """A queue whose first sweep of mesh 0 can never finish (one tile held
    back on the host, GmlxBatchSetWaitLimit) with a wait limit of 4096 tries
    (about 1 ms): the launch stops on its own with error bit 16,
    GmlxBatchRun returns 0 and says why; with the limit and the queue
    restored and the meshes set again, the same instance gives the results
    of each mesh processed alone.  Nothing on the GPU faults or hangs: the
    wait gives up and every block returns."""
    ms = meshes()
    g = make_batch(ms)
    try:
        if warp:
            assert G.lib.GmlxBatchSetTiles(g, 1, 4, 1024, 0) == 1
        res = (G.GmlxQuality * len(ms))()
        assert G.lib.GmlxBatchSetWaitLimit(g, 4096, 1) == 1
        assert G.lib.GmlxBatchRun(g, 2, OMEGA, G.GmlxBatchQueue, res) == 0
        assert "waited too long" in capfd.readouterr().out
        assert G.lib.GmlxBatchSetWaitLimit(g, 0, 0) == 1
        for i, (n, crd, tet, ref) in enumerate(ms):
            assert G.lib.GmlxBatchSetMesh(g, i, G.as_ptr(crd), G.as_ptr(ref), G.as_ptr(tet)) == 1
        assert G.lib.GmlxBatchSetup(g, 1) == 1
        assert G.lib.GmlxBatchRun(g, 2, OMEGA, G.GmlxBatchQueue, res) == 1
        got = batch_results(g, ms)
    finally:
        G.lib.GmlStop(g)
    for i, m in enumerate(ms):
        c, q, fl = alone(*m, 2)
        assert np.array_equal(got[i][0], c), i
        same_quality(res[i], q)
