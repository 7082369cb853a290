"""Parity at the benchmark configurations' own sizes, against the FP64
oracle:

  config 1  32^3-hex Kuhn cube, jitter 0.25 h, seed 12345 (196,608 tets):
            the native quality pass and the mean-ratio body through
            GmlCompileKernel give the oracle's argmin and argmax and its
            inverted flags exactly, and its qualities within 2e-5;
  config 2  128^3-hex reflected cube, jitter 0.3 h, seed 2024, boundary
            fixed (12,582,912 tets): 10 Jacobi sweeps and the quality
            statistics of every sweep (GmlxSmoothQualityLoop); coordinates
            within 2e-6 of the FP64 sweeps, the last sweep's histogram,
            extrema and flags against the oracle on the GPU's coordinates;
  config 3  the 96^3-hex SPD block system (912,673 rows): FP64 CG and FP32
            CG inside FP64 refinement, true residual |b - Ax| / |b| <= 1e-10
            computed by the oracle in long double.
"""
import ctypes

import numpy as np
import pytest

import gmlib_gb300 as G
from test_gpu_linalg import solve
from test_gpu_native import check_stats

pytestmark = pytest.mark.gpu


def test_config1_quality_argmin_exact(O, gpu):
    n = 32
    crd, tet, ref = G.cube_mesh(n, split=0, jitter=0.25, seed=12345)
    v, t = G.upload_mesh(gpu, crd, tet, ref)
    q, hist, flags, ninv = O.quality_stats(crd, tet)
    srt = np.sort(q)
    # the configuration has isolated extrema: argmin and argmax are decided
    assert srt[1] - srt[0] > 1e-4 and srt[-1] - srt[-2] > 1e-6
    assert G.lib.GmlxMeshSetup(gpu, 1) == 1
    res = G.GmlxQuality()
    qn = G.lib.GmlNewSolutionData(gpu, G.GmlTetrahedra, 1, G.GmlFlt, b"qn")
    assert G.lib.GmlxQualityStats(gpu, 1.0 / n, qn, ctypes.byref(res)) == 1
    assert res.MinIdx == int(np.argmin(q)) and res.MaxIdx == int(np.argmax(q))
    assert abs(res.MinQal - q.min()) <= 2e-5 and abs(res.MaxQal - q.max()) <= 2e-5
    assert res.NmbInv == ninv
    fl = np.zeros(len(flags), np.uint32)
    assert G.lib.GmlxInvertedFlags(gpu, G.as_ptr(fl), len(fl)) == 1
    assert np.array_equal(fl, flags)
    assert np.max(np.abs(G.get_data(gpu, qn, np.float32, len(tet)) - q)) <= 2e-5
    # the same measure as a dialect body through the generator
    qb = G.lib.GmlNewSolutionData(gpu, G.GmlTetrahedra, 1, G.GmlFlt, b"qal")
    k = G.compile_kernel(gpu, G.mean_ratio_body(), "mean_ratio", G.GmlTetrahedra,
                         [(v, G.GmlReadMode, 0), (qb, G.GmlWriteMode, 0)])
    assert k > 0 and G.lib.GmlLaunchKernel(gpu, k) == 1
    qg = G.get_data(gpu, qb, np.float32, len(tet))
    assert np.max(np.abs(np.abs(qg) - np.abs(q))) <= 2e-5
    fmin, imin, fmax, imax = ctypes.c_float(), ctypes.c_int(), ctypes.c_float(), ctypes.c_int()
    assert G.lib.GmlxReduceArg(gpu, qb, ctypes.byref(fmin), ctypes.byref(imin),
                               ctypes.byref(fmax), ctypes.byref(imax)) == 1
    assert imin.value == int(np.argmin(q)) and imax.value == int(np.argmax(q))


def test_config2_smoothing_at_size(O, gpu):
    n = 128
    crd, tet, ref = G.cube_mesh(n, split=1, jitter=0.3, seed=2024)
    v, t = G.upload_mesh(gpu, crd, tet, ref)
    assert G.lib.GmlxMeshSetup(gpu, 1) == 1
    res = (G.GmlxQuality * 10)()
    assert G.lib.GmlxSmoothQualityLoop(gpu, 10, ctypes.c_float(1.0), 1.0 / n, res) == 1
    got = G.get_data(gpu, v, np.float32, (len(crd), 4))
    fixed = (ref != 0).astype(np.int32)
    ptr, col = O.point_ball(len(crd), tet, fixed)
    exp = O.laplace(crd, ptr, col, 1.0, 10)
    assert np.max(np.abs(got - exp)) <= 2e-6
    assert np.array_equal(got[fixed == 1], crd[fixed == 1])
    q, flags = check_stats(O, got, tet, res[9], 1.0 / n)
    fl = np.zeros(len(flags), np.uint32)
    assert G.lib.GmlxInvertedFlags(gpu, G.as_ptr(fl), len(fl)) == 1
    assert np.array_equal(fl, flags)


@pytest.mark.parametrize("mode", [G.GmlxCgFp64, G.GmlxCgMixed])
def test_config3_cg_at_size(O, gpu, mode):
    lin, col, val, rhs = G.cube_spd(96, 0, seed=2024)
    assert len(lin) - 1 == 912673 and len(col) == 13465441
    rc, x, info = solve(gpu, lin, col, val, rhs, mode)
    assert rc == 1, (rc, info.NmbIte, info.RelRes)
    rel = O.rel_residual(lin, col, val, rhs, x)
    assert rel <= 1e-10
    assert info.RelRes == pytest.approx(rel, rel=1e-3, abs=1e-13)
