"""Edge cases on the GPU: empty datatypes, the smallest mesh, a zero
right-hand side, size mismatches and bad indices.  Each returns what the
reference's contract says (error codes, identities), without a device
error."""
import ctypes

import numpy as np
import pytest

from conftest import PARAMS

pytestmark = pytest.mark.gpu


def test_empty_datatypes(G, gpu):
    g = gpu
    G.lib.GmlNewParameters(g, 8, PARAMS)
    v = G.lib.GmlNewMeshData(g, G.GmlVertices, 0)
    t = G.lib.GmlNewMeshData(g, G.GmlTetrahedra, 0)
    assert v > 0 and t > 0
    q = G.lib.GmlNewSolutionData(g, G.GmlTetrahedra, 1, G.GmlFlt, b"qal")
    assert q > 0
    # a generated kernel over no tets launches nothing and succeeds
    body = b"qal = CalVol(VerCrd[0], VerCrd[1], VerCrd[2], VerCrd[3]);"
    k = G.compile_kernel(g, body, "vol", G.GmlTetrahedra,
                         [(v, G.GmlReadMode, 0), (q, G.GmlWriteMode, 0)])
    assert k > 0 and G.lib.GmlLaunchKernel(g, k) == 1
    # reductions of nothing: the identities of each operation
    assert G.reduce(g, q, G.GmlSum) == 0.0
    assert G.reduce(g, q, G.GmlMin) == pytest.approx(np.finfo(np.float32).max)
    assert G.reduce(g, q, G.GmlMax) == pytest.approx(-np.finfo(np.float32).max)
    # whole-datatype transfers of zero bytes
    buf = np.zeros(4, np.float32)
    assert G.lib.GmlxSetData(g, v, G.as_ptr(buf), 0) == 1
    assert G.lib.GmlxGetData(g, v, G.as_ptr(buf), 0) == 1


def test_single_hex(G, O, gpu):
    """The smallest mesh: one hex, 6 tets, 8 vertices, all on the boundary:
    sweeps leave it unchanged and the statistics match the oracle."""
    g = gpu
    crd, tet, ref = G.cube_mesh(1, split=0, jitter=0.0, seed=1)
    v, t = G.upload_mesh(g, crd, tet, ref)
    assert G.lib.GmlxMeshSetup(g, 1) == 1
    assert G.lib.GmlxSmooth(g, 3, ctypes.c_float(1.0)) == 1
    out = G.get_data(g, v, np.float32, crd.shape)
    assert np.array_equal(out, crd)
    res = G.GmlxQuality()
    assert G.lib.GmlxQualityStats(g, ctypes.c_double(1.0), 0, ctypes.byref(res)) == 1
    q = O.mean_ratio(crd, tet)
    assert res.MinQal == pytest.approx(q.min(), rel=1e-6)
    assert res.MaxQal == pytest.approx(q.max(), rel=1e-6)
    assert res.MinIdx == int(np.argmin(q))
    assert res.NmbInv == 0 and sum(res.Hist) == 6


@pytest.mark.parametrize("mode", [0, 1])
def test_cg_zero_rhs(G, gpu, mode):
    """b = 0: converged before the first iteration, x = 0."""
    lin, col, val, rhs = G.cube_spd(3, 0, seed=2)
    IP = ctypes.POINTER(ctypes.c_int)
    v64 = np.ascontiguousarray(val)
    m = G.lib.GmlNewMatrix(gpu, len(lin) - 1, len(col), 3, G.as_ptr(v64),
                           col.ctypes.data_as(IP), lin.ctypes.data_as(IP), G.GmlDbl)
    zero = np.zeros_like(rhs)
    ib = G.lib.GmlNewVector(gpu, len(rhs), 3, G.as_ptr(zero), G.GmlDbl)
    guess = np.ones_like(rhs)
    ix = G.lib.GmlNewVector(gpu, len(rhs), 3, G.as_ptr(guess), G.GmlDbl)
    info = G.GmlxSolveInfo()
    assert G.lib.GmlxSolveCG(gpu, m, ib, ix, mode, 1e-10, 100, ctypes.byref(info)) == 1
    assert info.NmbIte == 0 and info.RelRes == 0.0
    x = G.get_data(gpu, G.lib.GmlxVectorData(gpu, ix), np.float64, (len(rhs), 4))
    assert not x.any()


def test_size_mismatch_and_bad_indices(G, gpu, capfd):
    g = gpu
    v = G.lib.GmlNewMeshData(g, G.GmlVertices, 10)
    buf = np.zeros((10, 4), np.float32)
    assert G.lib.GmlxSetData(g, v, G.as_ptr(buf), buf.nbytes - 16) == 0
    assert G.lib.GmlxGetData(g, v, G.as_ptr(buf), buf.nbytes + 16) == 0
    assert G.lib.GmlxSetData(g, 99, G.as_ptr(buf), buf.nbytes) == 0
    r = ctypes.c_double()
    assert G.lib.GmlReduceVector(g, 99, G.GmlSum, ctypes.byref(r)) == -1
    assert G.lib.GmlReduceVector(g, v, G.GmlSum, ctypes.byref(r)) == -2      # float4 lines
    q = G.lib.GmlNewSolutionData(g, G.GmlVertices, 1, G.GmlFlt, b"q")
    assert G.lib.GmlReduceVector(g, q, 9, ctypes.byref(r)) == -3
    assert G.lib.GmlLaunchKernel(g, 77) == -1
    ctypes.CDLL(None).fflush(None)                 # the library's printf output
    out = capfd.readouterr().out
    assert "Invalid data index: 99" in out and "Invalid operation code 9" in out
