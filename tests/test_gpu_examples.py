"""Three more of the reference's example flows through this library's
reference API on the GPU, against the reference's own run of them on the
same meshes (tests/golden/refhost_examples.npz, made by
tests/golden/make_refhost.py from examples/GpuBandwidth, TestFeatures and
BallQuality with their own kernel bodies).  The bodies here
(tests/kernels/ex_*.cl, ball_min.cl) compute the same values in the same
order, with datatype names of this file's choosing.

  - GpuBandwidth (gpu_bandwidth.c:100-175): direct vertex and tetrahedron
    reads and writes, a tet -> vertex downlink sum, a vertex -> tet ball sum;
  - TestFeatures (TestFeatures.c:95-215): an FP64 datatype kernel, a
    downlink with reference flags and the launch's line count, an uplink
    with voyeurs, the residual sum, three iterations with GmlPar->res = i;
    and a kernel reading through the GmlSetNeighbours link (the reference's
    neighbours body writes nothing, and its link holds pointer bits, so this
    one is checked against numpy on this library's link);
  - BallQuality (BallQuality.c:73-130): CalTriQal per triangle, then the
    minimum over each vertex's triangles, on a 2D triangle mesh.

The reference's residual sums come from its truncating reduction (its
first launch, calibrating, drops whole work-groups); they are compared
over every line instead (ft_red_exact)."""
import ctypes
import os

import numpy as np
import pytest

from conftest import PARAMS

pytestmark = pytest.mark.gpu

KDIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "kernels")
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def body(name):
    with open(os.path.join(KDIR, name), "rb") as f:
        return f.read()


def fixture():
    return dict(np.load(os.path.join(GOLD, "refhost_examples.npz")))


def close(got, want, rel):
    return np.max(np.abs(got - want)) <= rel * max(1.0, float(np.max(np.abs(want))))


def test_bandwidth_flow(G, gpu):
    r = fixture()
    nv, nt = len(r["crd"]), len(r["tet"])
    G.lib.GmlNewParameters(gpu, 8, PARAMS)
    v, t = G.upload_mesh(gpu, r["crd"], r["tet"], r["ref"])
    pts = G.lib.GmlNewSolutionData(gpu, G.GmlVertices, 1, G.GmlFlt4, b"Pts")
    cel = G.lib.GmlNewSolutionData(gpu, G.GmlTetrahedra, 1, G.GmlFlt4, b"Cel")
    Rd, Wr = G.GmlReadMode, G.GmlWriteMode
    steps = [("ex_vertex_copy.cl", G.GmlVertices, [(v, Rd, 0), (pts, Wr, 0)], pts, (nv, 4), "bw_ver"),
             ("ex_tet_nodes.cl", G.GmlTetrahedra, [(t, Rd, 0), (cel, Wr, 0)], cel, (nt, 4),
              "bw_tet_nodes"),
             ("ex_tet_sum.cl", G.GmlTetrahedra, [(v, Rd, 0), (cel, Wr, 0)], cel, (nt, 4),
              "bw_tet_sum"),
             ("ex_ball_sum.cl", G.GmlVertices, [(pts, Wr, 0), (cel, Rd, 0)], pts, (nv, 4), "bw_ball")]
    ks = [G.compile_kernel(gpu, body(f), f[:-3], msh, dats) for f, msh, dats, _, _, _ in steps]
    assert all(k > 0 for k in ks)
    for k, (f, _, _, out, shape, key) in zip(ks, steps):
        assert G.lib.GmlLaunchKernel(gpu, k) == 1, f
        got = G.get_data(gpu, out, np.float32, shape)
        if key == "bw_ball":
            assert close(got, r[key], 1e-6), key
        else:
            assert np.array_equal(got, r[key]), key


def test_features_flow(G, gpu):
    r = fixture()
    nv, nt = len(r["crd"]), len(r["tet"])
    p = G.lib.GmlNewParameters(gpu, 8, PARAMS)
    assert p
    v, t = G.upload_mesh(gpu, r["crd"], r["tet"], r["ref"])
    ngb = G.lib.GmlSetNeighbours(gpu, G.GmlTetrahedra)
    assert ngb > 0
    sol = G.lib.GmlNewSolutionData(gpu, G.GmlVertices, 2, G.GmlFlt4, b"Sol")
    mid = G.lib.GmlNewSolutionData(gpu, G.GmlTetrahedra, 1, G.GmlFlt4, b"Mid")
    rsd = G.lib.GmlNewSolutionData(gpu, G.GmlTetrahedra, 1, G.GmlFlt, b"Rsd")
    nbs = G.lib.GmlNewSolutionData(gpu, G.GmlTetrahedra, 1, G.GmlFlt4, b"NbSum")
    wide = G.lib.GmlNewSolutionData(gpu, G.GmlTetrahedra, 1, G.GmlDbl, b"Wide")
    assert min(sol, mid, rsd, nbs, wide) > 0
    assert G.set_data(gpu, sol, np.full((nv, 2, 4), 0.125, np.float32)) == 1
    assert G.set_data(gpu, wide, np.linspace(0.0, 1.0, nt)) == 1
    Rd, Wr = G.GmlReadMode, G.GmlWriteMode
    kw = G.compile_kernel(gpu, body("ex_wide.cl"), "wide", G.GmlTetrahedra, [(wide, Rd, 0)])
    kn = G.compile_kernel(gpu, body("ex_neighbour_sum.cl"), "neighbour_sum", G.GmlTetrahedra,
                          [(mid, Rd, ngb), (nbs, Wr, 0)])
    kd = G.compile_kernel(gpu, body("ex_downlink.cl"), "downlink", G.GmlTetrahedra,
                          [(v, Rd | G.GmlRefFlag, 0), (sol, Rd, 0), (rsd, Wr, 0), (mid, Wr, 0)])
    ku = G.compile_kernel(gpu, body("ex_uplink.cl"), "uplink", G.GmlVertices,
                          [(sol, Wr, 0), (mid, Rd | G.GmlVoyeurs, 0)])
    assert min(kw, kn, kd, ku) > 0
    links = G.get_data(gpu, ngb, np.int32, (nt, 4))
    for it in range(1, len(r["ft_mid"]) + 1):
        ctypes.memmove(p + 4, np.float32(it).tobytes(), 4)      # GmlPar->res
        assert G.lib.GmlUploadParameters(gpu) == 1
        before = G.get_data(gpu, mid, np.float32, (nt, 4))
        for k in (kw, kn, kd, ku):
            assert G.lib.GmlLaunchKernel(gpu, k) == 1
        red = ctypes.c_double()
        assert G.lib.GmlReduceVector(gpu, rsd, G.GmlSum, ctypes.byref(red)) == 1
        assert red.value == pytest.approx(r["ft_red_exact"][it - 1], rel=1e-6)
        m = G.get_data(gpu, mid, np.float32, (nt, 4))
        s = G.get_data(gpu, sol, np.float32, (nv, 2, 4))
        assert close(m, r["ft_mid"][it - 1], 2e-6), it
        assert close(s, r["ft_sol"][it - 1], 1e-5), it
        # the neighbour kernel ran before this iteration's downlink: it saw
        # the previous Mid; a boundary face (link 0) reads the null value
        nb = G.get_data(gpu, nbs, np.float32, (nt, 4))
        want = np.zeros((nt, 4), np.float32)
        for j in range(4):
            want = want + np.where((links[:, j] != 0)[:, None], before[links[:, j]], 0.0).astype(np.float32)
        assert close(nb, want, 1e-6), it
    assert np.array_equal(G.get_data(gpu, rsd, np.float32, nt), r["ft_res"])


def test_ball_quality_flow(G, gpu):
    r = fixture()
    crd, tri = r["sq_crd"], r["sq_tri"]
    nv, ntri = len(crd), len(tri)
    G.lib.GmlNewParameters(gpu, 8, PARAMS)
    v = G.lib.GmlNewMeshData(gpu, G.GmlVertices, nv)
    tr = G.lib.GmlNewMeshData(gpu, G.GmlTriangles, ntri)
    assert v > 0 and tr > 0
    IP = ctypes.POINTER(ctypes.c_int)
    c = np.ascontiguousarray(crd, np.float32)
    a = np.ascontiguousarray(tri, np.int32)
    rv, rt = np.zeros(nv, np.int32), np.zeros(ntri, np.int32)
    for typ, arr, ref, n in ((G.GmlVertices, c, rv, nv), (G.GmlTriangles, a, rt, ntri)):
        assert G.lib.GmlSetDataBlock(gpu, typ, 0, n - 1, ctypes.c_void_p(arr.ctypes.data),
                                     ctypes.c_void_p(arr.ctypes.data + (n - 1) * arr.strides[0]),
                                     ref.ctypes.data_as(IP),
                                     ctypes.cast(ref.ctypes.data + (n - 1) * 4, IP)) == 1
    tq = G.lib.GmlNewSolutionData(gpu, G.GmlTriangles, 1, G.GmlFlt, b"TriQ")
    vq = G.lib.GmlNewSolutionData(gpu, G.GmlVertices, 1, G.GmlFlt, b"vq")
    tqb = G.lib.GmlNewSolutionData(gpu, G.GmlTriangles, 1, G.GmlFlt, b"tq")
    Rd, Wr = G.GmlReadMode, G.GmlWriteMode
    k1 = G.compile_kernel(gpu, body("ex_tri_quality.cl"), "triqal", G.GmlTriangles,
                          [(v, Rd, 0), (tq, Wr, 0)])
    assert k1 > 0 and G.lib.GmlLaunchKernel(gpu, k1) == 1
    q = G.get_data(gpu, tq, np.float32, ntri)
    assert close(q, r["bq_tq"], 2e-6)
    # the ball minimum over the triangles of each vertex (runtime degree),
    # on the qualities as computed here
    assert G.set_data(gpu, tqb, q) == 1
    k2 = G.compile_kernel(gpu, body("ball_min.cl"), "verqal", G.GmlVertices,
                          [(tr, Rd, 0), (tqb, Rd, 0), (vq, Wr, 0)])
    assert k2 > 0 and G.lib.GmlLaunchKernel(gpu, k2) == 1
    got = G.get_data(gpu, vq, np.float32, nv)
    exp = np.full(nv, np.inf, np.float32)
    np.minimum.at(exp, tri.ravel(), np.repeat(q, 3))
    assert np.array_equal(got, exp)
    assert close(got, r["bq_vq"], 2e-6)
