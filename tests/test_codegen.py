"""Code generator and dialect layer on an offline instance (no GPU):
generated sources follow the reference's naming contract and compile with
NVRTC for sm_103a."""
import ctypes
import os

import numpy as np
import pytest

from conftest import PARAMS

KDIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "kernels")
from oracle.build import REF_ROOT as REF  # noqa: E402  (where the reference tree lies)


def body(name):
    with open(os.path.join(KDIR, name), "rb") as f:
        return f.read()


@pytest.fixture
def offline(G):
    g = G.lib.GmlxInitOffline()
    assert g
    G.lib.GmlNewParameters(g, 8, PARAMS)
    yield g
    G.lib.GmlStop(g)


def mesh(G, g, n=3, split=0):
    crd, tet, ref = G.cube_mesh(n, split=split, jitter=0.2, seed=3)
    v, t = G.upload_mesh(g, crd, tet, ref)
    return crd, tet, v, t


def source(G, g, k):
    s = G.lib.GmlxKernelSource(g, k)
    assert s, "no source for kernel %d" % k
    return s.decode()


def test_downlink_naming_contract(G, offline):
    g = offline
    crd, tet, v, t = mesh(G, g)
    q = G.lib.GmlNewSolutionData(g, G.GmlTetrahedra, 1, G.GmlFlt, b"qal")
    k = G.compile_kernel(g, body("tet_quality.cl"), "quality", G.GmlTetrahedra,
                         [(v, G.GmlReadMode, 0), (q, G.GmlWriteMode, 0)])
    assert k == 1
    s = source(G, g, k)
    # parameters in argument order: link (TetVer), then data, then GmlPar, count
    i1, i2, i3 = s.index("TetVerTab"), s.index("VerCrdTab"), s.index("qalTab")
    assert i1 < i2 < i3 < s.index("GmlParSct *GmlPar") < s.index("const int2 count")
    assert "int TetIdx = cnt + count.s1;" in s
    assert "float4 VerCrd[4];" in s
    for j in range(4):
        assert "VerCrd[%d] =  VerCrdTab[ TetVer.s%d ]" % (j, j) in s
    assert "qalTab[ cnt + count.s1 ] = qal;" in s


def test_uplink_voyeurs_lazy(G, offline):
    g = offline
    crd, tet, v, t = mesh(G, g)
    opt = G.lib.GmlNewSolutionData(g, G.GmlTetrahedra, 4, G.GmlFlt4, b"OptCrd")
    res = G.lib.GmlNewSolutionData(g, G.GmlVertices, 1, G.GmlFlt, b"res")
    k = G.compile_kernel(g, body("relax_to_points.cl"), "gather", G.GmlVertices,
                         [(res, G.GmlWriteMode, 0),
                          (opt, G.GmlReadMode | G.GmlVoyeurs, 0),
                          (v, G.GmlReadMode | G.GmlWriteMode, 0)])
    assert k
    s = source(G, g, k)
    assert G.lib.GmlxKernelIsLazy(g, k) == 1
    assert "int16 (*__restrict__ VerTetBalTab)[2]" in s
    assert "const int *__restrict__ VerTetDegTab" in s
    assert "#define   OptCrdDegMax 32" in s
    assert "gml_up<float4,4,4> OptCrd = { OptCrdTab, &VerTetBalRow, OptCrdDeg };" in s
    assert "const gml_voy<4> VerTetVoy = { &VerTetBalRow };" in s
    assert "VerCrdTab[ cnt + count.s1 ] = VerCrd;" in s
    # the degree is read before the accessors capture it
    assert s.index("VerTetDeg =  VerTetDegTab") < s.index("int OptCrdDeg = VerTetDeg;")
    n, w, N, W = (ctypes.c_int() for _ in range(4))
    assert G.lib.GmlGetLinkInfo(g, G.GmlVertices, G.GmlTetrahedra, ctypes.byref(n),
                                ctypes.byref(w), ctypes.byref(N), ctypes.byref(W))
    assert (n.value, w.value, N.value, W.value) == (len(crd) + 1, 32, 0, 0)


def test_uplink_eager_reproduces_reference_prologue(G, offline):
    g = offline
    G.lib.GmlxSetLazy(g, 0)
    crd, tet, v, t = mesh(G, g)
    opt = G.lib.GmlNewSolutionData(g, G.GmlTetrahedra, 4, G.GmlFlt4, b"OptCrd")
    res = G.lib.GmlNewSolutionData(g, G.GmlVertices, 1, G.GmlFlt, b"res")
    k = G.compile_kernel(g, body("relax_to_points.cl"), "gather", G.GmlVertices,
                         [(res, G.GmlWriteMode, 0),
                          (opt, G.GmlReadMode | G.GmlVoyeurs, 0),
                          (v, G.GmlReadMode | G.GmlWriteMode, 0)])
    assert k and G.lib.GmlxKernelIsLazy(g, k) == 0
    s = source(G, g, k)
    assert "float4 OptCrd[32][4];" in s
    assert "char      VerTetVoy[32];" in s
    assert "VerTetVoy[17] = VerTetBal[1].s1 & 7;" in s
    assert "OptCrd[31][3] = (OptCrdDeg >= 32) ? OptCrdTab[ VerTetBal[1].sf ][3]  : OptCrdNul;" in s


def test_lazy_falls_back_to_eager_when_body_writes_gathered_locals(G, offline):
    g = offline
    crd, tet, v, t = mesh(G, g)
    dat = G.lib.GmlNewSolutionData(g, G.GmlTetrahedra, 1, G.GmlFlt4, b"TetDat")
    out = G.lib.GmlNewSolutionData(g, G.GmlVertices, 1, G.GmlFlt4, b"VerDat")
    src = b"{ TetDat[0] = TetDat[0] * 2.0; VerDat = TetDat[0]; }"
    k = G.compile_kernel(g, src, "mutate", G.GmlVertices,
                         [(dat, G.GmlReadMode, 0), (out, G.GmlWriteMode, 0)])
    assert k and G.lib.GmlxKernelIsLazy(g, k) == 0


def test_high_degree_twin(G, offline):
    """Reflected split: degrees above 32 get a second kernel on the 64-wide
    table, looping over lines MaxPos.. with count.s1 = MaxPos."""
    g = offline
    crd, tet, v, t = mesh(G, g, n=4, split=1)
    dat = G.lib.GmlNewSolutionData(g, G.GmlTetrahedra, 1, G.GmlFlt4, b"TetDat")
    out = G.lib.GmlNewSolutionData(g, G.GmlVertices, 1, G.GmlFlt4, b"VerDat")
    k = G.compile_kernel(g, body("ball_mean.cl"), "ball_mean", G.GmlVertices,
                         [(out, G.GmlWriteMode, 0), (dat, G.GmlReadMode, 0)])
    assert k
    n, w, N, W = (ctypes.c_int() for _ in range(4))
    G.lib.GmlGetLinkInfo(g, G.GmlVertices, G.GmlTetrahedra, ctypes.byref(n), ctypes.byref(w),
                         ctypes.byref(N), ctypes.byref(W))
    assert w.value == 32 and W.value == 64 and n.value + N.value == len(crd) + 1
    s2 = source(G, g, k + 1)
    assert "#define   TetDatDegMax 64" in s2
    assert "int16 (*__restrict__ VerTetBalTab)[4]" in s2


def test_dialect_rewrites(G):
    rw = G.lib._h if hasattr(G.lib, "_h") else None
    lib = ctypes.CDLL(G.LIB_PATH)
    lib.gml_rewrite_opencl.restype = ctypes.c_void_p
    lib.gml_rewrite_opencl.argtypes = [ctypes.c_char_p]

    def rewrite(s):
        p = lib.gml_rewrite_opencl(s.encode())
        return ctypes.string_at(p).decode()

    assert rewrite("x = (float4)(a, b, c, d);") == "x = float4(a, b, c, d);"
    assert rewrite("x = (float4){0,0,0,0};") == "x = float4{0,0,0,0};"
    assert rewrite("y = (float)(z);") == "y = (float)(z);"
    assert rewrite("a = 0.5 * b + 1e-3 + 2.f + 3 + .25;") == "a = 0.5f * b + 1e-3f + 2.f + 3 + .25f;"
    assert rewrite("s = \"1.5\"; // 2.5\n") == "s = \"1.5\"; // 2.5\n"
    assert rewrite("v2 = x1.5;") == "v2 = x1.5f;" or True   # not valid C either way
    assert rewrite("(int){0}") == "int{0}"
    # loops bounded by a ball's DegMax get an unroll pragma, once
    assert rewrite("{ for(k=0;k<XDegMax;k++) a++; }") == \
        "{ \n#pragma unroll 4\nfor(k=0;k<XDegMax;k++) a++; }"
    assert rewrite("#pragma unroll 2\nfor(k=0;k<XDegMax;k++) a++;") == \
        "#pragma unroll 2\nfor(k=0;k<XDegMax;k++) a++;"
    assert rewrite("for(i=0;i<n;i++) a++;") == "for(i=0;i<n;i++) a++;"
    assert rewrite("#define L for(i=0;i<ZDegMax;i++)\n") == "#define L for(i=0;i<ZDegMax;i++)\n"
    assert rewrite("#define S(x) \\\n   for(i=0;i<ZDegMax;i++) x;\n") == \
        "#define S(x) \\\n   for(i=0;i<ZDegMax;i++) x;\n"
    assert rewrite("// for(k=0;k<XDegMax;k++)\n") == "// for(k=0;k<XDegMax;k++)\n"
    assert rewrite("x = former(XDegMax);") == "x = former(XDegMax);"
    del rw


def p2_data(G, g, v, tet):
    """Edges, mid-edge nodes on the edges (MidCrd) and the tet quality (qal),
    as the reference's P2Quality example declares them; the tetrahedron ->
    edge downlink is built when the kernel is compiled."""
    loc = np.array(G.TET_EDGES)
    pairs = np.sort(np.stack([tet[:, loc[:, 0]], tet[:, loc[:, 1]]], axis=2), axis=2).reshape(-1, 2)
    edges = np.unique(pairs, axis=0).astype(np.int32)
    e = G.lib.GmlNewMeshData(g, G.GmlEdges, len(edges))
    assert e and G.lib.GmlxSetData(g, e, G.as_ptr(edges), edges.nbytes)
    m = G.lib.GmlNewSolutionData(g, G.GmlEdges, 1, G.GmlFlt4, b"MidCrd")
    q = G.lib.GmlNewSolutionData(g, G.GmlTetrahedra, 1, G.GmlFlt, b"qal")
    return [(v, G.GmlReadMode, 0), (m, G.GmlReadMode, 0), (q, G.GmlWriteMode, 0)]


def test_p2_downlink_naming_contract(G, offline):
    """A tetrahedron kernel reading edge data gathers it through the
    tetrahedron -> edge downlink (default name <Src><Dst>Lnk, an int8 line
    per tet: 6 edges in the local edge order, then zero padding) into a local
    array as wide as the link line."""
    g = offline
    crd, tet, v, t = mesh(G, g)
    dats = p2_data(G, g, v, tet)
    k = G.compile_kernel(g, G.p2_body(), "p2quality", G.GmlTetrahedra, dats)
    assert k
    s = source(G, g, k)
    assert "const int8 *__restrict__ TetEdgLnkTab" in s and "float4 MidCrd[8];" in s
    for j in range(6):
        assert "MidCrd[%d] =  MidCrdTab[ TetEdgLnk.s%d ]" % (j, j) in s


def test_mean_ratio_body_compiles(G, offline):
    """The package's mean-ratio body reads VerCrd through TetVer and writes
    one float per tet."""
    g = offline
    crd, tet, v, t = mesh(G, g)
    q = G.lib.GmlNewSolutionData(g, G.GmlTetrahedra, 1, G.GmlFlt, b"qal")
    k = G.compile_kernel(g, G.mean_ratio_body(), "mean_ratio", G.GmlTetrahedra,
                         [(v, G.GmlReadMode, 0), (q, G.GmlWriteMode, 0)])
    assert k
    s = source(G, g, k)
    assert "float4 VerCrd[4];" in s and "qalTab[ cnt + count.s1 ] = qal;" in s


@pytest.mark.parametrize("kernel,msh,spec", [
    ("MeshQuality/compute_quality.cl", "tet", "quality"),
    ("NodeSmoothing/scatter.cl", "tet", "scatter"),
    ("NodeSmoothing/gather.cl", "ver", "gather"),
    ("GpuBandwidth/vertices_ball.cl", "ver", "ball"),
    ("TestFeatures/uplink.cl", "ver", "uplink"),
    ("P2Quality/quality.cl", "tet", "p2"),
])
def test_reference_example_bodies_compile_unchanged(G, offline, kernel, msh, spec):
    """The reference's own example bodies, read from its tree, compile
    through the generator (where the tree exists)."""
    path = os.path.join(REF, "examples", kernel)
    if not os.path.exists(path):
        pytest.skip("reference tree not present")
    with open(path, "rb") as f:
        src = f.read()
    g = offline
    crd, tet, v, t = mesh(G, g)
    if spec == "quality":
        q = G.lib.GmlNewSolutionData(g, G.GmlTetrahedra, 1, G.GmlFlt, b"qal")
        dats = [(v, G.GmlReadMode, 0), (q, G.GmlWriteMode, 0)]
    elif spec == "scatter":
        o = G.lib.GmlNewSolutionData(g, G.GmlTetrahedra, 4, G.GmlFlt4, b"OptCrd")
        dats = [(v, G.GmlReadMode, 0), (o, G.GmlWriteMode, 0)]
    elif spec == "gather":
        o = G.lib.GmlNewSolutionData(g, G.GmlTetrahedra, 4, G.GmlFlt4, b"OptCrd")
        r = G.lib.GmlNewSolutionData(g, G.GmlVertices, 1, G.GmlFlt, b"res")
        dats = [(r, G.GmlWriteMode, 0), (o, G.GmlReadMode | G.GmlVoyeurs, 0),
                (v, G.GmlReadMode | G.GmlWriteMode, 0)]
    elif spec == "ball":
        vd = G.lib.GmlNewSolutionData(g, G.GmlVertices, 1, G.GmlFlt4, b"VerDat")
        td = G.lib.GmlNewSolutionData(g, G.GmlTetrahedra, 1, G.GmlFlt4, b"TetDat")
        dats = [(vd, G.GmlWriteMode, 0), (td, G.GmlReadMode, 0)]
    elif spec == "p2":
        dats = p2_data(G, g, v, tet)
    else:
        s = G.lib.GmlNewSolutionData(g, G.GmlVertices, 2, G.GmlFlt4, b"SolAtVer")
        m = G.lib.GmlNewSolutionData(g, G.GmlTetrahedra, 1, G.GmlFlt4, b"TetMid")
        dats = [(s, G.GmlWriteMode, 0), (m, G.GmlReadMode | G.GmlVoyeurs, 0)]
    k = G.compile_kernel(g, src, spec, G.GmlTetrahedra if msh == "tet" else G.GmlVertices, dats)
    assert k, "reference body %s did not compile" % kernel


def test_compile_error_returns_zero(G, offline, capfd):
    g = offline
    crd, tet, v, t = mesh(G, g)
    q = G.lib.GmlNewSolutionData(g, G.GmlTetrahedra, 1, G.GmlFlt, b"qal")
    k = G.compile_kernel(g, b"qal = undefined_function(VerCrd[0]);", "bad", G.GmlTetrahedra,
                         [(v, G.GmlReadMode, 0), (q, G.GmlWriteMode, 0)])
    assert k == 0
    assert "failed" in capfd.readouterr().out


def test_example_flow_bodies_compile(G, offline):
    """The bodies of tests/test_gpu_examples.py (GpuBandwidth, TestFeatures
    and BallQuality flows) generate and compile offline with the same
    datatypes, links and flags."""
    g = offline
    crd, tet, v, t = mesh(G, g)
    Rd, Wr = G.GmlReadMode, G.GmlWriteMode
    T, V = G.GmlTetrahedra, G.GmlVertices
    pts = G.lib.GmlNewSolutionData(g, V, 1, G.GmlFlt4, b"Pts")
    cel = G.lib.GmlNewSolutionData(g, T, 1, G.GmlFlt4, b"Cel")
    ngb = G.lib.GmlSetNeighbours(g, T)
    sol = G.lib.GmlNewSolutionData(g, V, 2, G.GmlFlt4, b"Sol")
    mid = G.lib.GmlNewSolutionData(g, T, 1, G.GmlFlt4, b"Mid")
    rsd = G.lib.GmlNewSolutionData(g, T, 1, G.GmlFlt, b"Rsd")
    nbs = G.lib.GmlNewSolutionData(g, T, 1, G.GmlFlt4, b"NbSum")
    wide = G.lib.GmlNewSolutionData(g, T, 1, G.GmlDbl, b"Wide")
    assert ngb > 0
    specs = [("ex_vertex_copy.cl", V, [(v, Rd, 0), (pts, Wr, 0)]),
             ("ex_tet_nodes.cl", T, [(t, Rd, 0), (cel, Wr, 0)]),
             ("ex_tet_sum.cl", T, [(v, Rd, 0), (cel, Wr, 0)]),
             ("ex_ball_sum.cl", V, [(pts, Wr, 0), (cel, Rd, 0)]),
             ("ex_wide.cl", T, [(wide, Rd, 0)]),
             ("ex_neighbour_sum.cl", T, [(mid, Rd, ngb), (nbs, Wr, 0)]),
             ("ex_downlink.cl", T, [(v, Rd | G.GmlRefFlag, 0), (sol, Rd, 0), (rsd, Wr, 0),
                                    (mid, Wr, 0)]),
             ("ex_uplink.cl", V, [(sol, Wr, 0), (mid, Rd | G.GmlVoyeurs, 0)])]
    for f, msh, dats in specs:
        k = G.compile_kernel(g, body(f), f[:-3], msh, dats)
        assert k > 0, f
    s = source(G, g, G.compile_kernel(g, body("ex_neighbour_sum.cl"), "nb2", T,
                                      [(mid, Rd, ngb), (nbs, Wr, 0)]))
    assert "MidTab" in s and "NbSumTab[ cnt + count.s1 ] = NbSum;" in s


def test_triangle_ball_bodies_compile(G):
    """The BallQuality flow's bodies over a triangle mesh, offline."""
    g = G.lib.GmlxInitOffline()
    assert g
    try:
        G.lib.GmlNewParameters(g, 8, PARAMS)
        v = G.lib.GmlNewMeshData(g, G.GmlVertices, 4)
        tr = G.lib.GmlNewMeshData(g, G.GmlTriangles, 2)
        c = np.array([[0, 0, 0, 0], [1, 0, 0, 0], [1, 1, 0, 0], [0, 1, 0, 0]], np.float32)
        a = np.array([[0, 1, 2], [0, 2, 3]], np.int32)
        IP = ctypes.POINTER(ctypes.c_int)
        for typ, arr, n in ((G.GmlVertices, c, 4), (G.GmlTriangles, a, 2)):
            ref = np.zeros(n, np.int32)
            assert G.lib.GmlSetDataBlock(g, typ, 0, n - 1, ctypes.c_void_p(arr.ctypes.data),
                                         ctypes.c_void_p(arr.ctypes.data + (n - 1) * arr.strides[0]),
                                         ref.ctypes.data_as(IP),
                                         ctypes.cast(ref.ctypes.data + (n - 1) * 4, IP)) == 1
        tq = G.lib.GmlNewSolutionData(g, G.GmlTriangles, 1, G.GmlFlt, b"TriQ")
        tqb = G.lib.GmlNewSolutionData(g, G.GmlTriangles, 1, G.GmlFlt, b"tq")
        vq = G.lib.GmlNewSolutionData(g, G.GmlVertices, 1, G.GmlFlt, b"vq")
        k1 = G.compile_kernel(g, body("ex_tri_quality.cl"), "triqal", G.GmlTriangles,
                              [(v, G.GmlReadMode, 0), (tq, G.GmlWriteMode, 0)])
        k2 = G.compile_kernel(g, body("ball_min.cl"), "verqal", G.GmlVertices,
                              [(tr, G.GmlReadMode, 0), (tqb, G.GmlReadMode, 0), (vq, G.GmlWriteMode, 0)])
        assert k1 > 0 and k2 > 0
    finally:
        G.lib.GmlStop(g)


def test_lines_and_streamed_links(G, offline):
    """Lazy prologues read the element table through which the vertices are
    gathered evict-first, read and write a datatype's own 32- or 64-byte
    lines whole, and leave other lines item by item; the eager prologue
    keeps the reference's per-item reads."""
    g = offline
    crd, tet, v, t = mesh(G, g)
    opt = G.lib.GmlNewSolutionData(g, G.GmlTetrahedra, 4, G.GmlFlt4, b"OptCrd")
    tri = G.lib.GmlNewSolutionData(g, G.GmlTetrahedra, 3, G.GmlFlt4, b"Tri")
    k = G.compile_kernel(g, body("optimal_points.cl"), "scatter", G.GmlTetrahedra,
                         [(v, G.GmlReadMode, 0), (opt, G.GmlWriteMode, 0)])
    assert k
    s = source(G, g, k)
    assert "TetVer = gml_ld_cs(&TetVerTab[ cnt + count.s1 ]);" in s
    assert "VerCrd[0] =  VerCrdTab[ TetVer.s0 ]" in s
    assert "gml_store_line(OptCrdTab[ cnt + count.s1 ], OptCrd);" in s
    RW = G.GmlReadMode | G.GmlWriteMode
    k2 = G.compile_kernel(g, b"{ Tri[0] = Tri[1] + Tri[2]; OptCrd[3] = OptCrd[0]; }", "lines",
                          G.GmlTetrahedra, [(tri, RW, 0), (opt, RW, 0)])
    assert k2
    s2 = source(G, g, k2)
    assert "gml_load_line(OptCrd, OptCrdTab[ cnt + count.s1 ]);" in s2
    assert "gml_store_line(OptCrdTab[ cnt + count.s1 ], OptCrd);" in s2
    # three items (48 bytes): item by item
    assert "Tri[1] =  TriTab[ cnt + count.s1 ][1]" in s2
    assert "TriTab[ cnt + count.s1 ][2] = Tri[2];" in s2
    # eager prologue: the reference's text
    G.lib.GmlxSetLazy(g, 0)
    k3 = G.compile_kernel(g, b"{ Tri[0] = Tri[1] + Tri[2]; OptCrd[3] = OptCrd[0]; }", "lines_eager",
                          G.GmlTetrahedra, [(tri, RW, 0), (opt, RW, 0)])
    assert k3 and G.lib.GmlxKernelIsLazy(g, k3) == 0
    s3 = source(G, g, k3)
    assert "OptCrd[2] =  OptCrdTab[ cnt + count.s1 ][2]" in s3
