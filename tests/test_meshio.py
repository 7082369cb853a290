"""Mesh files without libMeshb (offline instances, no GPU): write/read round
trips in both encodings, the reference's own sample meshes (where the
reference tree is present; the binary layout was checked against them),
and the ASCII solution writer."""
import ctypes
import lzma
import os

import numpy as np
import pytest

from oracle.build import REF_ROOT as REF  # noqa: E402  (where the reference tree lies)
KW_VER, KW_EDG, KW_TRI, KW_TET = 4, 5, 6, 8


@pytest.fixture
def inst(G):
    made = []

    def make():
        g = G.lib.GmlxInitOffline()
        assert g
        made.append(g)
        return g
    yield make
    for g in made:
        G.lib.GmlStop(g)


def read_back(G, g, typ, width, n, dtype):
    nl, di = ctypes.c_int(), ctypes.c_int()
    assert G.lib.GmlGetMeshInfo(g, typ, ctypes.byref(nl), ctypes.byref(di)) == 1
    assert nl.value == n
    return G.get_data(g, di.value, dtype, (n, width))


@pytest.mark.parametrize("ext", [".meshb", ".mesh"])
def test_round_trip(G, inst, tmp_path, ext):
    crd, tet, ref = G.cube_mesh(3, split=1, jitter=0.3, seed=8)
    g = inst()
    G.upload_mesh(g, crd, tet, ref)
    path = str(tmp_path / ("cube" + ext)).encode()
    types = (ctypes.c_int * 2)(G.GmlVertices, G.GmlTetrahedra)
    assert G.lib.GmlxExportMesh(g, path, 2, types) == 1
    h = inst()
    kw = (ctypes.c_int * 2)(KW_VER, KW_TET)
    assert G.lib.GmlxImportMesh(h, path, 2, kw) == 2
    c2 = read_back(G, h, G.GmlVertices, 4, len(crd), np.float32)
    t2 = read_back(G, h, G.GmlTetrahedra, 4, len(tet), np.int32)
    assert np.array_equal(c2[:, :3], crd[:, :3])
    assert np.array_equal(t2, tet)


def test_missing_file_and_bad_index(G, inst, tmp_path, capfd):
    g = inst()
    kw = (ctypes.c_int * 1)(KW_VER)
    assert G.lib.GmlxImportMesh(g, str(tmp_path / "none.meshb").encode(), 1, kw) == 0
    bad = tmp_path / "bad.mesh"
    bad.write_text("MeshVersionFormatted 2\nDimension 3\nVertices\n2\n0 0 0 0\n1 0 0 0\n"
                   "Edges\n1\n1 3 0\nEnd\n")
    kw2 = (ctypes.c_int * 2)(KW_VER, KW_EDG)
    assert G.lib.GmlxImportMesh(g, str(bad).encode(), 2, kw2) == 2
    assert "refers to vertex 3 of 2" in capfd.readouterr().out
    nl, di = ctypes.c_int(), ctypes.c_int()
    G.lib.GmlGetMeshInfo(g, G.GmlEdges, ctypes.byref(nl), ctypes.byref(di))
    assert nl.value == 0                      # the edges were not created


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "sample_meshes")),
                    reason="reference sample meshes not present")
@pytest.mark.parametrize("name,kw,typ,nv,ne,width", [
    ("edges", KW_EDG, 1, 202875, 1378058, 2),
    ("triangles", KW_TRI, 2, 181001, 362018, 4),
    ("naca012_2D_triangles", KW_TRI, 2, 36624, 72783, 4)])
def test_reference_sample_meshes(G, inst, tmp_path, name, kw, typ, nv, ne, width):
    raw = lzma.open(os.path.join(REF, "sample_meshes", name + ".meshb.xz")).read()
    path = tmp_path / (name + ".meshb")
    path.write_bytes(raw)
    g = inst()
    kws = (ctypes.c_int * 2)(KW_VER, kw)
    assert G.lib.GmlxImportMesh(g, str(path).encode(), 2, kws) == 2
    crd = read_back(G, g, G.GmlVertices, 4, nv, np.float32)
    ele = read_back(G, g, typ, width, ne, np.int32)
    nn = 2 if typ == 1 else 3
    assert ele[:, :nn].min() >= 0 and ele[:, :nn].max() < nv
    # every vertex of an edge/triangle mesh is used by some element
    assert len(np.unique(ele[:, :nn])) > 0.9 * nv
    # version-1 files store float32 coordinates: the first vertex is the
    # first 3 floats after the headers (code, version, dimension record,
    # vertex keyword, next position, count)
    dim = 2 if "2D" in name else 3
    first = np.frombuffer(raw[32:32 + 4 * dim], np.float32)
    assert np.array_equal(crd[0, :dim], first)
    if dim == 2:
        assert np.all(crd[:, 2] == 0)


def test_solution_ascii(G, inst, tmp_path):
    crd, tet, ref = G.cube_mesh(2, split=0, jitter=0.0, seed=1)
    g = inst()
    G.upload_mesh(g, crd, tet, ref)
    q = G.lib.GmlNewSolutionData(g, G.GmlTetrahedra, 1, G.GmlFlt, b"qal")
    vals = np.arange(len(tet), dtype=np.float32) / 7
    assert G.set_data(g, q, vals) == 1
    path = tmp_path / "q.sol"
    d = (ctypes.c_int * 1)(q)
    assert G.lib.GmlxExportSolution(g, str(path).encode(), 1, d) == 1
    words = path.read_text().split()
    k = words.index("SolAtTetrahedra")
    assert words[k + 1:k + 4] == [str(len(tet)), "1", "1"]
    got = np.array([float(w) for w in words[k + 4:k + 4 + len(tet)]], np.float32)
    assert np.array_equal(got, vals)


def read_solb(path):
    """A version-3 binary solution file: {keyword: (lines, types, values)}."""
    import struct
    b = path.read_bytes()
    code, ver = struct.unpack_from("<ii", b, 0)
    assert code == 1 and ver == 3
    pos, out = 8, {}
    while True:
        kwd, nxt = struct.unpack_from("<iq", b, pos)
        if kwd == 54:
            assert nxt == 0 and pos + 12 == len(b)
            return out
        if kwd == 3:
            out[3] = struct.unpack_from("<i", b, pos + 12)[0]
        else:
            nl, nf = struct.unpack_from("<ii", b, pos + 12)
            typ = np.frombuffer(b, np.int32, nf, pos + 20)
            val = np.frombuffer(b, np.float64, nl * nf, pos + 20 + 4 * nf).reshape(nl, nf)
            out[kwd] = (nl, typ, val)
        pos = nxt


def test_solution_binary(G, inst, tmp_path):
    """The .solb encoding: Dimension 3, one SolAtTetrahedra (66) keyword with
    one scalar field per float component (qal, then the 4 components of a
    float4 field) and SolAtVertices (62) for a vertex field, float64 values
    equal to the FP32 data."""
    crd, tet, ref = G.cube_mesh(2, split=1, jitter=0.1, seed=2)
    g = inst()
    G.upload_mesh(g, crd, tet, ref)
    q = G.lib.GmlNewSolutionData(g, G.GmlTetrahedra, 1, G.GmlFlt, b"qal")
    m = G.lib.GmlNewSolutionData(g, G.GmlTetrahedra, 1, G.GmlFlt4, b"mid")
    r = G.lib.GmlNewSolutionData(g, G.GmlVertices, 1, G.GmlFlt, b"res")
    qv = np.arange(len(tet), dtype=np.float32) / 3
    mv = np.random.default_rng(1).standard_normal((len(tet), 4)).astype(np.float32)
    rv = np.linspace(-1, 1, len(crd)).astype(np.float32)
    for idx, v in ((q, qv), (m, mv), (r, rv)):
        assert G.set_data(g, idx, v) == 1
    path = tmp_path / "s.solb"
    assert G.lib.GmlxExportSolution(g, str(path).encode(), 3, (ctypes.c_int * 3)(q, m, r)) == 2
    f = read_solb(path)
    assert f[3] == 3
    nl, typ, val = f[66]
    assert nl == len(tet) and list(typ) == [1] * 5
    assert np.array_equal(val, np.column_stack([qv, mv]).astype(np.float64))
    nl, typ, val = f[62]
    assert nl == len(crd) and list(typ) == [1] and np.array_equal(val[:, 0], rv.astype(np.float64))


@pytest.mark.gpu
def test_imported_mesh_on_the_gpu(G, inst, tmp_path):
    """A mesh read from a .meshb file gives the same quality statistics on
    the GPU as the same mesh uploaded directly."""
    crd, tet, ref = G.cube_mesh(6, split=1, jitter=0.3, seed=4)
    off = inst()
    G.upload_mesh(off, crd, tet, ref)
    path = str(tmp_path / "m.meshb").encode()
    assert G.lib.GmlxExportMesh(off, path, 2, (ctypes.c_int * 2)(G.GmlVertices, G.GmlTetrahedra)) == 1
    res = []
    for load in ("file", "direct"):
        g = G.lib.GmlInit(0)
        try:
            if load == "file":
                assert G.lib.GmlxImportMesh(g, path, 2, (ctypes.c_int * 2)(KW_VER, KW_TET)) == 2
            else:
                G.upload_mesh(g, crd, tet, ref)
            assert G.lib.GmlxMeshSetup(g, 1) == 1
            q = G.GmlxQuality()
            assert G.lib.GmlxSmooth(g, 2, ctypes.c_float(0.7)) == 1
            assert G.lib.GmlxQualityStats(g, 1.0 / 6, 0, ctypes.byref(q)) == 1
            res.append((q.MinQal, q.MinIdx, q.MaxQal, q.MaxIdx, tuple(q.Hist)))
        finally:
            G.lib.GmlStop(g)
    assert res[0] == res[1]
