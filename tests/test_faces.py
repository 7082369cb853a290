"""GmlExtractFaces against the oracle's restatement of the reference
(bit-exact, offline instances): tet cubes with and without existing surface
triangles, and a hexahedral grid (quadrilateral faces)."""
import ctypes

import numpy as np
import pytest


def datatype(G, g, typ, width):
    nl, di = ctypes.c_int(), ctypes.c_int()
    if G.lib.GmlGetMeshInfo(g, typ, ctypes.byref(nl), ctypes.byref(di)) != 1 or nl.value == 0:
        return np.zeros((0, width), np.int32), np.zeros(0, np.int32)
    nodes = G.get_data(g, di.value, np.int32, (nl.value, 4 if width <= 4 else 8))[:, :width]
    return nodes, None


def set_elements(G, g, typ, nodes, refs):
    n, k = nodes.shape
    idx = G.lib.GmlNewMeshData(g, typ, n)
    assert idx > 0
    w = {2: 4, 3: 4, 4: 4, 7: 8}[typ]
    pad = np.zeros((n, w), np.int32)
    pad[:, :k] = nodes
    refs = np.ascontiguousarray(refs, np.int32)
    base = pad.ctypes.data
    IP = ctypes.POINTER(ctypes.c_int)
    rc = G.lib.GmlSetDataBlock(g, typ, 0, n - 1, ctypes.c_void_p(base),
                               ctypes.c_void_p(base + (n - 1) * pad.strides[0]),
                               refs.ctypes.data_as(IP), ctypes.cast(refs.ctypes.data + (n - 1) * 4, IP))
    assert rc == 1
    return pad


def hex_grid(n):
    m = n + 1
    vid = lambda i, j, k: i + m * (j + m * k)   # noqa: E731
    hexes = []
    for k in range(n):
        for j in range(n):
            for i in range(n):
                hexes.append([vid(i, j, k), vid(i + 1, j, k), vid(i + 1, j + 1, k), vid(i, j + 1, k),
                              vid(i, j, k + 1), vid(i + 1, j, k + 1), vid(i + 1, j + 1, k + 1),
                              vid(i, j + 1, k + 1)])
    return m ** 3, np.array(hexes, np.int32)


def refs_of(G, g, typ, n):
    # the reference datatype follows its element datatype in the slot table
    nl, di = ctypes.c_int(), ctypes.c_int()
    G.lib.GmlGetMeshInfo(g, typ, ctypes.byref(nl), ctypes.byref(di))
    return G.get_data(g, di.value + 1, np.int32, (n,))


@pytest.mark.parametrize("n,split", [(2, 0), (3, 1)])
def test_tet_faces(G, O, n, split):
    crd, tet, ref = G.cube_mesh(n, split=split, jitter=0.0, seed=1)
    g = G.lib.GmlxInitOffline()
    try:
        G.upload_mesh(g, crd, tet, ref)
        cnt = G.lib.GmlExtractFaces(g)
        tri, _ = O.extract_faces({4: (tet, np.zeros(len(tet)))})
        assert cnt == len(tri) == 2 * len(tet) + 6 * n * n
        got, _ = datatype(G, g, 2, 3)
        assert np.array_equal(got, tri[:, :3])
        assert np.array_equal(refs_of(G, g, 2, len(tri)), tri[:, 3])
    finally:
        G.lib.GmlStop(g)


def test_existing_surface_triangles_come_first(G, O):
    crd, tet, ref = G.cube_mesh(2, split=1, jitter=0.0, seed=1)
    g = G.lib.GmlxInitOffline()
    try:
        G.upload_mesh(g, crd, tet, ref)
        # some tet faces as surface triangles, unsorted, one duplicated, refs 7..
        surf = np.array([tet[0][[1, 2, 3]], tet[5][[2, 0, 3]], tet[0][[3, 2, 1]]], np.int32)
        srefs = np.array([7, 8, 9], np.int32)
        set_elements(G, g, 2, surf, srefs)
        cnt = G.lib.GmlExtractFaces(g)
        tri, _ = O.extract_faces({2: (surf, srefs), 4: (tet, np.zeros(len(tet)))})
        assert cnt == len(tri)
        got, _ = datatype(G, g, 2, 3)
        assert np.array_equal(got, tri[:, :3])
        r = refs_of(G, g, 2, len(tri))
        assert list(r[:2]) == [7, 8] and np.array_equal(r, tri[:, 3])
    finally:
        G.lib.GmlStop(g)


def test_hex_faces(G, O):
    nv, hexes = hex_grid(2)
    g = G.lib.GmlxInitOffline()
    try:
        G.lib.GmlNewMeshData(g, G.GmlVertices, nv)
        set_elements(G, g, 7, hexes, np.arange(len(hexes)))
        cnt = G.lib.GmlExtractFaces(g)
        _, qad = O.extract_faces({7: (hexes, np.arange(len(hexes)))})
        assert cnt == len(qad) == 3 * 2 * 2 * 3            # 3 n^2 (n + 1) faces
        got, _ = datatype(G, g, 3, 4)
        assert np.array_equal(got, qad[:, :4])
        assert np.all(refs_of(G, g, 3, len(qad)) == 0)
    finally:
        G.lib.GmlStop(g)
