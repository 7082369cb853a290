"""Whole-datatype transfers (GmlxSetData / GmlxGetData): the direct path
(one kernel writing the destination and the host mirror) and the staged
path (host copy into the mirror, DMA) give the same device data and the
same mirror, which the line accessors read."""
import ctypes
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def instance(G, direct):
    old = os.environ.get("GML_DIRECT")
    os.environ["GML_DIRECT"] = "1" if direct else "0"
    try:
        g = G.lib.GmlInit(0)
    finally:
        if old is None:
            del os.environ["GML_DIRECT"]
        else:
            os.environ["GML_DIRECT"] = old
    assert g
    return g


def line(G, g, idx, lin):
    """Vertex line lin through the reference accessor (reads the mirror for
    lin > 0; line 0 downloads first)."""
    x, y, z = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    ref = ctypes.c_int()
    assert G.lib.GmlGetDataLine(ctypes.c_size_t(g), ctypes.c_int(idx), ctypes.c_int(lin),
                                ctypes.byref(x), ctypes.byref(y), ctypes.byref(z),
                                ctypes.byref(ref)) == 1
    return x.value, y.value, z.value


@pytest.mark.parametrize("direct", [True, False])
@pytest.mark.parametrize("offset", [0, 4])
def test_set_get_round_trip(G, direct, offset):
    nv = 300_001                                   # 4.8 MB of float4 lines: above the direct threshold
    rng = np.random.default_rng(7)
    store = np.zeros(nv * 4 + 4, np.float32)       # offset 4 bytes: unaligned source, staged path
    crd = store[offset // 4: offset // 4 + nv * 4].reshape(nv, 4)
    crd[:, :3] = rng.uniform(-1, 1, (nv, 3))
    g = instance(G, direct)
    try:
        v = G.lib.GmlNewMeshData(g, G.GmlVertices, nv)
        assert v and G.lib.GmlxSetData(g, v, crd.ctypes.data, crd.nbytes) == 1
        # the mirror holds what was set: line 7 is read from it without a
        # download (line 0 downloads first)
        assert line(G, g, v, 7) == tuple(float(c) for c in crd[7, :3])
        assert line(G, g, v, 0) == tuple(float(c) for c in crd[0, :3])
        out = np.zeros_like(crd)
        assert G.lib.GmlxGetData(g, v, out.ctypes.data, out.nbytes) == 1
        assert np.array_equal(out, crd)
    finally:
        G.lib.GmlStop(g)


def test_get_refreshes_the_mirror(G):
    """After a kernel changes the device data, GmlxGetData on either path
    leaves the mirror equal to the downloaded data (as a download does).
    48^3 hexes: 117,649 vertices, 1.9 MB, above the direct path's 1 MB."""
    n = 48
    crd, tet, ref = G.cube_mesh(n, split=1, jitter=0.3, seed=3)
    res = []
    for direct in (True, False):
        g = instance(G, direct)
        try:
            v, t = G.upload_mesh(g, crd, tet, ref)
            assert G.lib.GmlxMeshSetup(g, 1) == 1
            assert G.lib.GmlxSmooth(g, 3, ctypes.c_float(1.0)) == 1
            out = np.zeros_like(crd)
            assert G.lib.GmlxGetData(g, v, out.ctypes.data, out.nbytes) == 1
            assert not np.array_equal(out, crd)          # the sweeps moved interior vertices
            k = int(np.argmax(np.abs(out - crd).sum(axis=1)))
            assert line(G, g, v, k) == tuple(float(c) for c in out[k, :3])
            res.append(out)
        finally:
            G.lib.GmlStop(g)
    assert np.array_equal(res[0], res[1])


def test_new_mirrors_start_zeroed(G):
    """A datatype created after another instance used and freed the same
    amount of pinned host memory still reads as zeros, as the reference's
    calloc'd mirrors do."""
    nv = 200_000                                   # 3.2 MB: a pinned mirror
    crd = np.full((nv, 4), 7.0, np.float32)
    g = instance(G, True)
    g2 = instance(G, True)                         # a second instance stays alive meanwhile
    try:
        v = G.lib.GmlNewMeshData(g, G.GmlVertices, nv)
        assert G.lib.GmlxSetData(g, v, crd.ctypes.data, crd.nbytes) == 1
        G.lib.GmlStop(g)
        g = instance(G, True)
        v = G.lib.GmlNewMeshData(g, G.GmlVertices, nv)
        assert line(G, g, v, 5) == (0.0, 0.0, 0.0)      # the mirror, not downloaded
        out = np.ones_like(crd)
        assert G.lib.GmlxGetData(g, v, out.ctypes.data, out.nbytes) == 1
        assert not out.any()
    finally:
        G.lib.GmlStop(g)
        G.lib.GmlStop(g2)


def test_mirror_after_get_is_the_read_data(G):
    """GmlxGetData on the direct path refreshes the host mirror at the next
    call on the instance.  The mirror still holds the data of the read when
    a kernel changes the device data before the line accessor looks (the
    kernel's launch refreshes it first), and holds the new data when
    GmlxSetData rewrites the datatype in between (1.9 MB of vertices, so
    the transfers take the direct path)."""
    n = 48
    crd, tet, ref = G.cube_mesh(n, split=1, jitter=0.3, seed=4)
    g = instance(G, True)
    try:
        v, t = G.upload_mesh(g, crd, tet, ref)
        assert G.lib.GmlxMeshSetup(g, 1) == 1
        assert G.lib.GmlxSmooth(g, 2, ctypes.c_float(1.0)) == 1
        first = np.zeros_like(crd)
        assert G.lib.GmlxGetData(g, v, first.ctypes.data, first.nbytes) == 1
        # two reads in a row keep the same data
        again = np.zeros_like(crd)
        assert G.lib.GmlxGetData(g, v, again.ctypes.data, again.nbytes) == 1
        assert np.array_equal(first, again)
        # the sweeps change the device data; the mirror keeps the read
        assert G.lib.GmlxSmooth(g, 2, ctypes.c_float(1.0)) == 1
        now = np.zeros_like(crd)
        assert G.lib.GmlxGetData(g, v, now.ctypes.data, now.nbytes) == 1
        assert not np.array_equal(now, first)
        assert G.lib.GmlxSmooth(g, 1, ctypes.c_float(1.0)) == 1
        k = int(np.argmax(np.abs(now - first).sum(axis=1)))
        assert line(G, g, v, k) == tuple(float(c) for c in now[k, :3])
        # a read, then a whole rewrite: the mirror holds the rewrite
        assert G.lib.GmlxGetData(g, v, now.ctypes.data, now.nbytes) == 1
        new = np.ascontiguousarray(crd * np.float32(0.5))
        assert G.lib.GmlxSetData(g, v, new.ctypes.data, new.nbytes) == 1
        assert line(G, g, v, k) == tuple(float(c) for c in new[k, :3])
        back = np.zeros_like(crd)
        assert G.lib.GmlxGetData(g, v, back.ctypes.data, back.nbytes) == 1
        assert np.array_equal(back, new)
    finally:
        G.lib.GmlStop(g)
