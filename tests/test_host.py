"""Host-side data paths on an offline instance (no GPU): whole-datatype
copies in and out of the host mirrors, large enough to take the
multi-threaded copy path, and their size checks."""
import numpy as np
import pytest


@pytest.fixture
def offline(G):
    g = G.lib.GmlxInitOffline()
    assert g
    yield g
    G.lib.GmlStop(g)


@pytest.mark.parametrize("nv", [3, 1000, 700_001])      # 700k x 16 B > 8 MB
def test_set_get_round_trip(G, offline, nv):
    v = G.lib.GmlNewMeshData(offline, G.GmlVertices, nv)
    assert v > 0
    x = np.random.default_rng(nv).standard_normal((nv, 4)).astype(np.float32)
    assert G.set_data(offline, v, x) == 1
    y = G.get_data(offline, v, np.float32, (nv, 4))
    assert np.array_equal(x, y)


def test_size_mismatch_is_rejected(G, offline):
    v = G.lib.GmlNewMeshData(offline, G.GmlVertices, 10)
    x = np.zeros((9, 4), np.float32)
    assert G.set_data(offline, v, x) == 0
    with pytest.raises(RuntimeError):
        G.get_data(offline, v, np.float32, (11, 4))
