"""GmlxReduceNoAlloc (scratch in static device memory, nothing allocated)
against GmlReduceVector on the same field, and against numpy in FP64,
through the C ABI; also on a field that starts 4 bytes past a 16-byte
boundary (the kernel's scalar path).

The file name sorts last so that the entry point also runs after every other
test of the session; it passes alone in a fresh process as well."""
import ctypes

import numpy as np
import pytest

OPS = range(7)          # GmlMin .. GmlLinf


def _field(G, g, x):
    idx = G.lib.GmlNewSolutionData(g, G.GmlVertices, 1, G.GmlFlt, b"x")
    assert idx > 0
    assert G.set_data(g, idx, x) == 1
    return idx


def _close(a, b, op):
    if op in (0, 1, 3, 6):
        return a == b                      # min, max, count, max |x|: exact
    return abs(a - b) <= 1e-9 * max(1.0, abs(b))


def _numpy(x, op):
    """The same reductions in FP64 (sums of FP32 values are exact in FP64
    up to rounding of the FP64 accumulation itself)."""
    d = x.astype(np.float64)
    return [d.min(), d.max(), d.sum(), float(np.count_nonzero(d)), np.abs(d).sum(),
            (d * d).sum(), np.abs(d).max()][op]


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 1000, 3_000_001])
def test_no_alloc_matches_reduce_vector(G, n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n).astype(np.float32)
    x[rng.integers(0, n, size=max(1, n // 7))] = 0.0
    g = G.lib.GmlInit(0)
    assert g
    try:
        G.lib.GmlNewMeshData(g, G.GmlVertices, n)
        idx = _field(G, g, x)
        dev = G.lib.GmlxDevicePtr(g, idx)
        stream = G.lib.GmlxStream(g)
        assert dev
        for op in OPS:
            want = ctypes.c_double()
            assert G.lib.GmlReduceVector(g, idx, op, ctypes.byref(want)) == 1
            exact = _numpy(x, op)
            assert _close(want.value, exact, op), (op, want.value, exact)
            for _ in range(2):                     # two calls in a row
                got = ctypes.c_double(12345.0)
                rc = G.lib.GmlxReduceNoAlloc(dev, n, op, ctypes.byref(got), stream)
                assert rc == 1
                assert _close(got.value, want.value, op), (op, got.value, want.value)
                assert _close(got.value, exact, op), (op, got.value, exact)
            if n > 1:
                # lines 1..n-1: 4 bytes past the 16-byte boundary
                got = ctypes.c_double()
                assert G.lib.GmlxReduceNoAlloc(ctypes.c_void_p(dev + 4), n - 1, op,
                                               ctypes.byref(got), stream) == 1
                assert _close(got.value, _numpy(x[1:], op), op), (op, "unaligned")
    finally:
        G.lib.GmlStop(g)


@pytest.mark.gpu
def test_no_alloc_rejects_and_identities(G, capfd):
    res = ctypes.c_double(7.0)
    too_many = (1 << 31)                           # above GMLX_NOALLOC_MAX_LINES
    assert G.lib.GmlxReduceNoAlloc(ctypes.c_void_p(16), too_many, 2, ctypes.byref(res), None) == 0
    assert "exceed the maximum" in capfd.readouterr().err
    assert res.value == 7.0
    assert G.lib.GmlxReduceNoAlloc(None, 10, 2, ctypes.byref(res), None) == 0
    assert G.lib.GmlxReduceNoAlloc(None, 0, 9, ctypes.byref(res), None) == 0
    assert G.lib.GmlxReduceNoAlloc(None, 0, 2, ctypes.byref(res), None) == 1
    assert res.value == 0.0
    assert G.lib.GmlxReduceNoAlloc(None, 0, 0, ctypes.byref(res), None) == 1
    assert res.value == float(np.finfo(np.float32).max)
