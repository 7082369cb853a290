"""Generated kernels on the GPU against the oracle: the MeshQuality,
NodeSmoothing and P2Quality flows of the reference (downlink gathers, ball
gather with voyeurs, high-degree twin kernels), reductions, argmin, ball
tables."""
import ctypes
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import PARAMS

pytestmark = pytest.mark.gpu

KDIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "kernels")
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def body(name):
    with open(os.path.join(KDIR, name), "rb") as f:
        return f.read()


def setup_mesh(G, g, crd, tet, ref):
    G.lib.GmlNewParameters(g, 8, PARAMS)
    return G.upload_mesh(g, crd, tet, ref)


def quality_gpu(G, g, v, nt):
    q = G.lib.GmlNewSolutionData(g, G.GmlTetrahedra, 1, G.GmlFlt, b"qal")
    k = G.compile_kernel(g, body("tet_quality.cl"), "quality", G.GmlTetrahedra,
                         [(v, G.GmlReadMode, 0), (q, G.GmlWriteMode, 0)])
    assert k
    assert G.lib.GmlLaunchKernel(g, k) == 1
    return q, G.get_data(g, q, np.float32, nt)


@pytest.mark.parametrize("n,split", [(32, 0), (20, 1)])
def test_quality_matches_oracle(G, O, gpu, n, split):
    crd, tet, ref = G.cube_mesh(n, split=split, jitter=0.25, seed=12345)
    v, t = setup_mesh(G, gpu, crd, tet, ref)
    q, qg = quality_gpu(G, gpu, v, len(tet))
    qo = O.quality_ref(crd, tet)
    # FP32 kernel vs FP64 oracle of the same formula
    assert np.max(np.abs(qg - qo)) <= 2e-5 * np.max(np.abs(qo))


@pytest.mark.parametrize("case", ["kuhn_n5.npz", "reflected_n6.npz"])
def test_quality_matches_golden(G, gpu, case):
    gd = dict(np.load(os.path.join(GOLD, case)))
    v, t = setup_mesh(G, gpu, gd["crd"], gd["tet"], gd["ref"])
    q, qg = quality_gpu(G, gpu, v, len(gd["tet"]))
    assert np.max(np.abs(qg - gd["quality"])) <= 2e-5 * np.max(np.abs(gd["quality"]))


def p2_quality_gpu(G, g, crd, tet, edges, mid):
    """The P2Quality flow: tets read vertex coordinates through TetVer and
    mid-edge nodes through the tetrahedron -> edge downlink."""
    G.lib.GmlNewParameters(g, 8, PARAMS)
    v, t, e, m = G.upload_p2(g, crd, tet, edges, mid)
    q = G.lib.GmlNewSolutionData(g, G.GmlTetrahedra, 1, G.GmlFlt, b"qal")
    k = G.compile_kernel(g, G.p2_body(), "p2quality", G.GmlTetrahedra,
                         [(v, G.GmlReadMode, 0), (m, G.GmlReadMode, 0), (q, G.GmlWriteMode, 0)])
    assert k
    assert G.lib.GmlLaunchKernel(g, k) == 1
    return q, G.get_data(g, q, np.float32, len(tet))


# FP32 kernel against the FP64 oracle: triple products of control-net vectors
# and square roots in FP32, fast_length / fast_distance
P2_ATOL, P2_RTOL = 2e-5, 2e-4


@pytest.mark.parametrize("n,split,curve", [(12, 0, 0.1), (9, 1, 0.2)])
def test_p2_quality_matches_oracle(G, O, gpu, n, split, curve):
    crd, tet, edges, mid, tedg = G.p2_mesh(n, split=split, jitter=0.2, curve=curve, seed=n)
    q, qg = p2_quality_gpu(G, gpu, crd, tet, edges, mid)
    qo = O.p2_quality(crd, mid, tet, tedg)
    assert np.all(np.abs(qg - qo) <= P2_ATOL + P2_RTOL * np.abs(qo))
    # the example's own reductions: mean and minimum of the tet qualities
    assert G.reduce(gpu, q, G.GmlSum) == pytest.approx(float(np.sum(qg, dtype=np.float64)),
                                                       rel=1e-12, abs=1e-12)
    assert G.reduce(gpu, q, G.GmlMin) == float(qg.min())


def test_p2_quality_matches_golden(G, gpu):
    """Against the reference's P2Quality body evaluated on the CPU."""
    gd = dict(np.load(os.path.join(GOLD, "p2_n5.npz")))
    q, qg = p2_quality_gpu(G, gpu, gd["crd"], gd["tet"], gd["edges"], gd["mid"])
    assert np.all(np.abs(qg - gd["quality"]) <= P2_ATOL + P2_RTOL * np.abs(gd["quality"]))


@pytest.mark.parametrize("n,split,jitter", [(32, 0, 0.25), (12, 1, 0.45)])
def test_mean_ratio_body_matches_oracle_and_native(G, O, gpu, n, split, jitter):
    """The mean-ratio dialect body against the FP64 oracle (signed by the
    FP64 determinant) and against the native quality pass: the same values
    within 2e-5, the same sign wherever the FP32 determinant is not within
    its rounding error of zero, and the same argmin when the minimum is
    isolated."""
    crd, tet, ref = G.cube_mesh(n, split=split, jitter=jitter, seed=n)
    v, t = setup_mesh(G, gpu, crd, tet, ref)
    q = G.lib.GmlNewSolutionData(gpu, G.GmlTetrahedra, 1, G.GmlFlt, b"qal")
    k = G.compile_kernel(gpu, G.mean_ratio_body(), "mean_ratio", G.GmlTetrahedra,
                         [(v, G.GmlReadMode, 0), (q, G.GmlWriteMode, 0)])
    assert k and G.lib.GmlLaunchKernel(gpu, k) == 1
    qg = G.get_data(gpu, q, np.float32, len(tet)).astype(np.float64)
    qo, _, _, _ = O.quality_stats(crd, tet)
    near_flat = np.abs(qo) < 1e-4
    assert np.all(np.abs(np.abs(qg) - np.abs(qo)) <= 2e-5)
    assert np.array_equal(np.sign(qg[~near_flat]), np.sign(qo[~near_flat]))
    assert G.lib.GmlxMeshSetup(gpu, 1) == 1
    res = G.GmlxQuality()
    assert G.lib.GmlxQualityStats(gpu, 1.0 / n, 0, ctypes.byref(res)) == 1
    srt = np.sort(qo)
    if srt[1] - srt[0] > 1e-4:
        fmin, imin, fmax, imax = ctypes.c_float(), ctypes.c_int(), ctypes.c_float(), ctypes.c_int()
        assert G.lib.GmlxReduceArg(gpu, q, ctypes.byref(fmin), ctypes.byref(imin),
                                   ctypes.byref(fmax), ctypes.byref(imax)) == 1
        assert imin.value == res.MinIdx == int(np.argmin(qo))


def test_reductions_match_oracle(G, O, gpu):
    crd, tet, ref = G.cube_mesh(32, split=0, jitter=0.25, seed=5)
    v, t = setup_mesh(G, gpu, crd, tet, ref)
    q, qg = quality_gpu(G, gpu, v, len(tet))
    for op in range(7):
        got = G.reduce(gpu, q, op)
        exp = O.reduce(op, qg)
        if op in (0, 1, 6):
            assert got == exp, op                    # exact
        else:
            assert abs(got - exp) <= 1e-12 * max(1.0, abs(exp)), op
    fmin, imin, fmax, imax = ctypes.c_float(), ctypes.c_int(), ctypes.c_float(), ctypes.c_int()
    assert G.lib.GmlxReduceArg(gpu, q, ctypes.byref(fmin), ctypes.byref(imin),
                               ctypes.byref(fmax), ctypes.byref(imax)) == 1
    assert imin.value == int(np.argmin(qg)) and fmin.value == qg.min()
    assert imax.value == int(np.argmax(qg)) and fmax.value == qg.max()


def test_reduction_ties_and_odd_sizes(G, O, gpu):
    """Ragged sizes (not multiples of any block) and ties: the smallest index
    wins, sums are not truncated (the reference drops the last partial
    group, sources/gmlib3.c:3299)."""
    for nt_hex in (1, 3, 7):
        crd, tet, ref = G.cube_mesh(nt_hex, split=0, jitter=0.0, seed=1)
        g = G.lib.GmlInit(0)
        try:
            G.lib.GmlNewParameters(g, 8, PARAMS)
            v, t = G.upload_mesh(g, crd, tet, ref)
            q = G.lib.GmlNewSolutionData(g, G.GmlTetrahedra, 1, G.GmlFlt, b"qal")
            x = np.ones(len(tet), np.float32)
            x[len(tet) // 2:] = 0.5
            G.set_data(g, q, x)
            assert G.reduce(g, q, G.GmlSum) == pytest.approx(float(x.sum(dtype=np.float64)), abs=0)
            fmin, imin = ctypes.c_float(), ctypes.c_int()
            G.lib.GmlxReduceArg(g, q, ctypes.byref(fmin), ctypes.byref(imin), None, None)
            assert imin.value == len(tet) // 2
        finally:
            G.lib.GmlStop(g)


@pytest.mark.parametrize("first", [-0.0, 0.0])
def test_argmin_signed_zero_ties(G, gpu, first):
    """A minimum of zero held by -0.0 and +0.0 at several lines: the smallest
    index wins whichever sign it carries (numpy's argmin agrees)."""
    crd, tet, ref = G.cube_mesh(7, split=0, jitter=0.0, seed=1)
    G.lib.GmlNewParameters(gpu, 8, PARAMS)
    G.upload_mesh(gpu, crd, tet, ref)
    q = G.lib.GmlNewSolutionData(gpu, G.GmlTetrahedra, 1, G.GmlFlt, b"qal")
    x = np.ones(len(tet), np.float32)
    x[1000], x[777], x[1500], x[2000] = -first, first, -0.0, 0.0
    x[10], x[2040] = 5.0, 5.0                          # ties at the maximum too
    G.set_data(gpu, q, x)
    fmin, imin, fmax, imax = ctypes.c_float(), ctypes.c_int(), ctypes.c_float(), ctypes.c_int()
    assert G.lib.GmlxReduceArg(gpu, q, ctypes.byref(fmin), ctypes.byref(imin),
                               ctypes.byref(fmax), ctypes.byref(imax)) == 1
    assert imin.value == 777 == int(np.argmin(x)) and fmin.value == 0.0
    assert imax.value == 10 == int(np.argmax(x)) and fmax.value == 5.0


def smoothing_step(G, g, v, nt, nv, lazy=1):
    G.lib.GmlxSetLazy(g, lazy)
    opt = G.lib.GmlNewSolutionData(g, G.GmlTetrahedra, 4, G.GmlFlt4, b"OptCrd")
    res = G.lib.GmlNewSolutionData(g, G.GmlVertices, 1, G.GmlFlt, b"res")
    ks = G.compile_kernel(g, body("optimal_points.cl"), "scatter", G.GmlTetrahedra,
                          [(v, G.GmlReadMode, 0), (opt, G.GmlWriteMode, 0)])
    kg = G.compile_kernel(g, body("relax_to_points.cl"), "gather", G.GmlVertices,
                          [(res, G.GmlWriteMode, 0), (opt, G.GmlReadMode | G.GmlVoyeurs, 0),
                           (v, G.GmlReadMode | G.GmlWriteMode, 0)])
    assert ks and kg
    assert G.lib.GmlxKernelIsLazy(g, kg) == lazy
    assert G.lib.GmlLaunchKernel(g, ks) == 1
    optg = G.get_data(g, opt, np.float32, (nt, 4, 4))
    assert G.lib.GmlLaunchKernel(g, kg) == 1
    newc = G.get_data(g, v, np.float32, (nv, 4))
    resg = G.get_data(g, res, np.float32, nv)
    return optg, newc, resg, res


@pytest.mark.parametrize("n,split,lazy", [(12, 0, 1), (10, 1, 1), (10, 1, 0)])
def test_node_smoothing_matches_oracle(G, O, gpu, n, split, lazy):
    crd, tet, ref = G.cube_mesh(n, split=split, jitter=0.3, seed=4242)
    v, t = setup_mesh(G, gpu, crd, tet, ref)
    optg, newc, resg, res = smoothing_step(G, gpu, v, len(tet), len(crd), lazy)
    opto = O.scatter(crd, tet)
    assert np.max(np.abs(optg - opto)) <= 2e-6
    deg, full = O.ball_codes(len(crd), tet)
    newo, reso = O.gather(crd, deg, full, opto)
    assert np.max(np.abs(newc - newo)) <= 2e-6
    assert np.max(np.abs(resg - reso)) <= 1e-8
    # residual reduction as in the NodeSmoothing driver
    assert G.reduce(gpu, res, G.GmlSum) == pytest.approx(reso.sum(), rel=1e-4)


@pytest.mark.parametrize("case", ["kuhn_n5.npz", "reflected_n6.npz"])
def test_ball_tables_bit_exact(G, O, gpu, case):
    gd = dict(np.load(os.path.join(GOLD, case)))
    crd, tet = gd["crd"], gd["tet"]
    v, t = setup_mesh(G, gpu, crd, tet, gd["ref"])
    smoothing_step(G, gpu, v, len(tet), len(crd))
    b, d, h = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    assert G.lib.GmlxLinkData(gpu, G.GmlVertices, G.GmlTetrahedra, ctypes.byref(b),
                              ctypes.byref(d), ctypes.byref(h)) == 1
    nb = G.lib.GmlxDataLines(gpu, b.value)
    base = G.get_data(gpu, b.value, np.int32, (nb, 32))
    deg = G.get_data(gpu, d.value, np.int32, len(crd))
    assert np.array_equal(deg, gd["deg"])
    assert np.array_equal(base, gd["base"])
    if int(gd["hghsiz"]):
        nh = G.lib.GmlxDataLines(gpu, h.value)
        high = G.get_data(gpu, h.value, np.int32, (nh, int(gd["hghsiz"])))
        assert np.array_equal(high, gd["high"])
    else:
        assert h.value == 0


def test_uplink_ball_mean_and_min(G, O, gpu):
    crd, tet, ref = G.cube_mesh(9, split=1, jitter=0.2, seed=8)
    v, t = setup_mesh(G, gpu, crd, tet, ref)
    td = G.lib.GmlNewSolutionData(gpu, G.GmlTetrahedra, 1, G.GmlFlt4, b"TetDat")
    vd = G.lib.GmlNewSolutionData(gpu, G.GmlVertices, 1, G.GmlFlt4, b"VerDat")
    kc = G.compile_kernel(gpu, body("tet_centroid.cl"), "centroid", G.GmlTetrahedra,
                          [(v, G.GmlReadMode, 0), (td, G.GmlWriteMode, 0)])
    kb = G.compile_kernel(gpu, body("ball_mean.cl"), "ball_mean", G.GmlVertices,
                          [(vd, G.GmlWriteMode, 0), (td, G.GmlReadMode, 0)])
    assert kc and kb
    assert G.lib.GmlLaunchKernel(gpu, kc) == 1 and G.lib.GmlLaunchKernel(gpu, kb) == 1
    cen = G.get_data(gpu, td, np.float32, (len(tet), 4))
    got = G.get_data(gpu, vd, np.float32, (len(crd), 4))
    exp_c = crd[tet].astype(np.float64).mean(axis=1)
    assert np.max(np.abs(cen - exp_c)) <= 1e-6
    acc = np.zeros((len(crd), 4))
    np.add.at(acc, tet.ravel(), np.repeat(cen.astype(np.float64), 4, axis=0))
    cnt = np.bincount(tet.ravel(), minlength=len(crd))
    assert np.max(np.abs(got - acc / cnt[:, None])) <= 1e-5
    # minimum over the ball of a tet scalar (runtime degree loop)
    q, qg = quality_gpu(G, gpu, v, len(tet))
    vq = G.lib.GmlNewSolutionData(gpu, G.GmlVertices, 1, G.GmlFlt, b"vq")
    tq_src = body("ball_min.cl").replace(b"tq", b"qal")
    km = G.compile_kernel(gpu, tq_src, "ball_min", G.GmlVertices,
                          [(q, G.GmlReadMode, 0), (vq, G.GmlWriteMode, 0)])
    assert km and G.lib.GmlLaunchKernel(gpu, km) == 1
    vmin = G.get_data(gpu, vq, np.float32, len(crd))
    exp = np.full(len(crd), np.inf)
    np.minimum.at(exp, tet.ravel(), np.repeat(qg, 4))
    assert np.array_equal(vmin, exp.astype(np.float32))


def test_c_client_mesh_quality(G, O, tmp_path):
    """The variadic C API end to end (tests/c/mesh_quality.c)."""
    exe = tmp_path / "mq"
    inc = os.path.join(ROOT, "include")
    r = subprocess.run(["gcc", "-std=c99", "-O2", "-I" + inc,
                        os.path.join(ROOT, "tests", "c", "mesh_quality.c"), "-o", str(exe),
                        G.LIB_PATH, "-Wl,-rpath," + os.path.dirname(G.LIB_PATH), "-lm"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = tmp_path / "q.bin"
    r = subprocess.run([str(exe), "16", "1", str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    s, mn = map(float, r.stdout.split()[-2:])
    q = np.fromfile(str(out), np.float32)
    crd, tet, ref = G.cube_mesh(16, split=1, jitter=0.25, seed=12345)
    qo = O.quality_ref(crd, tet)
    assert np.max(np.abs(q - qo)) <= 2e-5 * np.max(np.abs(qo))
    assert mn == float(q.min())
    assert s == pytest.approx(O.reduce(2, q), rel=1e-12)


def test_kernel_timing_and_calibration(G, gpu):
    crd, tet, ref = G.cube_mesh(40, split=0, jitter=0.25, seed=5)
    v, t = setup_mesh(G, gpu, crd, tet, ref)
    q = G.lib.GmlNewSolutionData(gpu, G.GmlTetrahedra, 1, G.GmlFlt, b"qal")
    k = G.compile_kernel(gpu, body("tet_quality.cl"), "quality", G.GmlTetrahedra,
                         [(v, G.GmlReadMode, 0), (q, G.GmlWriteMode, 0)])
    first = None
    for i in range(1 + 2 * 6 + 2):            # warm-up, 2 timings of 6 candidates, choice
        assert G.lib.GmlLaunchKernel(gpu, k) == 1
        if i == 0:
            first = G.get_data(gpu, q, np.float32, len(tet))
    last = G.get_data(gpu, q, np.float32, len(tet))
    assert np.array_equal(first, last)       # block size does not change results
    assert G.lib.GmlxKernelBlockSize(gpu, k) in (32, 64, 128, 256, 512, 1024)
    assert G.lib.GmlGetKernelRunTime(gpu, k) > 0
    G.reduce(gpu, q, G.GmlSum)
    assert G.lib.GmlGetReduceRunTime(gpu, G.GmlSum) > 0


TUNE_SCRIPT = r"""
import sys, numpy as np
sys.path.insert(0, %r)
sys.path.insert(0, %r)
import gmlib_gb300 as G
from conftest import PARAMS
crd, tet, ref = G.cube_mesh(40, split=0, jitter=0.25, seed=5)
g = G.lib.GmlInit(0)
G.lib.GmlNewParameters(g, 8, PARAMS)
v, t = G.upload_mesh(g, crd, tet, ref)
q = G.lib.GmlNewSolutionData(g, G.GmlTetrahedra, 1, G.GmlFlt, b"qal")
src = open(%r, "rb").read()
k = G.compile_kernel(g, src, "quality", G.GmlTetrahedra, [(v, G.GmlReadMode, 0), (q, G.GmlWriteMode, 0)])
n = int(sys.argv[1])
for _ in range(n):
    assert G.lib.GmlLaunchKernel(g, k) == 1
print(G.lib.GmlxKernelBlockSize(g, k))
G.lib.GmlStop(g)
"""


def test_calibration_is_kept_in_the_tuning_file(tmp_path):
    """A process that calibrated a kernel writes its block size to
    GML_CACHE_DIR/tune.json; a later process compiling the same kernel on
    the same line count starts with that block size (no calibration)."""
    script = TUNE_SCRIPT % (ROOT, os.path.join(ROOT, "tests"), os.path.join(KDIR, "tet_quality.cl"))
    env = dict(os.environ, GML_CACHE_DIR=str(tmp_path))
    first = subprocess.run([sys.executable, "-c", script, "15"], env=env, capture_output=True,
                           text=True, timeout=300)
    assert first.returncode == 0, first.stderr
    chosen = int(first.stdout.split()[-1])
    assert chosen in (32, 64, 128, 256, 512, 1024)
    text = (tmp_path / "tune.json").read_text()
    assert text.startswith("{") and '"k:' in text and (": %d" % chosen) in text
    again = subprocess.run([sys.executable, "-c", script, "1"], env=env, capture_output=True,
                           text=True, timeout=300)
    assert again.returncode == 0, again.stderr
    assert int(again.stdout.split()[-1]) == chosen


def _line_items_expected(a, b, c, d):
    ea = np.stack([a[:, 1] + a[:, 2], a[:, 2] - a[:, 0], a[:, 3] + a[:, 3], a[:, 0] - a[:, 1]], 1)
    ec = np.stack([c[:, 3], c[:, 2] + c[:, 0], c[:, 1] - c[:, 3], c[:, 0]], 1)
    eb = np.stack([b[:, 1], b[:, 0] + b[:, 0]], 1)
    ed = np.stack([d[:, 1] + d[:, 0], d[:, 0] - d[:, 1]], 1)
    return ea, eb, ec, ed


def test_line_items_load_and_store(G, gpu):
    """Lines of 2 and 4 sixteen-byte items (float4, int4, double2), read and
    written whole by a tet kernel (32-byte loads and stores), against numpy;
    plus a vertex kernel rewriting its own 4-item line with a ball sum, whose
    high-degree twin launch starts at a line offset."""
    crd, tet, ref = G.cube_mesh(12, split=1, jitter=0.2, seed=5)
    nv, nt = len(crd), len(tet)
    v, t = setup_mesh(G, gpu, crd, tet, ref)
    rng = np.random.default_rng(11)
    a = rng.standard_normal((nt, 4, 4)).astype(np.float32)
    b = rng.standard_normal((nt, 2, 4)).astype(np.float32)
    c = rng.integers(-1000, 1000, (nt, 4, 4)).astype(np.int32)
    d = rng.standard_normal((nt, 2, 2))
    ia = G.lib.GmlNewSolutionData(gpu, G.GmlTetrahedra, 4, G.GmlFlt4, b"A")
    ib = G.lib.GmlNewSolutionData(gpu, G.GmlTetrahedra, 2, G.GmlFlt4, b"B")
    ic = G.lib.GmlNewSolutionData(gpu, G.GmlTetrahedra, 4, G.GmlInt4, b"C")
    idd = G.lib.GmlNewSolutionData(gpu, G.GmlTetrahedra, 2, G.GmlDbl2, b"D")
    for idx, x in ((ia, a), (ib, b), (ic, c), (idd, d)):
        assert G.set_data(gpu, idx, x) == 1
    RW = G.GmlReadMode | G.GmlWriteMode
    k = G.compile_kernel(gpu, body("line_items.cl"), "line_items", G.GmlTetrahedra,
                         [(ia, RW, 0), (ib, RW, 0), (ic, RW, 0), (idd, RW, 0)])
    assert k and G.lib.GmlxKernelIsLazy(gpu, k) == 1
    src = G.lib.GmlxKernelSource(gpu, k)
    src = ctypes.string_at(src).decode() if isinstance(src, int) else src.decode()
    assert "gml_load_line(A, ATab[ cnt + count.s1 ]);" in src
    assert "gml_store_line(DTab[ cnt + count.s1 ], D);" in src
    assert G.lib.GmlLaunchKernel(gpu, k) == 1
    ea, eb, ec, ed = _line_items_expected(a, b, c, d)
    assert np.array_equal(G.get_data(gpu, ia, np.float32, (nt, 4, 4)), ea)
    assert np.array_equal(G.get_data(gpu, ib, np.float32, (nt, 2, 4)), eb)
    assert np.array_equal(G.get_data(gpu, ic, np.int32, (nt, 4, 4)), ec)
    assert np.array_equal(G.get_data(gpu, idd, np.float64, (nt, 2, 2)), ed)

    # vertex lines, through the base and the high ball tables
    q = rng.standard_normal(nt).astype(np.float32)
    v4 = rng.standard_normal((nv, 4, 4)).astype(np.float32)
    iq = G.lib.GmlNewSolutionData(gpu, G.GmlTetrahedra, 1, G.GmlFlt, b"Q")
    iv = G.lib.GmlNewSolutionData(gpu, G.GmlVertices, 4, G.GmlFlt4, b"V4")
    assert G.set_data(gpu, iq, q) == 1 and G.set_data(gpu, iv, v4) == 1
    kb = G.compile_kernel(gpu, body("line_items_ball.cl"), "line_items_ball", G.GmlVertices,
                          [(iv, RW, 0), (iq, G.GmlReadMode, 0)])
    assert kb
    assert G.lib.GmlLaunchKernel(gpu, kb) == 1
    got = G.get_data(gpu, iv, np.float32, (nv, 4, 4))
    s = np.zeros(nv, np.float64)
    np.add.at(s, tet.reshape(-1), np.repeat(q.astype(np.float64), 4))
    want = np.stack([v4[:, 3] + s[:, None], v4[:, 0] + v4[:, 1], v4[:, 1] - v4[:, 2],
                     v4[:, 2] + v4[:, 0]], 1)
    # items 1..3 are exact; item 0 holds an FP32 ball sum (order differs)
    assert np.array_equal(got[:, 1:], want[:, 1:].astype(np.float32))
    assert np.max(np.abs(got[:, 0] - want[:, 0])) <= 1e-5 * max(1.0, float(np.abs(want[:, 0]).max()))
