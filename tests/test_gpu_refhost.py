"""The library on the GPU against what the reference's own host library
produced when run (tests/golden/refhost_*.npz, made by
tests/golden/make_refhost.py from the unmodified sources/gmlib3.c):

  - GmlExtractEdges / GmlExtractFaces / GmlEvaluateNumbering and the
    generated kernels' ball tables on GPU instances, bit for bit;
  - GmlSetNeighbours: the reference passes &TetNgb to the variadic
    GmlSetDataLine (gmlib3.c:4258), which reads ints, so its table holds
    pointer bits; the neighbours here are checked against the oracle's
    restatement of the hash walk and for symmetry;
  - the MeshQuality and NodeSmoothing flows (the bodies restated in
    tests/kernels/, compiled by GmlCompileKernel) against the reference's
    generated kernels run in FP32 on the CPU;
  - the LinearSolver flow (GmlNewMatrix, GmlMultDiagMatVec, GmlMultMatVec,
    GmlAddVec3, GmlNormVec) against the reference's flow.

Tolerances (FP32 GPU against FP32 CPU): quality 2e-5 of the largest |q|;
one sweep 2e-6; three sweeps 1e-5; FP64 vectors 1e-12 and FP32 2e-6 of the
largest magnitude; norms 2e-6 relative (the reference sums them in float).
"""
import ctypes
import hashlib
import importlib.util
import os

import numpy as np
import pytest

from conftest import PARAMS

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
KDIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "kernels")
CASES = [("refhost_kuhn_n5.npz", "kuhn_n5.npz"), ("refhost_reflected_n6.npz", "reflected_n6.npz")]


def load(name):
    return dict(np.load(os.path.join(GOLD, name)))


def body(name):
    with open(os.path.join(KDIR, name), "rb") as f:
        return f.read()


def fixture_script():
    spec = importlib.util.spec_from_file_location("mk", os.path.join(GOLD, "make_refhost.py"))
    mk = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mk)
    return mk


def mesh_info(G, g, typ):
    nl, di = ctypes.c_int(), ctypes.c_int()
    assert G.lib.GmlGetMeshInfo(g, typ, ctypes.byref(nl), ctypes.byref(di)) == 1
    return nl.value, di.value


def smoothing_kernels(G, g, v):
    opt = G.lib.GmlNewSolutionData(g, G.GmlTetrahedra, 4, G.GmlFlt4, b"OptCrd")
    res = G.lib.GmlNewSolutionData(g, G.GmlVertices, 1, G.GmlFlt, b"res")
    ks = G.compile_kernel(g, body("optimal_points.cl"), "scatter", G.GmlTetrahedra,
                          [(v, G.GmlReadMode, 0), (opt, G.GmlWriteMode, 0)])
    kg = G.compile_kernel(g, body("relax_to_points.cl"), "gather", G.GmlVertices,
                          [(res, G.GmlWriteMode, 0), (opt, G.GmlReadMode | G.GmlVoyeurs, 0),
                           (v, G.GmlReadMode | G.GmlWriteMode, 0)])
    assert ks > 0 and kg > 0
    return opt, res, ks, kg


@pytest.mark.parametrize("fix,mesh", CASES)
def test_tables_on_gpu_instance(G, gpu, fix, mesh):
    r, m = load(fix), load(mesh)
    G.lib.GmlNewParameters(gpu, 8, PARAMS)
    v, t = G.upload_mesh(gpu, m["crd"], m["tet"], m["ref"])
    smoothing_kernels(G, gpu, v)
    b, d, h = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    assert G.lib.GmlxLinkData(gpu, G.GmlVertices, G.GmlTetrahedra, ctypes.byref(b),
                              ctypes.byref(d), ctypes.byref(h)) == 1
    assert np.array_equal(G.get_data(gpu, d.value, np.int32, len(m["crd"])), r["deg"])
    base = G.get_data(gpu, b.value, np.int32, (G.lib.GmlxDataLines(gpu, b.value), 32))
    assert np.array_equal(base, r["base"])
    if int(r["n_high"]):
        high = G.get_data(gpu, h.value, np.int32, (G.lib.GmlxDataLines(gpu, h.value), 64))
        assert high.shape == r["high"].shape
        assert np.array_equal(high[1:], r["high"][1:])     # row 0: see the module doc
    ne = G.lib.GmlExtractEdges(gpu)
    n, e = mesh_info(G, gpu, G.GmlEdges)
    assert n == ne
    assert np.array_equal(G.get_data(gpu, e, np.int32, (ne, 2)), r["edges"])
    assert np.float32(G.lib.GmlEvaluateNumbering(gpu)) == r["numbering"]
    nf = G.lib.GmlExtractFaces(gpu)
    n, f = mesh_info(G, gpu, G.GmlTriangles)
    assert n == nf
    tri = G.get_data(gpu, f, np.int32, (nf, 4))[:, :3]
    tref = G.get_data(gpu, f + 1, np.int32, (nf,))
    assert np.array_equal(np.column_stack([tri, tref]), r["tri"])


@pytest.mark.parametrize("n,split", [(5, 0), (6, 1)])
def test_neighbours_on_gpu_instance(G, O, gpu, n, split):
    """Each tet's neighbour across its face j (the face opposite vertex j, in
    the reference's face order), 0 on the boundary; symmetric."""
    crd, tet, ref = G.cube_mesh(n, split=split, jitter=0.2, seed=n)
    G.upload_mesh(gpu, crd, tet, ref)
    idx = G.lib.GmlSetNeighbours(gpu, G.GmlTetrahedra)
    assert idx > 0
    ngb = G.get_data(gpu, idx, np.int32, (len(tet), 4))
    # the oracle: faces keyed by their sorted nodes, users in element order
    faces = {}
    loc = ((1, 2, 3), (2, 0, 3), (3, 0, 1), (0, 2, 1))
    for i, t4 in enumerate(tet):
        for j, l in enumerate(loc):
            faces.setdefault(tuple(sorted(t4[list(l)])), []).append((i, j))
    exp = np.zeros((len(tet), 4), np.int32)
    nbound = 0
    for users in faces.values():
        if len(users) == 2:
            (a, ja), (b, jb) = users
            exp[a, ja], exp[b, jb] = b, a
        else:
            nbound += 1
    assert np.array_equal(ngb, exp)
    assert nbound == 12 * n * n                  # two boundary triangles per square
    # symmetry: b is a's neighbour across face j iff a is one of b's
    for a in range(len(tet)):
        for j in range(4):
            b = ngb[a, j]
            if b or a == 0:
                assert a in ngb[b] or (b == 0 and exp[a, j] == 0)


def contaminated(tet, start, rings):
    """Vertices within `rings` tet-hops of `start` (the reference's corrupted
    MaxPos line spreads one ring per later sweep)."""
    cur = {start}
    for _ in range(rings):
        touch = np.isin(tet, list(cur)).any(1)
        cur |= set(np.unique(tet[touch]).tolist())
    return np.array(sorted(cur))


@pytest.mark.parametrize("fix,mesh", CASES)
def test_mesh_quality_and_node_smoothing_flows(G, gpu, fix, mesh):
    r, m = load(fix), load(mesh)
    crd, tet = m["crd"], m["tet"]
    nv, nt = len(crd), len(tet)
    G.lib.GmlNewParameters(gpu, 8, PARAMS)
    v, t = G.upload_mesh(gpu, crd, tet, m["ref"])
    q = G.lib.GmlNewSolutionData(gpu, G.GmlTetrahedra, 1, G.GmlFlt, b"qal")
    kq = G.compile_kernel(gpu, body("tet_quality.cl"), "quality", G.GmlTetrahedra,
                          [(v, G.GmlReadMode, 0), (q, G.GmlWriteMode, 0)])
    assert kq > 0 and G.lib.GmlLaunchKernel(gpu, kq) == 1
    qg = G.get_data(gpu, q, np.float32, nt)
    scale = np.max(np.abs(r["mq_qal"]))
    assert np.max(np.abs(qg - r["mq_qal"])) <= 2e-5 * scale
    assert np.max(np.abs(qg - r["ns_qal0"])) <= 2e-5 * scale
    # GmlReduceVector(min) over every line (the reference drops the last
    # partial work-group; its value is checked against that rule on the CPU)
    assert G.reduce(gpu, q, G.GmlMin) == float(qg.min())
    opt, res, ks, kg = smoothing_kernels(G, gpu, v)
    bad = np.zeros(nv, bool)
    if int(r["n_high"]):
        mp = int(np.argmax(r["deg"] > 32))
        bad1 = np.zeros(nv, bool)
        bad1[mp] = True
        bad[contaminated(tet, mp, 2)] = True
    else:
        bad1 = bad
    for s in range(1, 4):
        assert G.lib.GmlLaunchKernel(gpu, ks) == 1
        if s == 1:
            assert np.max(np.abs(G.get_data(gpu, opt, np.float32, (nt, 4, 4)) - r["ns_opt1"])) <= 2e-6
        assert G.lib.GmlLaunchKernel(gpu, kg) == 1
        if s == 1:
            c1 = G.get_data(gpu, v, np.float32, (nv, 4))
            r1 = G.get_data(gpu, res, np.float32, nv)
            assert np.max(np.abs(c1[~bad1] - r["ns_crd1"][~bad1])) <= 2e-6
            assert np.max(np.abs(r1[~bad1] - r["ns_res1"][~bad1])) <= 1e-8
    c3 = G.get_data(gpu, v, np.float32, (nv, 4))
    assert np.max(np.abs(c3[~bad] - r["ns_crd3"][~bad])) <= 1e-5


def test_32cube_tables_and_quality(G, gpu):
    """The 32^3-hex Kuhn cube: ball tables and edges by digest, and the
    MeshQuality minimum, against the reference's run."""
    r = load("refhost_c1.npz")
    crd, tet, ref = G.cube_mesh(32, split=0, jitter=0.25, seed=12345)
    dig = lambda a: hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()  # noqa: E731
    assert dig(crd) + dig(tet) == str(r["mesh"])
    G.lib.GmlNewParameters(gpu, 8, PARAMS)
    v, t = G.upload_mesh(gpu, crd, tet, ref)
    smoothing_kernels(G, gpu, v)
    b, d, h = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    assert G.lib.GmlxLinkData(gpu, G.GmlVertices, G.GmlTetrahedra, ctypes.byref(b),
                              ctypes.byref(d), ctypes.byref(h)) == 1
    assert h.value == 0 and int(r["n_high"]) == 0
    assert dig(G.get_data(gpu, d.value, np.int32, len(crd))) == str(r["deg"])
    base = G.get_data(gpu, b.value, np.int32, (G.lib.GmlxDataLines(gpu, b.value), 32))
    assert dig(base) == str(r["base"])
    ne = G.lib.GmlExtractEdges(gpu)
    n, e = mesh_info(G, gpu, G.GmlEdges)
    assert ne == int(r["n_edges"]) and dig(G.get_data(gpu, e, np.int32, (ne, 2))) == str(r["edges"])
    q = G.lib.GmlNewSolutionData(gpu, G.GmlTetrahedra, 1, G.GmlFlt, b"qal")
    kq = G.compile_kernel(gpu, body("tet_quality.cl"), "quality", G.GmlTetrahedra,
                          [(v, G.GmlReadMode, 0), (q, G.GmlWriteMode, 0)])
    assert kq > 0 and G.lib.GmlLaunchKernel(gpu, kq) == 1
    qg = G.get_data(gpu, q, np.float32, len(tet))
    mn = G.reduce(gpu, q, G.GmlMin)
    assert mn == float(qg.min())
    assert abs(mn - float(r["mq_min"])) <= 2e-5 * abs(float(r["mq_min"]))
    srt = np.sort(qg)
    if srt[1] - srt[0] > 1e-4:
        assert int(np.argmin(qg)) == int(r["mq_argmin"])


def vec(G, g, arr, flt):
    a = np.ascontiguousarray(arr, np.float32 if flt == G.GmlFlt else np.float64)
    idx = G.lib.GmlNewVector(g, a.shape[0], a.shape[1], G.as_ptr(a), flt)
    assert idx > 0
    return idx


def read_vec(G, g, idx, nv, b, flt):
    dt = np.float32 if flt == G.GmlFlt else np.float64
    w = 4 if b <= 4 else 8
    return G.get_data(g, G.lib.GmlxVectorData(g, idx), dt, (nv, w))[:, :b]


def matrix(G, g, lin, col, vals, b, flt):
    v = np.ascontiguousarray(vals, np.float32 if flt == G.GmlFlt else np.float64)
    IP = ctypes.POINTER(ctypes.c_int)
    lin = np.ascontiguousarray(lin, np.int32)
    col = np.ascontiguousarray(col, np.int32)
    idx = G.lib.GmlNewMatrix(g, len(lin) - 1, len(col), b, G.as_ptr(v),
                             col.ctypes.data_as(IP), lin.ctypes.data_as(IP), flt)
    assert idx > 0
    return idx


def test_linear_solver_flow(G):
    mk = fixture_script()
    r = load("refhost_linsolve.npz")
    crd, tet, ref = mk.linsolve_mesh()
    assert mk.digest(crd) + mk.digest(tet) == str(r["mesh"])
    nv = len(crd)
    for b, dbl, use_diag in mk.LINSOLVE:
        tag = "b%d_%s" % (b, "f64" if dbl else "f32")
        flt = G.GmlDbl if dbl else G.GmlFlt
        tol = 1e-12 if dbl else 2e-6
        vals, diag, x0, rhs = mk.linsolve_inputs(nv, len(r["col"]), b, dbl)
        g = G.lib.GmlInit(0)
        assert g
        try:
            G.lib.GmlNewParameters(g, 8, PARAMS)
            G.upload_mesh(g, crd, tet, ref)
            ne = G.lib.GmlExtractEdges(g)
            n, e = mesh_info(G, g, G.GmlEdges)
            assert np.array_equal(G.get_data(g, e, np.int32, (ne, 2)), r["edges"])
            lin, col = mk.csr_from_edges(nv, r["edges"])
            mat = matrix(G, g, lin, col, vals, b, flt)
            dia = vec(G, g, diag, flt)
            xk0, xk1, tmp, rhv = (vec(G, g, x0, flt), vec(G, g, x0, flt), vec(G, g, x0, flt),
                                  vec(G, g, rhs, flt))
            red = G.lib.GmlNewSolutionData(g, G.GmlVertices, 1, G.GmlFlt, b"reduction")
            norms = []
            for _ in range(5):
                if use_diag:
                    assert G.lib.GmlMultDiagMatVec(g, dia, xk0, xk1) == 1
                assert G.lib.GmlMultMatVec(g, mat, xk0, tmp) == 1
                assert G.lib.GmlAddVec3(g, rhv, tmp, xk1, xk0) == 1
                nrm = ctypes.c_double()
                assert G.lib.GmlNormVec(g, xk0, red, ctypes.byref(nrm)) == 1
                norms.append(nrm.value)
            assert np.allclose(norms, r[tag + "_norms"], rtol=2e-6, atol=0), tag
            x = read_vec(G, g, xk0, nv, b, flt)
            assert np.max(np.abs(x - r[tag + "_x"])) <= tol * max(1.0, np.abs(x).max()), tag
            # one product on its own: y = A x
            y = vec(G, g, np.zeros((nv, b)), flt)
            xi = vec(G, g, x0, flt)
            assert G.lib.GmlMultMatVec(g, mat, y, xi) == 1
            ax = read_vec(G, g, y, nv, b, flt)
            assert np.max(np.abs(ax - r[tag + "_ax"])) <= tol * max(1.0, np.abs(ax).max()), tag
        finally:
            G.lib.GmlStop(g)
