"""Parity with the reference's own host library, executed.

tests/golden/refhost_*.npz were made by tests/golden/make_refhost.py, which
runs the reference's unmodified sources/gmlib3.c (compiled against an OpenCL
stand-in, its kernels built by g++ and run on the CPU).  These tests check,
without a GPU:

  - this library's host-built tables (offline instances): the vertex -> tet
    ball tables, GmlExtractEdges, GmlExtractFaces, GmlEvaluateNumbering, bit
    for bit, on the fixture meshes and on the 32^3-hex cube by digest;
  - the oracle's restatements against the same fixtures (ball tables, edges,
    faces, the MeshQuality and NodeSmoothing bodies, the reductions' group
    and truncation semantics, the LinearSolver flow).

One documented difference is masked: the reference never writes row 0 of
the high-degree ball table (gmlib3.c:1126-1129, the MaxPos line lands in the
base table instead), so its high kernel reads zeros for that line; here that
row holds the line's ball.
"""
import ctypes
import hashlib
import os

import numpy as np
import pytest

from conftest import PARAMS

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
KDIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "kernels")
CASES = [("refhost_kuhn_n5.npz", "kuhn_n5.npz"), ("refhost_reflected_n6.npz", "reflected_n6.npz")]


def load(name):
    return dict(np.load(os.path.join(GOLD, name)))


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def offline_tables(G, crd, tet, ref):
    """Ball tables, edges, faces and the numbering factor built by this
    library on an offline instance (host code only)."""
    g = G.lib.GmlxInitOffline()
    try:
        G.lib.GmlNewParameters(g, 8, PARAMS)
        v, t = G.upload_mesh(g, crd, tet, ref)
        opt = G.lib.GmlNewSolutionData(g, G.GmlTetrahedra, 4, G.GmlFlt4, b"OptCrd")
        res = G.lib.GmlNewSolutionData(g, G.GmlVertices, 1, G.GmlFlt, b"res")
        with open(os.path.join(KDIR, "relax_to_points.cl"), "rb") as f:
            src = f.read()
        k = G.compile_kernel(g, src, "gather", G.GmlVertices,
                             [(res, G.GmlWriteMode, 0), (opt, G.GmlReadMode | G.GmlVoyeurs, 0),
                              (v, G.GmlReadMode | G.GmlWriteMode, 0)])
        assert k > 0
        b, d, h = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        assert G.lib.GmlxLinkData(g, G.GmlVertices, G.GmlTetrahedra, ctypes.byref(b),
                                  ctypes.byref(d), ctypes.byref(h)) == 1
        out = {"deg": G.get_data(g, d.value, np.int32, len(crd))}
        nb = G.lib.GmlxDataLines(g, b.value)
        out["base"] = G.get_data(g, b.value, np.int32, (nb, 32))
        if h.value:
            nh = G.lib.GmlxDataLines(g, h.value)
            out["high"] = G.get_data(g, h.value, np.int32, (nh, 64))
        else:
            out["high"] = np.zeros((0, 64), np.int32)
        ne = G.lib.GmlExtractEdges(g)
        nl, di = ctypes.c_int(), ctypes.c_int()
        assert G.lib.GmlGetMeshInfo(g, G.GmlEdges, ctypes.byref(nl), ctypes.byref(di)) == 1
        assert nl.value == ne
        out["edges"] = G.get_data(g, di.value, np.int32, (ne, 2))
        # measured, as in the fixture script, with the edges present
        out["numbering"] = np.float32(G.lib.GmlEvaluateNumbering(g))
        nf = G.lib.GmlExtractFaces(g)
        assert G.lib.GmlGetMeshInfo(g, G.GmlTriangles, ctypes.byref(nl), ctypes.byref(di)) == 1
        assert nl.value == nf
        tri = G.get_data(g, di.value, np.int32, (nf, 4))[:, :3]
        tref = G.get_data(g, di.value + 1, np.int32, (nf,))
        out["tri"] = np.column_stack([tri, tref]).astype(np.int32)
        return out
    finally:
        G.lib.GmlStop(g)


def check_high(ours, ref):
    """Rows 1.. bit for bit; row 0: zeros in the reference, the MaxPos
    line's ball here."""
    assert len(ours) == len(ref)
    if len(ref):
        assert ours.shape == ref.shape
        assert np.array_equal(ours[1:], ref[1:])
        assert not ref[0].any()


@pytest.mark.parametrize("fix,mesh", CASES)
def test_library_tables_match_reference_host(G, fix, mesh):
    r, m = load(fix), load(mesh)
    ours = offline_tables(G, m["crd"], m["tet"], m["ref"])
    assert np.array_equal(ours["deg"], r["deg"])
    assert np.array_equal(ours["base"], r["base"])
    check_high(ours["high"], r["high"])
    assert np.array_equal(ours["edges"], r["edges"])
    assert np.array_equal(ours["tri"], r["tri"])
    assert ours["numbering"] == r["numbering"]


def test_library_tables_match_reference_host_32cube(G):
    """The 32^3-hex Kuhn cube (jitter 0.25 h, seed 12345): ball tables, edges
    and faces by SHA-256 against the reference's own run."""
    r = load("refhost_c1.npz")
    crd, tet, ref = G.cube_mesh(32, split=0, jitter=0.25, seed=12345)
    assert digest(crd) + digest(tet) == str(r["mesh"]), "mesh generator changed"
    ours = offline_tables(G, crd, tet, ref)
    assert len(ours["base"]) == int(r["n_base"]) and len(ours["high"]) == int(r["n_high"])
    assert digest(ours["deg"]) == str(r["deg"])
    assert digest(ours["base"]) == str(r["base"])
    assert digest(ours["high"]) == str(r["high"])
    assert len(ours["edges"]) == int(r["n_edges"]) and digest(ours["edges"]) == str(r["edges"])
    assert len(ours["tri"]) == int(r["n_tri"]) and digest(ours["tri"]) == str(r["tri"])
    assert ours["numbering"] == r["numbering"]


@pytest.mark.parametrize("fix,mesh", CASES)
def test_oracle_tables_match_reference_host(O, fix, mesh):
    r, m = load(fix), load(mesh)
    deg, mp, hs, base, high = O.ver_tet_ball(len(m["crd"]), m["tet"], 32, 64)
    assert np.array_equal(deg, r["deg"])
    assert np.array_equal(base[:int(r["n_base"])], r["base"])
    check_high(high, r["high"])
    assert np.array_equal(O.tet_edges(m["tet"]), r["edges"])
    tri, _ = O.extract_faces({4: (m["tet"], np.zeros(len(m["tet"])))})
    assert np.array_equal(tri, r["tri"])


@pytest.mark.parametrize("fix,mesh", CASES)
def test_oracle_bodies_match_reference_host(O, fix, mesh):
    """MeshQuality and NodeSmoothing bodies as the reference generated and
    ran them (FP32 on the CPU) against the oracle's restatements."""
    r, m = load(fix), load(mesh)
    crd, tet = m["crd"], m["tet"]
    q = O.quality_ref(crd, tet)
    scale = np.max(np.abs(q))
    assert np.max(np.abs(q - r["mq_qal"])) <= 1e-6 * scale
    assert np.max(np.abs(q - r["ns_qal0"])) <= 1e-6 * scale
    opt = O.scatter(crd, tet)
    assert np.max(np.abs(opt - r["ns_opt1"])) <= 1e-6
    deg, full = O.ball_codes(len(crd), tet)
    new, res = O.gather(crd, deg, full, opt)
    keep = np.ones(len(crd), bool)
    if int(r["n_high"]):
        # the reference's high kernel reads the unwritten row 0 for line MaxPos
        keep[int(np.argmax(r["deg"] > 32))] = False
    assert np.max(np.abs(new[keep] - r["ns_crd1"][keep])) <= 1e-6
    assert np.max(np.abs(res[keep] - r["ns_res1"][keep])) <= 1e-7


def reference_reduce(op, x, grp=16):
    """The reference's reduction on its first call: work-groups of 16
    (RunOclKrn's first run, gmlib3.c:3146-3152), a shared-memory tree per
    group (reduce.cl), then a float loop over the N / 16 complete groups on
    the host (gmlib3.c:3296-3324): the last partial group is dropped."""
    x = np.asarray(x, np.float32)
    f = {0: lambda v: v, 1: lambda v: v, 2: lambda v: v,
         3: lambda v: (v != 0).astype(np.float32), 4: np.abs,
         5: lambda v: v * v, 6: np.abs}[op]
    comb = {0: np.minimum, 1: np.maximum, 6: np.maximum}.get(op, np.add)
    ng = len(x) // grp
    t = f(x[:ng * grp]).reshape(ng, grp).astype(np.float32)
    i = grp // 2
    while i:
        t[:, :i] = comb(t[:, :i], t[:, i:2 * i]).astype(np.float32)
        i //= 2
    part = t[:, 0]
    res = np.float32({0: 3.4028234663852886e38, 1: -3.4028234663852886e38, 6: -3.4028234663852886e38}
                     .get(op, 0.0))
    for p in part:
        res = np.float32(comb(res, p))
    return float(res)


@pytest.mark.parametrize("fix", [c[0] for c in CASES])
def test_reference_reduction_semantics(fix):
    """The reductions the reference ran, reproduced bit for bit from their
    definition (float group trees, truncated last group)."""
    r = load(fix)
    for op in range(7):
        assert reference_reduce(op, r["mq_qal"]) == r["red"][op], op
    assert reference_reduce(0, r["mq_qal"]) == r["mq_min"]


def spmv(lin, col, vals, x, b, dt):
    rows = np.repeat(np.arange(len(lin) - 1), np.diff(lin))
    y = np.zeros_like(x, dtype=dt)
    np.add.at(y, rows, np.einsum("kij,kj->ki", vals.astype(dt).reshape(-1, b, b), x.astype(dt)[col]))
    return y


def linsolve_flow(lin, col, vals, diag, x0, rhs, b, use_diag, iters, dt):
    """The example's loop (LinearSolver.c:311-336) with the reference's
    argument semantics: GmlMultDiagMatVec(D, Xk0, Xk1) writes Xk1 = D Xk0;
    GmlMultMatVec(M, Xk0, Tmp) writes Xk0 = A Tmp (its first vector is the
    output, gmlib3.c:3383-3389), which GmlAddVec3(Rhs, Tmp, Xk1, Xk0) then
    overwrites with Rhs + Tmp + Xk1, so Tmp keeps its initial value; the
    norm is sqrt(sum_l |x_l|_2) (GmlNormVec, gmlib3.c:3534-3575)."""
    x = x0.astype(dt)
    tmp = x0.astype(dt)
    x1 = x0.astype(dt)
    norms = []
    for _ in range(iters):
        if use_diag:
            x1 = np.einsum("lij,lj->li", diag.astype(dt).reshape(-1, b, b), x).astype(dt)
        x = spmv(lin, col, vals, tmp, b, dt)          # overwritten below
        x = ((rhs.astype(dt) + tmp) + x1).astype(dt)
        norms.append(np.sqrt(np.sum(np.sqrt(np.sum(x.astype(np.float64) ** 2, 1)))))
    return np.array(norms), x


def test_linsolve_restatement_matches_reference_host():
    import importlib.util
    spec = importlib.util.spec_from_file_location("mk", os.path.join(GOLD, "make_refhost.py"))
    mk = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mk)
    r = load("refhost_linsolve.npz")
    lin, col = r["lin"], r["col"]
    nv = len(lin) - 1
    # the CSR the example builds from the reference's edges
    l2, c2 = mk.csr_from_edges(nv, r["edges"])
    assert np.array_equal(l2, lin) and np.array_equal(c2, col)
    for b, dbl, use_diag in mk.LINSOLVE:
        tag = "b%d_%s" % (b, "f64" if dbl else "f32")
        vals, diag, x0, rhs = mk.linsolve_inputs(nv, len(col), b, dbl)
        norms, x = linsolve_flow(lin, col, vals, diag, x0, rhs, b, use_diag, 5,
                                 np.float64 if dbl else np.float32)
        tol = 1e-12 if dbl else 2e-6
        # the norm's L1 sum is a float reduction in both precisions
        assert np.allclose(norms, r[tag + "_norms"], rtol=2e-6, atol=0), tag
        assert np.max(np.abs(x - r[tag + "_x"])) <= tol * max(1.0, np.max(np.abs(x))), tag
        ax = spmv(lin, col, vals, x0, b, np.float64 if dbl else np.float32)
        assert np.max(np.abs(ax - r[tag + "_ax"])) <= tol * max(1.0, np.max(np.abs(ax))), tag


def examples_restated(r):
    """The GpuBandwidth, TestFeatures and BallQuality flows of
    make_refhost.make_examples restated in numpy (FP32 where the kernels
    compute in FP32, sums in the kernels' order)."""
    crd, tet = r["crd"], r["tet"]
    nv, nt = len(crd), len(tet)
    f = np.float32
    c = crd.astype(f)
    out = {"bw_ver": c.copy(), "bw_tet_nodes": tet.astype(f)}
    ts = ((c[tet[:, 0]] + c[tet[:, 1]]) + c[tet[:, 2]]) + c[tet[:, 3]]
    out["bw_tet_sum"] = ts
    # balls in increasing tet order, as the tables hold them
    order = np.argsort(tet.ravel(), kind="stable")
    owner = tet.ravel()[order]
    tets = order // 4
    ball = np.zeros((nv, 4), f)
    for v_, t_ in zip(owner, tets):
        ball[v_] = ball[v_] + ts[t_]
    out["bw_ball"] = ball
    deg = np.bincount(tet.ravel(), minlength=nv).astype(f)
    sol = np.full((nv, 2, 4), 0.125, f)
    mids, sols = [], []
    for i in range(1, int(len(r["ft_mid"])) + 1):
        left = ((sol[tet[:, 0], 0] + sol[tet[:, 1], 0]) + sol[tet[:, 2], 0]) + sol[tet[:, 3], 0]
        right = ((sol[tet[:, 0], 1] + sol[tet[:, 1], 1]) + sol[tet[:, 2], 1]) + sol[tet[:, 3], 1]
        m = ts * (left + right)
        m = m / np.sqrt(np.sum(m.astype(np.float64) ** 2, axis=1))[:, None].astype(f)
        acc = np.zeros((nv, 4), f)
        for v_, t_ in zip(owner, tets):
            acc[v_] = acc[v_] + m[t_]
        sol = np.repeat((f(i) * acc / deg[:, None])[:, None, :], 2, axis=1)
        mids.append(m)
        sols.append(sol.copy())
    out["ft_mid"], out["ft_sol"] = np.array(mids), np.array(sols)
    out["ft_res"] = np.full(nt, f(nt) / f(len(mids)), f)
    # triangle quality, 3.4641 |ab x ac| / (hmax (ha + hb + hc)) (1 for an
    # equilateral triangle), and its vertex-ball minimum
    p = r["sq_crd"].astype(np.float64)[:, :3]
    a, b, cc = p[r["sq_tri"][:, 0]], p[r["sq_tri"][:, 1]], p[r["sq_tri"][:, 2]]
    ha, hb, hc = (np.linalg.norm(b - cc, axis=1), np.linalg.norm(cc - a, axis=1),
                  np.linalg.norm(a - b, axis=1))
    s = np.linalg.norm(np.cross(b - a, cc - a), axis=1)
    out["bq_tq"] = 3.46410 * s / (np.maximum(np.maximum(ha, hb), hc) * (ha + hb + hc))
    vq = np.full(len(p), np.inf)
    np.minimum.at(vq, r["sq_tri"].ravel(), np.repeat(r["bq_tq"].astype(np.float64), 3))
    out["bq_vq"] = vq
    return out


def test_example_flows_restatement_matches_reference_host():
    r = load("refhost_examples.npz")
    o = examples_restated(r)
    for k in ("bw_ver", "bw_tet_nodes", "bw_tet_sum"):
        assert np.array_equal(o[k], r[k]), k
    assert np.max(np.abs(o["bw_ball"] - r["bw_ball"])) <= 1e-6 * np.max(np.abs(r["bw_ball"]))
    for k in ("ft_mid", "ft_sol"):
        assert np.max(np.abs(o[k] - r[k])) <= 2e-6 * max(1.0, np.max(np.abs(r[k]))), k
    assert np.array_equal(o["ft_res"], r["ft_res"])
    nt = len(r["tet"])
    # the exact residual sums; the reference's own first one misses the
    # work-groups its calibration launch truncated
    assert np.allclose(r["ft_red_exact"], [nt * nt / i for i in (1, 2, 3)], rtol=1e-7)
    assert r["ft_red"][0] < r["ft_red_exact"][0]
    assert np.max(np.abs(o["bq_tq"] - r["bq_tq"])) <= 2e-6
    assert np.array_equal(o["bq_vq"].astype(np.float32), r["bq_vq"])
