"""Generate tests/golden/refhost_*.npz by running the reference's own host
library (sources/gmlib3.c, unmodified) on the CPU.

oracle/_ref/librefhost.so is that file compiled against an OpenCL stand-in
header, with a host-CPU OpenCL runtime that builds the kernels the reference
generates (and its library kernels) with g++ and runs them
(oracle/refhost/, recipe oracle/build.py build_refhost).  This script calls
the reference's API the way its examples do and stores what the reference
produced:

  refhost_kuhn_n5.npz, refhost_reflected_n6.npz   (inputs: kuhn_n5.npz and
      reflected_n6.npz of this directory)
    deg, base, high, n_base, n_high  vertex -> tet ball tables as uploaded by
        NewBallData (gmlib3.c:743-1168), read from the arguments of the
        generated NodeSmoothing gather kernel and of its high-degree twin;
        `high` row 0 is left as the reference leaves it (never written)
    edges          GmlExtractEdges (:3719-3873), (v0, v1) per edge
    tri            GmlExtractFaces (:3880-4171), (v0, v1, v2, ref)
    numbering      GmlEvaluateNumbering (:4409-4442)
    mq_qal         examples/MeshQuality/compute_quality.cl through
                   GmlCompileKernel/GmlLaunchKernel
    mq_min         GmlReduceVector(GmlMin) of it (first reduction of a fresh
                   instance; later calls with the same operation rebind no
                   arguments, gmlib3.c:3098-3135)
    red            GmlReduceVector(op) of mq_qal for op = Min..Linf, each the
                   first reduction of a fresh instance
    ns_qal0, ns_opt1, ns_crd1, ns_res1, ns_crd3
                   the NodeSmoothing flow (NodeSmoothing.c:114-161): quality
                   before smoothing, OptCrd and coordinates and residuals
                   after one scatter+gather sweep, coordinates after three
  refhost_c1.npz   the 32^3-hex Kuhn cube (jitter 0.25 h, seed 12345, Hilbert
                   order): SHA-256 digests of deg, base, high (row 0 as
                   above) and edges, plus numbering and the MeshQuality
                   minimum
  refhost_linsolve.npz   the LinearSolver flow (LinearSolver.c:157-340) on the
                   7^3-hex Kuhn cube: CSR from GmlExtractEdges, block
                   values from pseudo(), then D.x (b = 5 only), A.x,
                   AddVec3, NormVec for 5 iterations, for the (block,
                   precision) pairs of LINSOLVE: each iteration's norm and
                   the final x; and `_ax`, y = A x0 from one
                   GmlMultMatVec(mat, y, x) in a fresh instance.  In the
                   example's loop GmlMultMatVec(mat, Xk0, Tmp) writes
                   Xk0 = A Tmp, which GmlAddVec3 then overwrites, so the
                   loop itself does not depend on A
  refhost_heat.npz the HeatCellCentered flow (HeatCellCentered.c:90-180) on a
                   4^3-hex Kuhn cube with side-referenced boundary triangles:
                   faces, triangle -> tet shells, tet -> triangle links, the
                   time step, 30 explicit steps (see make_heat)
  refhost_examples.npz   the GpuBandwidth, TestFeatures and BallQuality
                   flows with their own bodies (see make_examples): on the
                   5^3-hex Kuhn cube the direct, downlink and ball kernels'
                   outputs, and three TestFeatures iterations (tet and
                   vertex fields, residual sums as returned and over every
                   line); on a 12 x 12 jittered square of triangles the
                   triangle qualities and their vertex-ball minima.  The
                   example's neighbours kernel is left out: it writes
                   nothing, and the reference's neighbour link holds pointer
                   bits (gmlib3.c:4258), so its reads would leave the arrays

Usage:  python tests/golden/make_refhost.py        (needs the reference tree)
"""
import ctypes
import hashlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import build as OB  # noqa: E402
from oracle import refhost as R  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
EX = os.path.join(OB.REF_ROOT, "examples")


def body(rel):
    with open(os.path.join(EX, rel), "rb") as f:
        return f.read()


def f32(b, shape):
    return np.frombuffer(b, np.float32)[:int(np.prod(shape))].reshape(shape).copy()


def i32(b, shape):
    return np.frombuffer(b, np.int32)[:int(np.prod(shape))].reshape(shape).copy()


def ball_and_smoothing(crd, tet, ref, sweeps):
    """NodeSmoothing flow; returns the ball tables and the flow's results."""
    nv, nt = len(crd), len(tet)
    I = R.Instance()
    I.parameters(64, body("NodeSmoothing/parameters.cl"))
    v = I.mesh(R.GmlVertices, crd, ref)
    I.mesh(R.GmlTetrahedra, tet)
    q = I.solution(R.GmlTetrahedra, 1, R.GmlFlt, b"qal")
    o = I.solution(R.GmlTetrahedra, 4, R.GmlFlt4, b"OptCrd")
    r = I.solution(R.GmlVertices, 1, R.GmlFlt, b"res")
    first = R.lib().refhost_nkernels()
    kq = I.compile(body("NodeSmoothing/quality.cl"), b"quality", R.GmlTetrahedra,
                   [(v, R.GmlReadMode), (q, R.GmlWriteMode)])
    ks = I.compile(body("NodeSmoothing/scatter.cl"), b"scatter", R.GmlTetrahedra,
                   [(v, R.GmlReadMode), (o, R.GmlWriteMode)])
    kg = I.compile(body("NodeSmoothing/gather.cl"), b"gather", R.GmlVertices,
                   [(r, R.GmlWriteMode), (o, R.GmlReadMode | R.GmlVoyeurs),
                    (v, R.GmlReadMode | R.GmlWriteMode)])
    objs = [k for k in R.kernel_objects("gather") if k >= first]
    kobj = [k for k in R.kernel_objects("quality") if k >= first][0]
    sobj = [k for k in R.kernel_objects("scatter") if k >= first][0]
    out = {}
    I.launch(kq)
    out["ns_qal0"] = f32(R.kernel_buffers(kobj)["qalTab"], (nt,))
    for s in range(1, sweeps + 1):
        I.launch(ks)
        I.launch(kg)
        if s == 1:
            out["ns_opt1"] = f32(R.kernel_buffers(sobj)["OptCrdTab"], (nt, 4, 4))
            b = R.kernel_buffers(objs[0])
            out["ns_crd1"] = f32(b["VerCrdTab"], (nv, 4))
            out["ns_res1"] = f32(b["resTab"], (nv,))
    out["ns_crd3"] = f32(R.kernel_buffers(objs[0])["VerCrdTab"], (nv, 4))
    ok, n, w, N, W = I.link_info(R.GmlVertices, R.GmlTetrahedra)
    assert ok == 1
    b0 = R.kernel_buffers(objs[0])
    out["deg"] = i32(b0["VerTetDegTab"], (nv,))
    out["base"] = i32(b0["VerTetBalTab"], (n, w))
    out["n_base"] = n
    out["n_high"] = N
    if N:
        out["high"] = i32(R.kernel_buffers(objs[1])["VerTetBalTab"], (N, W))
    else:
        out["high"] = np.zeros((0, 64), np.int32)
    I.stop()
    return out


def topology(crd, tet, ref):
    I = R.Instance()
    I.mesh(R.GmlVertices, crd, ref)
    I.mesh(R.GmlTetrahedra, tet)
    out = {}
    ne = I.L.GmlExtractEdges(I.g)
    n, e = I.mesh_info(R.GmlEdges)
    assert ne == n
    out["edges"] = I.get_lines(e, n, "ii")[:, :2].astype(np.int32)
    out["numbering"] = np.float32(I.L.GmlEvaluateNumbering(I.g))
    nf = I.L.GmlExtractFaces(I.g)
    n, f = I.mesh_info(R.GmlTriangles)
    assert nf == n
    out["tri"] = I.get_lines(f, n, "iii").astype(np.int32)
    I.stop()
    return out


def mesh_quality(crd, tet, ref, op=R.GmlMin):
    """MeshQuality flow (MeshQuality.c:94-127): the compute_quality body, then
    one reduction, the first of a fresh instance."""
    I = R.Instance()
    I.parameters(64, body("MeshQuality/parameters.cl"))
    v = I.mesh(R.GmlVertices, crd, ref)
    I.mesh(R.GmlTetrahedra, tet)
    q = I.solution(R.GmlTetrahedra, 1, R.GmlFlt, b"qal")
    first = R.lib().refhost_nkernels()
    k = I.compile(body("MeshQuality/compute_quality.cl"), b"quality", R.GmlTetrahedra,
                  [(v, R.GmlReadMode), (q, R.GmlWriteMode)])
    I.launch(k)
    kobj = [x for x in R.kernel_objects("quality") if x >= first][0]
    qal = f32(R.kernel_buffers(kobj)["qalTab"], (len(tet),))
    red = I.reduce(q, op)
    I.stop()
    return qal, red


def make_case(name, src):
    g = dict(np.load(os.path.join(OUT, src)))
    crd, tet, ref = g["crd"], g["tet"], g["ref"]
    out = ball_and_smoothing(crd, tet, ref, 3)
    out.update(topology(crd, tet, ref))
    out["mq_qal"], out["mq_min"] = mesh_quality(crd, tet, ref)
    out["red"] = np.array([mesh_quality(crd, tet, ref, op)[1] for op in range(7)])
    np.savez_compressed(os.path.join(OUT, name), **out)
    print(name, {k: getattr(v, "shape", v) for k, v in out.items()})


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def make_c1():
    import gmlib_gb300 as G
    crd, tet, ref = G.cube_mesh(32, split=0, jitter=0.25, seed=12345)
    out = ball_and_smoothing(crd, tet, ref, 1)
    top = topology(crd, tet, ref)
    qal, mn = mesh_quality(crd, tet, ref)
    res = dict(deg=digest(out["deg"]), base=digest(out["base"]), high=digest(out["high"]),
               edges=digest(top["edges"]), n_base=out["n_base"], n_high=out["n_high"],
               n_edges=len(top["edges"]), n_tri=len(top["tri"]), tri=digest(top["tri"]),
               numbering=top["numbering"], mq_min=mn, mq_argmin=int(np.argmin(qal)),
               mesh=digest(crd) + digest(tet))
    np.savez_compressed(os.path.join(OUT, "refhost_c1.npz"), **res)
    print("refhost_c1.npz", res)


def csr_from_edges(nv, edges):
    """The LinearSolver example's CSR (LinearSolver.c:157-234): per vertex, its
    edge partners in edge order; the diagonal lives in a separate vector."""
    deg = np.zeros(nv + 1, np.int64)
    for j, k in edges:
        deg[j] += 1
        deg[k] += 1
    lin = np.zeros(nv + 1, np.int32)
    lin[1:] = np.cumsum(deg[:nv])
    fill = np.zeros(nv, np.int64)
    col = np.zeros(lin[-1], np.int32)
    for j, k in edges:
        col[lin[j] + fill[j]] = k
        fill[j] += 1
        col[lin[k] + fill[k]] = j
        fill[k] += 1
    return lin, col


def pseudo(shape, salt):
    """Deterministic values in [-1, 1) (a 64-bit LCG step of the index), so
    that tests rebuild the LinearSolver inputs without storing them."""
    n = int(np.prod(shape))
    k = (np.arange(n, dtype=np.uint64) + np.uint64(salt)) * np.uint64(6364136223846793005)
    k = (k + np.uint64(1442695040888963407)) >> np.uint64(40)
    return (k.astype(np.float64) / 8388608.0 - 1.0).reshape(shape)


def linsolve_inputs(nv, nnz, b, dbl):
    """Block values of the LinearSolver flow: off-diagonal and diagonal blocks
    small enough that x <- D x + A x + rhs contracts, x0 and rhs in [-1, 1)."""
    vals = 0.01 * pseudo((nnz, b * b), 11 * b + dbl)
    diag = 0.01 * pseudo((nv, b * b), 13 * b + dbl)
    x0 = pseudo((nv, b), 17 * b + dbl)
    rhs = pseudo((nv, b), 19 * b + dbl)
    if not dbl:
        vals, diag, x0, rhs = (a.astype(np.float32) for a in (vals, diag, x0, rhs))
    return vals, diag, x0, rhs


# (block size, FP64, diagonal product): the reference's GmlMultDiagMatVec
# runs the diagonal vector's own kernel, built with BLKSIZ = b*b
# (gmlib3.c:3626, 1549-1553), whose #else branch is the 5x5 product on
# double-width lines (multdiagmatvec.cl:44-75); it is right for b = 5 only
# and reads and writes past its vectors otherwise, so the b = 4 flows leave
# it out (x1 then stays x0).  b = 7 has no matrix kernels at all
# (multmatvec.cl:1645-1663 defines only the block product), so GmlNewMatrix
# cannot create its slice kernels and the flow cannot run.
LINSOLVE = ((4, 0, 0), (4, 1, 0), (5, 0, 1), (5, 1, 1))


def linsolve_run(mesh, lin, col, b, dbl, use_diag, vals, diag, x0, rhs, iters):
    crd, tet, ref = mesh
    nv = len(crd)
    I = R.Instance()
    L = I.L
    # the mesh, as the example imports it: the norm's "reduction" field is a
    # vertex solution and takes its line count from the vertices
    I.mesh(R.GmlVertices, crd, ref)
    I.mesh(R.GmlTetrahedra, tet)
    fty = R.GmlDbl if dbl else R.GmlFlt
    npt = np.float64 if dbl else np.float32
    first = R.lib().refhost_nkernels()
    A = np.ascontiguousarray(vals, npt)
    mat = L.GmlNewMatrix(I.g, nv, len(col), b, R._p(A), R._p(col), R._p(lin), fty)
    assert mat > 0
    D = np.ascontiguousarray(diag, npt)
    dia = L.GmlNewVector(I.g, nv, b * b, R._p(D), fty)
    X = np.ascontiguousarray(x0, npt)
    xk0 = L.GmlNewVector(I.g, nv, b, R._p(X), fty)
    xk1 = L.GmlNewVector(I.g, nv, b, R._p(X), fty)
    tmp = L.GmlNewVector(I.g, nv, b, R._p(X), fty)
    Bv = np.ascontiguousarray(rhs, npt)
    rhv = L.GmlNewVector(I.g, nv, b, R._p(Bv), fty)
    red = I.solution(R.GmlVertices, 1, R.GmlFlt, b"reduction")
    assert min(dia, xk0, xk1, tmp, rhv) > 0
    norms = []
    for _ in range(iters):
        if use_diag:
            assert L.GmlMultDiagMatVec(I.g, dia, xk0, xk1) == 1
        assert L.GmlMultMatVec(I.g, mat, xk0, tmp) == 1
        assert L.GmlAddVec3(I.g, rhv, tmp, xk1, xk0) == 1
        nrm = ctypes.c_double()
        assert L.GmlNormVec(I.g, xk0, red, ctypes.byref(nrm)) == 1
        norms.append(nrm.value)
    # GmlNewVector builds kernels per vector; GmlAddVec3 runs the first
    # vector's (rhs here), the only AddVec object with bound arguments
    add = [k for k in R.kernel_objects("AddVec") if k >= first and "Y" in R.kernel_buffers(k)][0]
    width = 4 if b <= 4 else 8
    x = np.frombuffer(R.kernel_buffers(add)["Y"], npt)[:nv * width].reshape(nv, width)[:, :b].copy()
    I.stop()
    return np.array(norms), x


def spmv_run(mesh, lin, col, b, dbl, vals, x0):
    """One GmlMultMatVec(mat, y, x) as the first call of a fresh instance:
    the kernel takes (degrees, columns, blocks, B, X) and the library binds
    B = its first vector, X = its second (gmlib3.c:3383-3389), so y = A x."""
    crd, tet, ref = mesh
    nv = len(crd)
    I = R.Instance()
    L = I.L
    I.mesh(R.GmlVertices, crd, ref)
    fty = R.GmlDbl if dbl else R.GmlFlt
    npt = np.float64 if dbl else np.float32
    first = R.lib().refhost_nkernels()
    A = np.ascontiguousarray(vals, npt)
    mat = L.GmlNewMatrix(I.g, nv, len(col), b, R._p(A), R._p(col), R._p(lin), fty)
    X = np.ascontiguousarray(x0, npt)
    Z = np.zeros_like(X)
    y = L.GmlNewVector(I.g, nv, b, R._p(Z), fty)
    x = L.GmlNewVector(I.g, nv, b, R._p(X), fty)
    assert min(mat, y, x) > 0 and L.GmlMultMatVec(I.g, mat, y, x) == 1
    k = [k for k in R.kernel_objects("MulMatVecSlc16") if k >= first][0]
    width = 4 if b <= 4 else 8
    ax = np.frombuffer(R.kernel_buffers(k)["B"], npt)[:nv * width].reshape(nv, width)[:, :b].copy()
    I.stop()
    return ax


def linsolve_mesh():
    import gmlib_gb300 as G
    return G.cube_mesh(7, split=0, jitter=0.1, seed=99)


def make_linsolve():
    crd, tet, ref = linsolve_mesh()
    top = topology(crd, tet, ref)
    nv = len(crd)
    lin, col = csr_from_edges(nv, top["edges"])
    out = dict(mesh=digest(crd) + digest(tet), edges=top["edges"], lin=lin, col=col)
    for b, dbl, use_diag in LINSOLVE:
        vals, diag, x0, rhs = linsolve_inputs(nv, len(col), b, dbl)
        norms, x = linsolve_run((crd, tet, ref), lin, col, b, dbl, use_diag, vals, diag, x0, rhs, 5)
        tag = "b%d_%s" % (b, "f64" if dbl else "f32")
        ax = spmv_run((crd, tet, ref), lin, col, b, dbl, vals, x0)
        out.update({tag + "_norms": norms, tag + "_x": x, tag + "_ax": ax})
        print(tag, norms)
    np.savez_compressed(os.path.join(OUT, "refhost_linsolve.npz"), **out)


TET_FACES = ((1, 2, 3), (2, 0, 3), (3, 0, 1), (0, 2, 1))


def boundary_triangles(crd, tet):
    """The boundary faces of a cube mesh as triangles, each referenced by its
    cube side: 1/2 for x = 0/1, 3/4 for y, 5/6 for z, in tet then face order."""
    seen = {}
    for i, t in enumerate(tet):
        for j, f in enumerate(TET_FACES):
            key = tuple(sorted(t[list(f)]))
            seen[key] = None if key in seen else (i, j)
    tri, ref = [], []
    for key, v in seen.items():
        if v is None:
            continue
        i, j = v
        nodes = tet[i][list(TET_FACES[j])]
        c = crd[nodes, :3]
        for axis in range(3):
            for side in (0, 1):
                if np.all(np.abs(c[:, axis] - side) < 1e-6):
                    ref.append(1 + 2 * axis + side)
        tri.append(nodes)
    return np.array(tri, np.int32), np.array(ref, np.int32)


HEAT_ITERS = 30


def heat_mesh():
    import gmlib_gb300 as G
    crd, tet, ref = G.cube_mesh(4, split=0, jitter=0.2, seed=77)
    tri, tref = boundary_triangles(crd, tet)
    return crd, tet, ref, tri, tref


def heat_parameters():
    """The example's parameter block (HeatCellCentered.c:80): boundary types
    (DIRICHLET 0, NEUMANN 1) of sides 1..6, their references, their values."""
    import struct
    return struct.pack("6i6i6ff", 1, 1, 1, 0, 0, 1, 1, 2, 3, 4, 5, 6,
                       0., 0., 0., 300., 250., 0., 0.)


def make_heat():
    """The HeatCellCentered flow (HeatCellCentered.c:90-180) with the
    example's own kernel bodies: faces, the triangle -> tet shells and tet ->
    triangle links those kernels build, the time step and HEAT_ITERS
    iterations, with the cell values, face values and residual norms (as the
    reference's GmlReduceVector returned them, and over every line)."""
    crd, tet, ref, tri, tref = heat_mesh()
    I = R.Instance()
    par = heat_parameters()
    p = I.parameters(len(par), body("HeatCellCentered/param.cl"))
    ctypes.memmove(p, par, len(par))
    v = I.mesh(R.GmlVertices, crd, ref)
    I.mesh(R.GmlTetrahedra, tet)
    I.mesh(R.GmlTriangles, tri, tref)
    nf = I.L.GmlExtractFaces(I.g)
    ntri, t = I.mesh_info(R.GmlTriangles)
    assert nf == ntri
    faces = I.get_lines(t, ntri, "iii").astype(np.int32)
    nt = len(tet)
    sol = I.solution(R.GmlTetrahedra, 1, R.GmlFlt, b"SolTet")
    grd = I.solution(R.GmlTetrahedra, 1, R.GmlFlt4, b"GrdTet")
    sext = I.solution(R.GmlTriangles, 1, R.GmlFlt, b"SolExt")
    gext = I.solution(R.GmlTriangles, 1, R.GmlFlt4, b"GrdExt")
    rhs = I.solution(R.GmlTetrahedra, 1, R.GmlFlt, b"Rhs")
    dt = I.solution(R.GmlTetrahedra, 1, R.GmlFlt, b"dt")
    first = R.lib().refhost_nkernels()
    K = {}
    K["sol_ext"] = I.compile(body("HeatCellCentered/sol_ext.cl"), b"sol_ext", R.GmlTriangles,
                             [(t, R.GmlReadMode | R.GmlRefFlag), (sol, R.GmlReadMode),
                              (sext, R.GmlWriteMode)])
    K["grd_tet"] = I.compile(body("HeatCellCentered/grd_tet.cl"), b"grd_tet", R.GmlTetrahedra,
                             [(v, R.GmlReadMode), (sext, R.GmlReadMode), (grd, R.GmlWriteMode)])
    K["grd_ext"] = I.compile(body("HeatCellCentered/grd_ext.cl"), b"grd_ext", R.GmlTriangles,
                             [(t, R.GmlReadMode | R.GmlRefFlag), (grd, R.GmlReadMode),
                              (gext, R.GmlWriteMode)])
    K["flx_bal"] = I.compile(body("HeatCellCentered/flx_bal.cl"), b"flx_bal", R.GmlTetrahedra,
                             [(v, R.GmlReadMode), (gext, R.GmlReadMode), (rhs, R.GmlWriteMode)])
    K["tim_int"] = I.compile(body("HeatCellCentered/tim_int.cl"), b"tim_int", R.GmlTetrahedra,
                             [(rhs, R.GmlReadMode), (sol, R.GmlReadMode | R.GmlWriteMode)])
    K["dt"] = I.compile(body("HeatCellCentered/dt.cl"), b"dt", R.GmlTetrahedra,
                        [(v, R.GmlReadMode), (dt, R.GmlWriteMode)])
    obj = {n: [k for k in R.kernel_objects(n) if k >= first][0] for n in K}
    I.launch(K["dt"])
    dtmin = I.reduce(dt, R.GmlMin)
    # GmlPar->dt, then GmlUploadParameters (HeatCellCentered.c:166-169)
    ctypes.memmove(p + 72, np.float32(dtmin).tobytes(), 4)
    assert I.L.GmlUploadParameters(I.g) == 1
    res, exact = [], []
    for _ in range(HEAT_ITERS):
        for n in ("sol_ext", "grd_tet", "grd_ext", "flx_bal", "tim_int"):
            I.launch(K[n])
        res.append(I.reduce(rhs, R.GmlL2))
        # the sum of squares over every line: the reference's reduction
        # drops the last partial work-group (gmlib3.c:3299), and its group
        # size changes while it calibrates
        r32 = np.frombuffer(R.kernel_buffers(obj["flx_bal"])["RhsTab"], np.float32)[:nt]
        exact.append(float(np.sum(r32.astype(np.float64) ** 2)))
    sb = R.kernel_buffers(obj["sol_ext"])
    gb = R.kernel_buffers(obj["grd_tet"])
    out = dict(crd=crd, tet=tet, ref=ref, tri=tri, tref=tref, faces=faces,
               dt=np.float32(dtmin), res=np.array(res), res_exact=np.array(exact),
               sol=f32(R.kernel_buffers(obj["tim_int"])["SolTetTab"], (nt,)),
               sext=f32(sb["SolExtTab"], (ntri,)),
               grd=f32(gb["GrdTetTab"], (nt, 4)))
    # the link tables the kernels read: triangle -> tet shells (entries
    # (tet << 4) | local face, degree per triangle) and tet -> triangle faces
    names = R.kernel_signature(obj["sol_ext"])
    shl = [n for n in names if n.endswith("BalTab")][0]
    deg = [n for n in names if n.endswith("DegTab")][0]
    out["shell"] = np.frombuffer(sb[shl], np.int32)[:2 * ntri].reshape(ntri, 2).copy()
    out["shell_deg"] = np.frombuffer(sb[deg], np.int32)[:ntri].copy()
    lnk = [n for n in R.kernel_signature(obj["grd_tet"]) if n.endswith("LnkTab")][0]
    out["tet_faces"] = np.frombuffer(gb[lnk], np.int32)[:4 * nt].reshape(nt, 4).copy()
    np.savez_compressed(os.path.join(OUT, "refhost_heat.npz"), **out)
    print("refhost_heat.npz", ntri, "faces", shl, deg, lnk, "dt", dtmin, "res", res[0], res[-1])
    I.stop()


EX_ITERS = 3


def examples_mesh():
    import gmlib_gb300 as G
    return G.cube_mesh(5, split=0, jitter=0.2, seed=31)


def square_mesh(n=12, jitter=0.3, seed=8):
    """A jittered n x n square of the z = 0 plane, each cell split into two
    triangles; interior vertices move by up to jitter * h in x and y."""
    rng = np.random.default_rng(seed)
    i, j = np.meshgrid(np.arange(n + 1), np.arange(n + 1), indexing="ij")
    i, j = i.ravel(), j.ravel()
    crd = np.zeros((len(i), 4), np.float32)
    crd[:, 0], crd[:, 1] = i / n, j / n
    inner = (i > 0) & (i < n) & (j > 0) & (j < n)
    crd[inner, :2] += rng.uniform(-jitter / n, jitter / n, (int(inner.sum()), 2)).astype(np.float32)
    tri = []
    for a in range(n):
        for b in range(n):
            p, q, r, s = a * (n + 1) + b, (a + 1) * (n + 1) + b, (a + 1) * (n + 1) + b + 1, a * (n + 1) + b + 1
            tri += [(p, q, r), (p, r, s)]
    return crd, np.array(tri, np.int32)


def make_examples():
    """Three more example flows, with the examples' own bodies, on small
    meshes (the 5^3-hex Kuhn cube, and a 12 x 12 jittered square of
    triangles): GpuBandwidth (gpu_bandwidth.c:100-175), TestFeatures
    (TestFeatures.c:95-215, EX_ITERS iterations with GmlPar->res = i) and
    BallQuality (BallQuality.c:73-130)."""
    crd, tet, ref = examples_mesh()
    nv, nt = len(crd), len(tet)
    out = dict(crd=crd, tet=tet, ref=ref)
    Rd, Wr = R.GmlReadMode, R.GmlWriteMode

    # GpuBandwidth: the four kernels in the example's order
    I = R.Instance()
    I.parameters(8, body("GpuBandwidth/parameters.cl"))
    v = I.mesh(R.GmlVertices, crd, ref)
    t = I.mesh(R.GmlTetrahedra, tet)
    vd = I.solution(R.GmlVertices, 1, R.GmlFlt4, b"VerDat")
    td = I.solution(R.GmlTetrahedra, 1, R.GmlFlt4, b"TetDat")
    first = R.lib().refhost_nkernels()
    ks = [I.compile(body("GpuBandwidth/direct_vertices.cl"), b"direct_vertices", R.GmlVertices,
                    [(v, Rd), (vd, Wr)]),
          I.compile(body("GpuBandwidth/direct_tets.cl"), b"direct_tets", R.GmlTetrahedra,
                    [(t, Rd), (td, Wr)]),
          I.compile(body("GpuBandwidth/indirect_tets.cl"), b"indirect_tets", R.GmlTetrahedra,
                    [(v, Rd), (td, Wr)]),
          I.compile(body("GpuBandwidth/vertices_ball.cl"), b"vertices_ball", R.GmlVertices,
                    [(vd, Wr), (td, Rd)])]
    names = ["direct_vertices", "direct_tets", "indirect_tets", "vertices_ball"]
    obj = {n: [k for k in R.kernel_objects(n) if k >= first][0] for n in names}
    ok, n, w, N, W = I.link_info(R.GmlVertices, R.GmlTetrahedra)
    assert ok == 1 and N == 0, "the ball fits the base table"
    for k, nm, key, dat, shape in zip(ks, names, ["bw_ver", "bw_tet_nodes", "bw_tet_sum", "bw_ball"],
                                      ["VerDatTab", "TetDatTab", "TetDatTab", "VerDatTab"],
                                      [(nv, 4), (nt, 4), (nt, 4), (nv, 4)]):
        I.launch(k)
        out[key] = f32(R.kernel_buffers(obj[nm])[dat], shape)
    I.stop()

    # TestFeatures: neighbours (left out below), the FP64 kernel, downlink,
    # uplink and the residual sum, EX_ITERS times
    I = R.Instance()
    p = I.parameters(8, body("TestFeatures/parameters.cl"))
    v = I.mesh(R.GmlVertices, crd, ref)
    I.mesh(R.GmlTetrahedra, tet)
    sol = I.solution(R.GmlVertices, 2, R.GmlFlt4, b"SolAtVer")
    I.set_lines(sol, np.full((nv, 8), 0.125, np.float32))
    mid = I.solution(R.GmlTetrahedra, 1, R.GmlFlt4, b"TetMid")
    res = I.solution(R.GmlTetrahedra, 1, R.GmlFlt, b"ResVec")
    f64 = I.solution(R.GmlTetrahedra, 1, R.GmlDbl, b"F64Dat")
    first = R.lib().refhost_nkernels()
    kf = I.compile(body("TestFeatures/double_precision.cl"), b"double_precision", R.GmlTetrahedra,
                   [(f64, Rd)])
    kd = I.compile(body("TestFeatures/downlink.cl"), b"downlink", R.GmlTetrahedra,
                   [(v, Rd | R.GmlRefFlag), (sol, Rd), (res, Wr), (mid, Wr)])
    ku = I.compile(body("TestFeatures/uplink.cl"), b"uplink", R.GmlVertices,
                   [(sol, Wr), (mid, Rd | R.GmlVoyeurs)])
    od = [k for k in R.kernel_objects("downlink") if k >= first][0]
    ou = [k for k in R.kernel_objects("uplink") if k >= first][0]
    red, exact, mids, sols = [], [], [], []
    for i in range(1, EX_ITERS + 1):
        ctypes.memmove(p + 4, np.float32(i).tobytes(), 4)     # GmlPar->res
        assert I.L.GmlUploadParameters(I.g) == 1
        I.launch(kf)
        I.launch(kd)
        I.launch(ku)
        red.append(I.reduce(res, R.GmlSum))
        r32 = f32(R.kernel_buffers(od)["ResVecTab"], (nt,))
        exact.append(float(np.sum(r32.astype(np.float64))))
        mids.append(f32(R.kernel_buffers(od)["TetMidTab"], (nt, 4)))
        sols.append(f32(R.kernel_buffers(ou)["SolAtVerTab"], (nv, 2, 4)))
    out.update(ft_mid=np.array(mids), ft_sol=np.array(sols), ft_res=f32(
        R.kernel_buffers(od)["ResVecTab"], (nt,)), ft_red=np.array(red), ft_red_exact=np.array(exact))
    I.stop()

    # BallQuality on the triangle square
    crd2, tri2 = square_mesh()
    I = R.Instance()
    I.parameters(8, body("BallQuality/parameters.cl"))
    v = I.mesh(R.GmlVertices, crd2)
    tr = I.mesh(R.GmlTriangles, tri2)
    tq = I.solution(R.GmlTriangles, 1, R.GmlFlt, b"tq")
    vq = I.solution(R.GmlVertices, 1, R.GmlFlt, b"vq")
    first = R.lib().refhost_nkernels()
    k1 = I.compile(body("BallQuality/triqal.cl"), b"triqal", R.GmlTriangles, [(v, Rd), (tq, Wr)])
    k2 = I.compile(body("BallQuality/verqal.cl"), b"verqal", R.GmlVertices,
                   [(tr, Rd), (tq, Rd), (vq, Wr)])
    I.launch(k1)
    I.launch(k2)
    o1 = [k for k in R.kernel_objects("triqal") if k >= first][0]
    o2 = [k for k in R.kernel_objects("verqal") if k >= first][0]
    out.update(sq_crd=crd2, sq_tri=tri2, bq_tq=f32(R.kernel_buffers(o1)["tqTab"], (len(tri2),)),
               bq_vq=f32(R.kernel_buffers(o2)["vqTab"], (len(crd2),)))
    I.stop()
    np.savez_compressed(os.path.join(OUT, "refhost_examples.npz"), **out)
    print("refhost_examples.npz", {k: getattr(x, "shape", x) for k, x in out.items()},
          "residuals", red, exact)


CASES = {
    "kuhn_n5": lambda: make_case("refhost_kuhn_n5.npz", "kuhn_n5.npz"),
    "reflected_n6": lambda: make_case("refhost_reflected_n6.npz", "reflected_n6.npz"),
    "linsolve": make_linsolve,
    "c1": make_c1,
    "heat": make_heat,
    "examples": make_examples,
}

if __name__ == "__main__":
    if R.lib() is None:
        sys.exit("the reference tree is needed to run the reference host library")
    if len(sys.argv) > 1:
        CASES[sys.argv[1]]()
    else:
        # one process per case: with a vertex degree above the base width the
        # reference writes that vertex's whole ball into its base-table row
        # (gmlib3.c:1126-1129), past the end of the host mirror, which can
        # corrupt the process heap; a fresh process keeps that out of the other
        # cases, and every fixture is read before the process exits
        import subprocess
        for c in CASES:
            subprocess.run([sys.executable, os.path.abspath(__file__), c], check=False)
            print("case", c, "done")
