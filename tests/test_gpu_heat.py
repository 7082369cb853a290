"""The HeatCellCentered flow (face shells) on the GPU against the reference's
own run of it (tests/golden/refhost_heat.npz, made by make_refhost.py from
examples/HeatCellCentered with the reference's kernel bodies).

A 4^3-hex Kuhn cube with its boundary triangles referenced by cube side:
  - GmlExtractFaces keeps the boundary triangles first and adds the inner
    ones, bit for bit as the reference;
  - the triangle -> tet shells (two entries, the second empty on the
    boundary) and the tet -> triangle face links, read by probe kernels, are
    the reference's tables;
  - the flow itself, with this project's statements of the same six bodies
    (tests/kernels/heat_*.cl): the time step within 1e-5, and after 30
    explicit steps the cell values within 1e-4 of their range, the face
    values likewise, the residual norms (sums of squares over every cell)
    within 1e-3 relative (FP32 on both sides; pow and the FMA contractions
    differ in the last bits)."""
import ctypes
import importlib.util
import os
import struct

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
KDIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "kernels")
PARAM = (b"enum { DIRICHLET, NEUMANN };\n"
         b"typedef struct {\n   int BoCo[6];\n   int BoCo_Ref[6];\n   float BoCo_Val[6];\n"
         b"   float dt;\n}GmlParSct;\n")


def body(name):
    with open(os.path.join(KDIR, name), "rb") as f:
        return f.read()


def set_elements(G, g, typ, nodes, refs):
    n, k = nodes.shape
    idx = G.lib.GmlNewMeshData(g, typ, n)
    assert idx > 0
    a = np.ascontiguousarray(nodes, np.int32)
    r = np.ascontiguousarray(refs, np.int32)
    IP = ctypes.POINTER(ctypes.c_int)
    assert G.lib.GmlSetDataBlock(g, typ, 0, n - 1, ctypes.c_void_p(a.ctypes.data),
                                 ctypes.c_void_p(a.ctypes.data + (n - 1) * a.strides[0]),
                                 r.ctypes.data_as(IP),
                                 ctypes.cast(r.ctypes.data + (n - 1) * 4, IP)) == 1
    G.lib.GmlxSynchronize(g)
    return idx


def test_heat_cell_centered_flow(G, gpu):
    r = dict(np.load(os.path.join(GOLD, "refhost_heat.npz")))
    spec = importlib.util.spec_from_file_location("mk", os.path.join(GOLD, "make_refhost.py"))
    mk = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mk)
    g = gpu
    par = mk.heat_parameters()
    p = G.lib.GmlNewParameters(g, len(par), PARAM)
    assert p
    ctypes.memmove(p, par, len(par))
    assert G.lib.GmlUploadParameters(g) == 1
    v, t = G.upload_mesh(g, r["crd"], r["tet"], r["ref"])
    set_elements(G, g, G.GmlTriangles, r["tri"], r["tref"])
    nf = G.lib.GmlExtractFaces(g)
    nl, ti = ctypes.c_int(), ctypes.c_int()
    assert G.lib.GmlGetMeshInfo(g, G.GmlTriangles, ctypes.byref(nl), ctypes.byref(ti)) == 1
    ntri, tri = nl.value, ti.value
    assert nf == ntri == len(r["faces"])
    faces = G.get_data(g, tri, np.int32, (ntri, 4))[:, :3]
    frefs = G.get_data(g, tri + 1, np.int32, (ntri,))
    assert np.array_equal(np.column_stack([faces, frefs]), r["faces"])
    nt = len(r["tet"])

    # the link tables, through probe kernels
    tnum = G.lib.GmlNewSolutionData(g, G.GmlTetrahedra, 1, G.GmlFlt, b"TetNum")
    rnum = G.lib.GmlNewSolutionData(g, G.GmlTriangles, 1, G.GmlFlt, b"TriNum")
    shl = G.lib.GmlNewSolutionData(g, G.GmlTriangles, 1, G.GmlFlt4, b"ShlTet")
    tft = G.lib.GmlNewSolutionData(g, G.GmlTetrahedra, 1, G.GmlFlt4, b"TetTri")
    G.set_data(g, tnum, np.arange(1, nt + 1, dtype=np.float32))
    G.set_data(g, rnum, np.arange(1, ntri + 1, dtype=np.float32))
    k1 = G.compile_kernel(g, body("shell_probe.cl"), "shell_probe", G.GmlTriangles,
                          [(tnum, G.GmlReadMode, 0), (shl, G.GmlWriteMode, 0)])
    k2 = G.compile_kernel(g, body("face_probe.cl"), "face_probe", G.GmlTetrahedra,
                          [(rnum, G.GmlReadMode, 0), (tft, G.GmlWriteMode, 0)])
    assert k1 > 0 and k2 > 0
    assert G.lib.GmlLaunchKernel(g, k1) == 1 and G.lib.GmlLaunchKernel(g, k2) == 1
    sh = G.get_data(g, shl, np.float32, (ntri, 4))
    deg = r["shell_deg"]
    want = np.where(np.arange(2)[None, :] < deg[:, None], (r["shell"] >> 4) + 1, 0)
    assert np.array_equal(sh[:, 2].astype(np.int32), deg)
    assert np.array_equal(sh[:, :2].astype(np.int64), want)
    tf = G.get_data(g, tft, np.float32, (nt, 4))
    assert np.array_equal(tf.astype(np.int64), r["tet_faces"] + 1)

    # the flow
    sol = G.lib.GmlNewSolutionData(g, G.GmlTetrahedra, 1, G.GmlFlt, b"SolTet")
    grd = G.lib.GmlNewSolutionData(g, G.GmlTetrahedra, 1, G.GmlFlt4, b"GrdTet")
    sext = G.lib.GmlNewSolutionData(g, G.GmlTriangles, 1, G.GmlFlt, b"SolExt")
    gext = G.lib.GmlNewSolutionData(g, G.GmlTriangles, 1, G.GmlFlt4, b"GrdExt")
    rhs = G.lib.GmlNewSolutionData(g, G.GmlTetrahedra, 1, G.GmlFlt, b"Rhs")
    dt = G.lib.GmlNewSolutionData(g, G.GmlTetrahedra, 1, G.GmlFlt, b"dt")
    for idx, shape in ((sol, nt), (grd, (nt, 4)), (sext, ntri), (gext, (ntri, 4)), (rhs, nt)):
        G.set_data(g, idx, np.zeros(shape, np.float32))
    R, W, RF = G.GmlReadMode, G.GmlWriteMode, G.GmlRefFlag
    ks = [G.compile_kernel(g, body("heat_face_value.cl"), "sol_ext", G.GmlTriangles,
                           [(tri, R | RF, 0), (sol, R, 0), (sext, W, 0)]),
          G.compile_kernel(g, body("heat_cell_gradient.cl"), "grd_tet", G.GmlTetrahedra,
                           [(v, R, 0), (sext, R, 0), (grd, W, 0)]),
          G.compile_kernel(g, body("heat_face_gradient.cl"), "grd_ext", G.GmlTriangles,
                           [(tri, R | RF, 0), (grd, R, 0), (gext, W, 0)]),
          G.compile_kernel(g, body("heat_flux_balance.cl"), "flx_bal", G.GmlTetrahedra,
                           [(v, R, 0), (gext, R, 0), (rhs, W, 0)]),
          G.compile_kernel(g, body("heat_step.cl"), "tim_int", G.GmlTetrahedra,
                           [(rhs, R, 0), (sol, R | W, 0)])]
    kdt = G.compile_kernel(g, body("heat_dt.cl"), "dt", G.GmlTetrahedra, [(v, R, 0), (dt, W, 0)])
    assert min(ks) > 0 and kdt > 0
    assert G.lib.GmlLaunchKernel(g, kdt) == 1
    mydt = G.reduce(g, dt, G.GmlMin)
    assert abs(mydt - float(r["dt"])) <= 1e-5 * float(r["dt"])
    # the step the reference used, so that both runs integrate the same ODE
    ctypes.memmove(p + 72, struct.pack("f", float(r["dt"])), 4)
    assert G.lib.GmlUploadParameters(g) == 1
    res = []
    for _ in range(len(r["res"])):
        for k in ks:
            assert G.lib.GmlLaunchKernel(g, k) == 1
        res.append(G.reduce(g, rhs, G.GmlL2))
    # the residual over every line (the reference's own reduction drops the
    # last partial work-group: r["res"] is kept for the record)
    assert np.allclose(res, r["res_exact"], rtol=1e-3, atol=0)
    s = G.get_data(g, sol, np.float32, nt)
    span = float(np.ptp(r["sol"])) or 1.0
    assert np.max(np.abs(s - r["sol"])) <= 1e-4 * span
    se = G.get_data(g, sext, np.float32, ntri)
    assert np.max(np.abs(se - r["sext"])) <= 1e-4 * max(span, float(np.ptp(r["sext"])))
