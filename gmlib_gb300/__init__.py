"""Python access to libgmlib3.so, the GB300-native GMlib.

The product is the C library (include/gmlib3.h is the drop-in interface of
the reference, include/gmlib3_gb300.h the extensions).  This module loads it
with ctypes, declares argument types for every exported entry point, and adds
a few numpy conveniences used by the tests and the benchmark.  There is no
fallback: if the library is missing, importing `lib` raises.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
# GML_LIB overrides the library path (tuning builds made with build(out=...))
LIB_PATH = os.environ.get("GML_LIB") or os.path.join(_HERE, "libgmlib3.so")

# enums of gmlib3.h
GmlVertices, GmlEdges, GmlTriangles, GmlQuadrilaterals, GmlTetrahedra, \
    GmlPyramids, GmlPrisms, GmlHexahedra = range(8)
GmlInt, GmlInt2, GmlInt4, GmlInt8, GmlInt16, GmlFlt, GmlFlt2, GmlFlt4, GmlFlt8, \
    GmlFlt16, GmlDbl, GmlDbl2, GmlDbl4, GmlDbl8, GmlDbl16 = range(15)
GmlMin, GmlMax, GmlSum, GmlL0, GmlL1, GmlL2, GmlLinf = range(7)
GmlRefFlag, GmlReadMode, GmlWriteMode, GmlVoyeurs, GmlManual = 1, 2, 4, 8, 16

_s = ctypes.c_size_t
_i = ctypes.c_int
_d = ctypes.c_double
_f = ctypes.c_float
_p = ctypes.c_void_p
_cp = ctypes.c_char_p
_ip = ctypes.POINTER(ctypes.c_int)
_fp = ctypes.POINTER(ctypes.c_float)
_dp = ctypes.POINTER(ctypes.c_double)

# name: (restype, argtypes); variadic entry points are declared without
# argtypes and called through their non-variadic Gmlx forms.
SIGNATURES = {
    "GmlInit": (_s, [_i]),
    "GmlStop": (None, [_s]),
    "GmlListGPU": (None, []),
    "GmlNewParameters": (_p, [_s, _i, _cp]),
    "GmlNewMeshData": (_i, [_s, _i, _i]),
    "GmlNewSolutionData": (_i, [_s, _i, _i, _i, _cp]),
    "GmlNewLinkData": (_i, [_s, _i, _i, _i, _cp]),
    "GmlNewMatrix": (_i, [_s, _i, _i, _i, _p, _ip, _ip, _i]),
    "GmlNewVector": (_i, [_s, _i, _i, _p, _i]),
    "GmlFreeData": (_i, [_s, _i]),
    "GmlSetDataLine": (_i, None),
    "GmlGetDataLine": (_i, None),
    "GmlSetCompilerOptions": (None, [_s, _cp]),
    "GmlCompileKernel": (_i, None),
    "GmlLaunchKernel": (_i, [_s, _i]),
    "GmlReduceVector": (_i, [_s, _i, _i, _dp]),
    "GmlGetMemoryUsage": (_s, [_s]),
    "GmlGetMemoryTransfer": (_s, [_s]),
    "GmlGetMemoryAccess": (_f, [_s]),
    "GmlGetFlops": (_f, [_s]),
    "GmlDebugOn": (None, [_s]),
    "GmlDebugOff": (None, [_s]),
    "GmlExtractEdges": (_i, [_s]),
    "GmlExtractFaces": (_i, [_s]),
    "GmlSetNeighbours": (_i, [_s, _i]),
    "GmlCheckFP64": (_i, [_s]),
    "GmlGetMeshInfo": (_i, [_s, _i, _ip, _ip]),
    "GmlGetLinkInfo": (_i, [_s, _i, _i, _ip, _ip, _ip, _ip]),
    "GmlSetDataBlock": (_i, [_s, _i, _i, _i, _p, _p, _ip, _ip]),
    "GmlGetDataBlock": (_i, [_s, _i, _i, _i, _p, _p, _ip, _ip]),
    "GmlGetKernelRunTime": (_d, [_s, _i]),
    "GmlGetReduceRunTime": (_d, [_s, _i]),
    "GmlGetWallClock": (_d, []),
    "GmlUploadParameters": (_i, [_s]),
    "GmlDownloadParameters": (_i, [_s]),
    "GmlEvaluateNumbering": (_f, [_s]),
    "GmlIncludeUserToolkit": (None, [_s, _cp]),
    "GmlMultMatVec": (_i, [_s, _i, _i, _i]),
    "GmlMultDiagMatVec": (_i, [_s, _i, _i, _i]),
    "GmlAddVec3": (_i, [_s, _i, _i, _i, _i]),
    "GmlScaleVec": (_i, [_s, _i, _dp]),
    "GmlNormVec": (_i, [_s, _i, _i, _dp]),
    # extensions (gmlib3_gb300.h)
    "GmlxInitOffline": (_s, []),
    "GmlxSetTiming": (_i, [_s, _i]),
    "GmlxSetTuning": (_i, [_s, _i, _i]),
    "GmlxKernelBlockSize": (_i, [_s, _i]),
    "GmlxKernelSource": (_cp, [_s, _i]),
    "GmlxKernelIsLazy": (_i, [_s, _i]),
    "GmlxKernelRegisters": (_i, [_s, _i]),
    "GmlxSetLazy": (_i, [_s, _i]),
    "GmlxLinkData": (_i, [_s, _i, _i, _ip, _ip, _ip]),
    "GmlxSynchronize": (_i, [_s]),
    "GmlxStream": (_p, [_s]),
    "GmlxCompileKernelV": (_i, [_s, _cp, _cp, _i, _i, _ip, _ip, _ip]),
    "GmlxSetData": (_i, [_s, _i, _p, _s]),
    "GmlxGetData": (_i, [_s, _i, _p, _s]),
    "GmlxDataBytes": (_s, [_s, _i]),
    "GmlxDataLines": (_i, [_s, _i]),
    "GmlxDevicePtr": (_p, [_s, _i]),
    "GmlxReduceArg": (_i, [_s, _i, _fp, _ip, _fp, _ip]),
    "GmlxCubeSizes": (None, [_i, _ip, _ip]),
    "GmlxCubeMesh": (_i, [_i, _i, _d, ctypes.c_uint64, _p, _p, _p]),
    "GmlxHilbertRenumber": (_i, [_i, _p, _p, _i, _p, _p]),
    "GmlxDegreeSort": (_i, [_i, _p, _p, _i, _p, _i, _p]),
}


class GmlxQuality(ctypes.Structure):
    _fields_ = [("MinQal", ctypes.c_float), ("MaxQal", ctypes.c_float),
                ("MinIdx", ctypes.c_int), ("MaxIdx", ctypes.c_int),
                ("SumQal", ctypes.c_double), ("NmbInv", ctypes.c_uint),
                ("NmbF64", ctypes.c_uint), ("Hist", ctypes.c_uint * 64)]


_qp = ctypes.POINTER(GmlxQuality)
_llp = ctypes.POINTER(ctypes.c_longlong)
SIGNATURES.update({
    "GmlxMeshSetup": (_i, [_s, _i]),
    "GmlxMeshBallInfo": (_i, [_s, _llp, _llp, _ip]),
    "GmlxSmooth": (_i, [_s, _i, _f]),
    "GmlxQualityStats": (_i, [_s, _d, _i, _qp]),
    "GmlxInvertedFlags": (_i, [_s, _p, _s]),
    "GmlxSmoothQualityLoop": (_i, [_s, _i, _f, _d, _qp]),
    "GmlxMeshBytes": (_i, [_s, _dp, _dp]),
    "GmlxEventCreate": (_p, []),
    "GmlxEventRecord": (_i, [_s, _p]),
    "GmlxEventElapsed": (_d, [_p, _p]),
    "GmlxEventDestroy": (None, [_p]),
    "GmlxReduceNoAlloc": (_i, [_p, _s, _i, _dp, _p]),
})


class GmlxSolveInfo(ctypes.Structure):
    _fields_ = [("NmbIte", ctypes.c_int), ("NmbOut", ctypes.c_int),
                ("RelRes", ctypes.c_double), ("Seconds", ctypes.c_double)]


GmlxCgFp64, GmlxCgMixed = 0, 1
GmlxBatchQueue, GmlxBatchLoop = 0, 1
GmlxReqQuality, GmlxReqSmooth, GmlxReqSolve = 0, 1, 2
GmlxServeBatching, GmlxServeSerial = 0, 1


class GmlxRequest(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("target", ctypes.c_int), ("arrival", ctypes.c_double),
                ("start", ctypes.c_double), ("finish", ctypes.c_double),
                ("status", ctypes.c_int), ("NmbIte", ctypes.c_int), ("RelRes", ctypes.c_double),
                ("qal", GmlxQuality)]


class GmlxServeStats(ctypes.Structure):
    _fields_ = [("completed", ctypes.c_int), ("failed", ctypes.c_int), ("loads", ctypes.c_int),
                ("evictions", ctypes.c_int), ("seconds", ctypes.c_double),
                ("throughput", ctypes.c_double), ("mean", ctypes.c_double),
                ("p50", ctypes.c_double), ("p99", ctypes.c_double), ("max", ctypes.c_double),
                ("peak_bytes", ctypes.c_double)]
SIGNATURES.update({
    "GmlxSolveCG": (_i, [_s, _i, _i, _i, _i, _d, _i, ctypes.POINTER(GmlxSolveInfo)]),
    "GmlxCubeSpdSizes": (_i, [_i, _i, _ip, _ip]),
    "GmlxVectorData": (_i, [_s, _i]),
    "GmlxImportMesh": (_i, [_s, _cp, _i, _ip]),
    "GmlxExportMesh": (_i, [_s, _cp, _i, _ip]),
    "GmlxExportSolution": (_i, [_s, _cp, _i, _ip]),
    "GmlxBatchCreate": (_i, [_s, _i, _p, _p, _p]),
    "GmlxBatchSetMesh": (_i, [_s, _i, _p, _p, _p]),
    "GmlxBatchSetup": (_i, [_s, _i]),
    "GmlxBatchRun": (_i, [_s, _i, _f, _i, ctypes.POINTER(GmlxQuality)]),
    "GmlxBatchGetMesh": (_i, [_s, _i, _p]),
    "GmlxBatchFlags": (_i, [_s, _i, _p, _s]),
    "GmlxBatchTune": (_i, [_s, _i, _f]),
    "GmlxBatchSetTiles": (_i, [_s, _i, _i, _i, _i]),
    "GmlxSetBallWindow": (_i, [_s, _i]),
    "GmlxBallWindow": (_i, [_s]),
    "GmlxMeshTune": (_i, [_s, _i, ctypes.c_float]),
    "GmlxBatchSetWaitLimit": (_i, [_s, _i, _i]),
    "GmlxBatchInfo": (_i, [_s, _ip, _ip, _ip, _ip, _ip]),
    "GmlxServeNew": (_s, [_i, _d, _i]),
    "GmlxServeAddMesh": (_i, [_s, _i, _p, _p, _i, _p, _d]),
    "GmlxServeAddSystem": (_i, [_s, _i, _i, _p, _p, _p, _p]),
    "GmlxServeRun": (_i, [_s, _p, _i, _i, _p]),
    "GmlxServeResident": (_i, [_s, _dp]),
    "GmlxServeTargetBytes": (_d, [_s, _i]),
    "GmlxServeFree": (None, [_s]),
    "GmlxCubeSpdMatrix": (_i, [_i, _i, ctypes.c_uint64, _p, _p, _p, _p]),
})


def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError("libgmlib3.so is not built: run `python -m gmlib_gb300.build` "
                          "or __graft_entry__.build()")
    h = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(h, name, None)
        if fn is None:
            continue
        fn.restype = res
        if args is not None:
            fn.argtypes = args
    return h


class _Lazy:
    _h = None

    def __getattr__(self, name):
        if _Lazy._h is None:
            _Lazy._h = _load()
        return getattr(_Lazy._h, name)


lib = _Lazy()


def exported_symbols():
    """Names declared by SIGNATURES (the public C ABI)."""
    return sorted(SIGNATURES)


# ---------------------------------------------------------------- helpers

def as_ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


def cube_mesh(n, split=0, jitter=0.25, seed=12345, hilbert=True, degree_sort=0):
    """Jittered n^3-hex cube split in 6 tets per hex (library generator),
    Hilbert renumbered; degree_sort > 0 then puts the vertices in at most
    that many tets first (GmlxDegreeSort)."""
    nv, nt = ctypes.c_int(), ctypes.c_int()
    lib.GmlxCubeSizes(n, ctypes.byref(nv), ctypes.byref(nt))
    crd = np.zeros((nv.value, 4), np.float32)
    tet = np.zeros((nt.value, 4), np.int32)
    ref = np.zeros(nv.value, np.int32)
    lib.GmlxCubeMesh(n, split, float(jitter), int(seed), as_ptr(crd), as_ptr(tet), as_ptr(ref))
    if hilbert:
        lib.GmlxHilbertRenumber(nv.value, as_ptr(crd), as_ptr(ref), nt.value, as_ptr(tet), None)
    if degree_sort > 0 and lib.GmlxDegreeSort(nv.value, as_ptr(crd), as_ptr(ref), nt.value,
                                              as_ptr(tet), degree_sort, None) < 0:
        raise RuntimeError("GmlxDegreeSort failed")
    return crd, tet, ref


# local edges of a tetrahedron, in the order of the library's edge table
TET_EDGES = ((0, 1), (1, 2), (2, 0), (3, 0), (3, 1), (3, 2))


def p2_mesh(n, split=0, jitter=0.2, curve=0.15, seed=12345):
    """Quadratic (P2) tetrahedra on the jittered n^3-hex cube: the unique
    edges (ascending vertex pairs, sorted), one mid-edge node per edge (the
    midpoint moved by up to curve * h in each coordinate, seeded) and the
    tet -> edge table in TET_EDGES order.
    Returns crd (nv,4), tet (nt,4), edges (ne,2), mid (ne,4), tedg (nt,6)."""
    crd, tet, _ = cube_mesh(n, split=split, jitter=jitter, seed=seed)
    nv = len(crd)
    loc = np.array(TET_EDGES, np.int64)
    a = tet[:, loc[:, 0]].astype(np.int64)
    b = tet[:, loc[:, 1]].astype(np.int64)
    key = np.minimum(a, b) * nv + np.maximum(a, b)
    uniq, inv = np.unique(key.ravel(), return_inverse=True)
    edges = np.stack([uniq // nv, uniq % nv], axis=1).astype(np.int32)
    rng = np.random.default_rng(seed + 1)
    mid = np.zeros((len(edges), 4), np.float32)
    mid[:, :3] = 0.5 * (crd[edges[:, 0], :3] + crd[edges[:, 1], :3])
    mid[:, :3] += (curve / n) * rng.uniform(-1.0, 1.0, (len(edges), 3)).astype(np.float32)
    return crd, tet, edges, mid, inv.reshape(len(tet), 6).astype(np.int32)


def p2_body():
    """The P2 tetrahedron quality as a GMlib-dialect kernel body
    (kernels/p2_quality.cl): reads VerCrd[4] and MidCrd[6..8], writes qal."""
    with open(os.path.join(_HERE, "kernels", "p2_quality.cl"), "rb") as f:
        return f.read()


def mean_ratio_body():
    """The mean-ratio tetrahedron quality as a GMlib-dialect kernel body
    (kernels/mean_ratio.cl): reads VerCrd[4], writes qal."""
    with open(os.path.join(_HERE, "kernels", "mean_ratio.cl"), "rb") as f:
        return f.read()


def compile_kernel(g, src, name, msh, dats):
    """dats: list of (index, flags, link) triplets."""
    n = len(dats)
    I = ctypes.c_int * n
    idx = I(*[d[0] for d in dats])
    flg = I(*[d[1] for d in dats])
    lnk = I(*[d[2] for d in dats])
    if isinstance(src, str):
        src = src.encode()
    return lib.GmlxCompileKernelV(g, src, name.encode(), msh, n, idx, flg, lnk)


def set_data(g, idx, arr):
    arr = np.ascontiguousarray(arr)
    return lib.GmlxSetData(g, idx, as_ptr(arr), arr.nbytes)


def get_data(g, idx, dtype, shape):
    out = np.empty(shape, dtype)
    ok = lib.GmlxGetData(g, idx, as_ptr(out), out.nbytes)
    if not ok:
        raise RuntimeError("GmlxGetData failed for datatype %d" % idx)
    return out


def cube_spd(n, split=0, seed=7):
    """Block CSR system of GmlxCubeSpdMatrix: (lin, col, val[nnzb,3,3], rhs[nv,3])."""
    nl, nb = ctypes.c_int(), ctypes.c_int()
    if not lib.GmlxCubeSpdSizes(n, split, ctypes.byref(nl), ctypes.byref(nb)):
        raise ValueError("bad cube size")
    lin = np.zeros(nl.value + 1, np.int32)
    col = np.zeros(nb.value, np.int32)
    val = np.zeros((nb.value, 3, 3), np.float64)
    rhs = np.zeros((nl.value, 3), np.float64)
    if not lib.GmlxCubeSpdMatrix(n, split, int(seed), as_ptr(lin), as_ptr(col), as_ptr(val),
                                 as_ptr(rhs)):
        raise RuntimeError("GmlxCubeSpdMatrix failed")
    return lin, col, val, rhs


def upload_mesh(g, crd, tet, ref=None):
    """Create vertex and tetrahedron datatypes and upload them (GmlSetDataBlock)."""
    nv, nt = len(crd), len(tet)
    vidx = lib.GmlNewMeshData(g, GmlVertices, nv)
    tidx = lib.GmlNewMeshData(g, GmlTetrahedra, nt)
    if not vidx or not tidx:
        raise RuntimeError("GmlNewMeshData failed")
    crd = np.ascontiguousarray(crd, np.float32)
    tet = np.ascontiguousarray(tet, np.int32)
    vref = np.ascontiguousarray(ref if ref is not None else np.zeros(nv), np.int32)
    tref = np.zeros(nt, np.int32)
    base = crd.ctypes.data
    rc = lib.GmlSetDataBlock(g, GmlVertices, 0, nv - 1, ctypes.c_void_p(base),
                             ctypes.c_void_p(base + (nv - 1) * crd.strides[0]),
                             vref.ctypes.data_as(_ip),
                             ctypes.cast(vref.ctypes.data + (nv - 1) * 4, _ip))
    if rc != 1:
        raise RuntimeError("GmlSetDataBlock(vertices) failed")
    base = tet.ctypes.data
    rc = lib.GmlSetDataBlock(g, GmlTetrahedra, 0, nt - 1, ctypes.c_void_p(base),
                             ctypes.c_void_p(base + (nt - 1) * tet.strides[0]),
                             tref.ctypes.data_as(_ip),
                             ctypes.cast(tref.ctypes.data + (nt - 1) * 4, _ip))
    if rc != 1:
        raise RuntimeError("GmlSetDataBlock(tets) failed")
    # keep the host arrays alive until the asynchronous upload is done
    lib.GmlxSynchronize(g)
    return vidx, tidx


def upload_p2(g, crd, tet, edges, mid):
    """The data of the reference's P2Quality example: vertices and tets,
    the edges (GmlEdges lines) and the mid-edge nodes as an edge solution
    named MidCrd.  Returns (vertex, tet, edge, MidCrd) indices."""
    vidx, tidx = upload_mesh(g, crd, tet)
    eidx = lib.GmlNewMeshData(g, GmlEdges, len(edges))
    midx = lib.GmlNewSolutionData(g, GmlEdges, 1, GmlFlt4, b"MidCrd")
    if not eidx or not midx:
        raise RuntimeError("edge datatypes could not be created")
    if not set_data(g, eidx, np.ascontiguousarray(edges, np.int32)) \
       or not set_data(g, midx, np.ascontiguousarray(mid, np.float32)):
        raise RuntimeError("edge upload failed")
    lib.GmlxSynchronize(g)
    return vidx, tidx, eidx, midx


def reduce(g, idx, op):
    r = ctypes.c_double()
    rc = lib.GmlReduceVector(g, idx, op, ctypes.byref(r))
    if rc != 1:
        raise RuntimeError("GmlReduceVector returned %d" % rc)
    return r.value
