"""Oracle: CPU restatement of the GMlib mesh-kernel path.

TEST INFRASTRUCTURE.  Only tests/, __graft_entry__.smoke() and the CPU
baseline leg of bench.py use it, as the checker.  The library never imports,
links or calls anything here.

  liboracle.so      C restatement (oracle.c, oracle_mesh.c), FP64
  _ref/librefcl.so  the reference's kernel bodies compiled as C++, built only
                    where the reference tree is present (see build.py)
"""
import ctypes
import os

import numpy as np

from . import build as _build

HERE = os.path.dirname(os.path.abspath(__file__))

_c = None
_r = None


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def lib():
    global _c
    if _c is None:
        _build.build_oracle()
        _c = ctypes.CDLL(_build.LIB)
        _c.orc_quality_ref1.restype = ctypes.c_double
        _c.orc_mean_ratio1.restype = ctypes.c_double
        _c.orc_det1.restype = ctypes.c_double
        _c.orc_reduce.restype = ctypes.c_double
        _c.orc_reduce.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
        _c.orc_rel_residual.restype = ctypes.c_double
        _c.orc_cg.argtypes = [ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 5 + \
            [ctypes.c_double, ctypes.c_int]
    return _c


def refcl():
    """The reference's own kernel bodies on the CPU, or None where the
    reference tree is absent."""
    global _r
    if _r is None:
        path = _build.build_refcl()
        if path is None:
            return None
        _r = ctypes.CDLL(path)
    return _r


# ------------------------------------------------------------------ wrappers

def ver_tet_ball(nv, tet, bal_siz=32, max_siz=64, tables=True):
    tet = np.ascontiguousarray(tet, np.int32)
    nt = len(tet)
    deg = np.zeros(nv, np.int32)
    mp, hs = ctypes.c_int(), ctypes.c_int()
    ok = lib().orc_ver_tet_ball(nv, nt, _ptr(tet), bal_siz, max_siz, _ptr(deg),
                                ctypes.byref(mp), ctypes.byref(hs), None, None)
    if not ok:
        raise ValueError("degree above the maximum link width")
    base = high = None
    if tables:
        base = np.zeros((mp.value + 1, bal_siz), np.int32)
        high = np.zeros((max(nv - mp.value, 0), max(hs.value, 1)), np.int32)
        lib().orc_ver_tet_ball(nv, nt, _ptr(tet), bal_siz, max_siz, _ptr(deg),
                               ctypes.byref(mp), ctypes.byref(hs), _ptr(base),
                               _ptr(high) if hs.value else None)
        if not hs.value:
            high = np.zeros((0, 0), np.int32)
    return deg, mp.value, hs.value, base, high


def tet_edges(tet):
    tet = np.ascontiguousarray(tet, np.int32)
    n = lib().orc_tet_edges(len(tet), _ptr(tet), None)
    e = np.zeros((n, 2), np.int32)
    lib().orc_tet_edges(len(tet), _ptr(tet), _ptr(e))
    return e


def quality_ref(crd, tet):
    crd = np.ascontiguousarray(crd, np.float32)
    tet = np.ascontiguousarray(tet, np.int32)
    q = np.zeros(len(tet), np.float64)
    lib().orc_quality_ref(len(tet), _ptr(crd), _ptr(tet), _ptr(q))
    return q


def mean_ratio(crd, tet):
    crd = np.ascontiguousarray(crd, np.float32)
    tet = np.ascontiguousarray(tet, np.int32)
    q = np.zeros(len(tet), np.float64)
    lib().orc_mean_ratio(len(tet), _ptr(crd), _ptr(tet), _ptr(q))
    return q


def reduce(op, x):
    x = np.ascontiguousarray(x, np.float32)
    return lib().orc_reduce(op, len(x), _ptr(x))


def scatter(crd, tet):
    crd = np.ascontiguousarray(crd, np.float32)
    tet = np.ascontiguousarray(tet, np.int32)
    opt = np.zeros((len(tet), 4, 4), np.float64)
    lib().orc_scatter(len(tet), _ptr(crd), _ptr(tet), _ptr(opt))
    return opt


def gather(crd, deg, ball, opt):
    crd = np.ascontiguousarray(crd, np.float32)
    deg = np.ascontiguousarray(deg, np.int32)
    ball = np.ascontiguousarray(ball, np.int32)
    opt = np.ascontiguousarray(opt, np.float64)
    nv = len(crd)
    new = np.zeros((nv, 4), np.float64)
    res = np.zeros(nv, np.float64)
    lib().orc_gather(nv, _ptr(crd), _ptr(deg), _ptr(ball), ball.shape[1], _ptr(opt),
                     _ptr(new), _ptr(res))
    return new, res


def ball_codes(nv, tet):
    """Full vertex->tet ball (all entries, descending tet order) as a
    (nv, maxdeg) table, built with the reference algorithm."""
    deg, mp, hs, base, high = ver_tet_ball(nv, tet, 32, 64)
    width = max(32, hs)
    full = np.zeros((nv, width), np.int32)
    full[:min(mp, nv), :32] = base[:min(mp, nv)]
    if hs:
        full[mp:, :hs] = high
    return deg, full


# --------------------------------------------------- reference bodies on CPU

def ref_quality(crd, tet):
    r = refcl()
    if r is None:
        return None
    crd = np.ascontiguousarray(crd, np.float32)
    tet = np.ascontiguousarray(tet, np.int32)
    out = np.zeros(len(tet), np.float32)
    r.ref_compute_quality(_ptr(crd), len(tet), _ptr(tet), _ptr(out))
    return out


def ref_scatter(crd, tet):
    r = refcl()
    if r is None:
        return None
    crd = np.ascontiguousarray(crd, np.float32)
    tet = np.ascontiguousarray(tet, np.int32)
    out = np.zeros((len(tet), 4, 4), np.float32)
    r.ref_scatter(_ptr(crd), len(tet), _ptr(tet), _ptr(out))
    return out


def ref_gather(crd, deg, ball, opt):
    r = refcl()
    if r is None:
        return None
    crd = np.array(crd, np.float32, copy=True)
    deg = np.ascontiguousarray(deg, np.int32)
    ball = np.ascontiguousarray(ball, np.int32)
    opt = np.ascontiguousarray(opt, np.float32)
    res = np.zeros(len(crd), np.float32)
    r.ref_gather(_ptr(crd), len(crd), _ptr(deg), _ptr(ball), ball.shape[1], _ptr(opt), _ptr(res))
    return crd, res


def ref_p2_quality(crd, mid, tet, tedg):
    """The reference's P2Quality body on the CPU (float32), or None."""
    r = refcl()
    if r is None:
        return None
    crd = np.ascontiguousarray(crd, np.float32)
    mid = np.ascontiguousarray(mid, np.float32)
    tet = np.ascontiguousarray(tet, np.int32)
    tedg = np.ascontiguousarray(tedg, np.int32)
    out = np.zeros(len(tet), np.float32)
    r.ref_p2_quality(_ptr(crd), _ptr(mid), len(tet), _ptr(tet), _ptr(tedg), _ptr(out))
    return out


def ref_toolkit_table(pts):
    """Every function of the reference's sources/toolkit.cl on point sets
    pts (n, 8, 4) float32, through tests/kernels/toolkit_table.cl: (n, 64)
    float32, or None where the reference tree is absent."""
    r = refcl()
    if r is None:
        return None
    pts = np.ascontiguousarray(pts, np.float32)
    out = np.zeros((len(pts), 64), np.float32)
    r.ref_toolkit_table(_ptr(pts), len(pts), _ptr(out))
    return out


def p2_quality(crd, mid, tet, tedg):
    """FP64 restatement of the P2 quality (orc_p2_quality)."""
    crd = np.ascontiguousarray(crd, np.float32)
    mid = np.ascontiguousarray(mid, np.float32)
    tet = np.ascontiguousarray(tet, np.int32)
    tedg = np.ascontiguousarray(tedg, np.int32)
    q = np.zeros(len(tet), np.float64)
    lib().orc_p2_quality(len(tet), _ptr(tet), _ptr(tedg), _ptr(crd), _ptr(mid), _ptr(q))
    return q


# ------------------------------------------------------ native mesh kernels

def boundary_vertices(nv, tet):
    tet = np.ascontiguousarray(tet, np.int32)
    fixed = np.zeros(nv, np.int32)
    lib().orc_boundary_vertices(nv, len(tet), _ptr(tet), _ptr(fixed))
    return fixed


def point_ball(nv, tet, fixed=None):
    """CSR (ptr, col) of the distinct neighbours of each vertex, ascending;
    fixed vertices get an empty ball."""
    tet = np.ascontiguousarray(tet, np.int32)
    fx = None if fixed is None else np.ascontiguousarray(fixed, np.int32)
    f = lib().orc_point_ball
    f.restype = ctypes.c_longlong
    n = f(nv, len(tet), _ptr(tet), _ptr(fx), None, None, ctypes.c_longlong(0))
    ptr = np.zeros(nv + 1, np.int64)
    col = np.zeros(max(n, 1), np.int32)
    f(nv, len(tet), _ptr(tet), _ptr(fx), _ptr(ptr), _ptr(col), ctypes.c_longlong(n))
    return ptr, col[:n]


def laplace(crd, ptr, col, omega, nsweeps):
    c = np.array(crd, np.float64, copy=True)
    lib().orc_laplace(len(c), _ptr(c), _ptr(np.ascontiguousarray(ptr, np.int64)),
                      _ptr(np.ascontiguousarray(col, np.int32)), ctypes.c_double(omega), nsweeps)
    return c


def quality_stats(crd, tet):
    """Mean-ratio q (FP64, signed by the FP64 determinant), 64-bin histogram,
    inverted flags (bit words) and inverted count."""
    crd = np.ascontiguousarray(crd, np.float32)
    tet = np.ascontiguousarray(tet, np.int32)
    nt = len(tet)
    q = np.zeros(nt, np.float64)
    hist = np.zeros(64, np.uint32)
    flags = np.zeros((nt + 31) // 32, np.uint32)
    ninv = ctypes.c_uint()
    lib().orc_quality_stats(nt, _ptr(crd), _ptr(tet), _ptr(q), _ptr(hist), _ptr(flags),
                            ctypes.byref(ninv))
    return q, hist, flags, ninv.value


# ------------------------------------------------------------ block algebra

def _bsr_args(lin, col, val):
    lin = np.ascontiguousarray(lin, np.int32)
    col = np.ascontiguousarray(col, np.int32)
    val = np.ascontiguousarray(val, np.float64)
    b = val.shape[-1]
    return lin, col, val, b


def bsr_spmv(lin, col, val, x):
    """y = A x (FP64, long-double accumulation); val is [nnzb, b, b]."""
    lin, col, val, b = _bsr_args(lin, col, val)
    nrow = len(lin) - 1
    x = np.ascontiguousarray(x, np.float64).reshape(nrow, b)
    y = np.zeros((nrow, b), np.float64)
    lib().orc_bsr_spmv(nrow, b, _ptr(lin), _ptr(col), _ptr(val), _ptr(x), _ptr(y))
    return y


def rel_residual(lin, col, val, rhs, x):
    lin, col, val, b = _bsr_args(lin, col, val)
    nrow = len(lin) - 1
    rhs = np.ascontiguousarray(rhs, np.float64)
    x = np.ascontiguousarray(x, np.float64)
    return lib().orc_rel_residual(nrow, b, _ptr(lin), _ptr(col), _ptr(val), _ptr(rhs), _ptr(x))


def cg(lin, col, val, rhs, tol, maxit):
    """FP64 CG from x = 0; returns (x, iterations)."""
    lin, col, val, b = _bsr_args(lin, col, val)
    nrow = len(lin) - 1
    rhs = np.ascontiguousarray(rhs, np.float64)
    x = np.zeros((nrow, b), np.float64)
    it = lib().orc_cg(nrow, b, _ptr(lin), _ptr(col), _ptr(val), _ptr(rhs), _ptr(x),
                      float(tol), int(maxit))
    return x, it


# ------------------------------------------------------------ face extraction

# local face nodes and face sizes per element type (sources/gmlib3.c:342-358)
FACE_NODES = {
    2: [(0, 1, 2)],
    3: [(0, 1, 2, 3)],
    4: [(1, 2, 3), (2, 0, 3), (3, 0, 1), (0, 2, 1)],
    5: [(0, 1, 4), (1, 2, 4), (2, 3, 4), (3, 0, 4), (3, 2, 1, 0)],
    6: [(0, 2, 1), (3, 4, 5), (0, 1, 4, 3), (1, 2, 5, 4), (3, 5, 2, 0)],
    7: [(0, 4, 7, 3), (1, 2, 6, 5), (0, 1, 5, 4), (3, 7, 6, 2), (0, 3, 2, 1), (4, 5, 6, 7)],
}


def extract_faces(elements, quad_ref_quirk=False):
    """Restatement of GmlExtractFaces (sources/gmlib3.c:3880-4171), pure
    Python for small meshes.  elements: {type: (nodes [n, k], refs [n])}
    for types 2 (triangles) .. 7 (hexahedra).  Faces are visited type by
    type, element by element, face by face; the first visit of a sorted
    node tuple defines the face (sorted nodes, the element's reference for
    existing triangles / quadrilaterals, 0 otherwise).  With quad_ref_quirk
    an existing quadrilateral gets its fourth node as reference, as the
    reference code does (:4093).  Returns (triangles [n, 4], quads [n, 5])
    with the reference in the last column."""
    seen = [dict(), dict()]
    out = [[], []]
    for typ in range(2, 8):
        if typ not in elements:
            continue
        nodes, refs = elements[typ]
        for i in range(len(nodes)):
            for loc in FACE_NODES[typ]:
                key = tuple(sorted(int(nodes[i][c]) for c in loc))
                k = len(key) == 4
                if key in seen[k]:
                    continue
                seen[k][key] = len(out[k])
                if typ in (2, 3):
                    r = int(refs[i])
                    if k and quad_ref_quirk:
                        r = int(nodes[i][3])
                else:
                    r = 0
                out[k].append(list(key) + [r])
    tri = np.array(out[0], np.int32).reshape(-1, 4)
    qad = np.array(out[1], np.int32).reshape(-1, 5)
    return tri, qad
