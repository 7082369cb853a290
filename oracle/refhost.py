"""The reference's host library run on the CPU (test infrastructure).

oracle/_ref/librefhost.so is the unmodified sources/gmlib3.c of the
reference, compiled against the OpenCL stand-in header and linked with the
host-CPU OpenCL runtime of oracle/refhost/mockcl.cpp (recipe:
oracle/build.py build_refhost).  Through it the reference's own code builds
its link tables, edge/face/neighbour lists and matrix slices, generates its
kernel sources and runs them (compiled by g++) on the CPU.  The fixture
scripts under tests/golden/ drive it through this module; nothing in the
library or in bench.py does.

The calls below follow the reference's API (sources/gmlib3.h:77-118); the
variadic ones are called the way its examples call them.
"""
import ctypes
import os
import re

import numpy as np

from . import build as _build

GmlVertices, GmlEdges, GmlTriangles, GmlQuadrilaterals, GmlTetrahedra = 0, 1, 2, 3, 4
GmlPyramids, GmlPrisms, GmlHexahedra = 5, 6, 7
GmlInt, GmlInt2, GmlInt4, GmlInt8, GmlInt16 = 0, 1, 2, 3, 4
GmlFlt, GmlFlt2, GmlFlt4, GmlFlt8, GmlFlt16 = 5, 6, 7, 8, 9
GmlDbl, GmlDbl2, GmlDbl4, GmlDbl8, GmlDbl16 = 10, 11, 12, 13, 14
GmlRefFlag, GmlReadMode, GmlWriteMode, GmlVoyeurs, GmlManual = 1, 2, 4, 8, 16
GmlMin, GmlMax, GmlSum, GmlL0, GmlL1, GmlL2, GmlLinf = range(7)

_lib = None


def available():
    return _build.reference_available()


def lib():
    """Build (if needed) and load librefhost.so; None without the reference tree."""
    global _lib
    if _lib is None:
        path = _build.build_refhost()
        if path is None:
            return None
        os.environ.setdefault("REFHOST_CACHE", _build.HOST_JIT)
        L = ctypes.CDLL(path)
        L.GmlInit.restype = ctypes.c_size_t
        L.GmlInit.argtypes = [ctypes.c_int]
        L.GmlStop.argtypes = [ctypes.c_size_t]
        L.GmlNewMeshData.argtypes = [ctypes.c_size_t, ctypes.c_int, ctypes.c_int]
        L.GmlNewSolutionData.argtypes = [ctypes.c_size_t, ctypes.c_int, ctypes.c_int,
                                         ctypes.c_int, ctypes.c_char_p]
        L.GmlNewParameters.restype = ctypes.c_void_p
        L.GmlNewParameters.argtypes = [ctypes.c_size_t, ctypes.c_int, ctypes.c_char_p]
        L.GmlSetDataBlock.argtypes = [ctypes.c_size_t, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                      ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_void_p]
        L.GmlGetDataBlock.argtypes = L.GmlSetDataBlock.argtypes
        L.GmlLaunchKernel.argtypes = [ctypes.c_size_t, ctypes.c_int]
        L.GmlReduceVector.argtypes = [ctypes.c_size_t, ctypes.c_int, ctypes.c_int,
                                      ctypes.POINTER(ctypes.c_double)]
        L.GmlGetMeshInfo.argtypes = [ctypes.c_size_t, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                     ctypes.POINTER(ctypes.c_int)]
        L.GmlGetLinkInfo.argtypes = [ctypes.c_size_t, ctypes.c_int, ctypes.c_int] + \
            [ctypes.POINTER(ctypes.c_int)] * 4
        L.GmlExtractEdges.argtypes = [ctypes.c_size_t]
        L.GmlExtractFaces.argtypes = [ctypes.c_size_t]
        L.GmlSetNeighbours.argtypes = [ctypes.c_size_t, ctypes.c_int]
        L.GmlNewMatrix.argtypes = [ctypes.c_size_t, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                   ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        L.GmlNewVector.argtypes = [ctypes.c_size_t, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                   ctypes.c_int]
        L.GmlMultMatVec.argtypes = [ctypes.c_size_t, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.GmlMultDiagMatVec.argtypes = L.GmlMultMatVec.argtypes
        L.GmlAddVec3.argtypes = [ctypes.c_size_t] + [ctypes.c_int] * 4
        L.GmlScaleVec.argtypes = [ctypes.c_size_t, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
        L.GmlNormVec.argtypes = [ctypes.c_size_t, ctypes.c_int, ctypes.c_int,
                                 ctypes.POINTER(ctypes.c_double)]
        L.GmlEvaluateNumbering.restype = ctypes.c_float
        L.GmlEvaluateNumbering.argtypes = [ctypes.c_size_t]
        L.refhost_program_source.restype = ctypes.c_char_p
        L.refhost_program_options.restype = ctypes.c_char_p
        L.refhost_kernel_args.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_void_p),
                                          ctypes.POINTER(ctypes.c_size_t), ctypes.c_int]
        L.refhost_kernel_program.argtypes = [ctypes.c_int]
        L.refhost_kernel_name.restype = ctypes.c_char_p
        L.refhost_kernel_name.argtypes = [ctypes.c_int]
        L.refhost_set_max_group.argtypes = [ctypes.c_int]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class Instance:
    """One GmlInit instance of the reference library."""

    def __init__(self):
        self.L = lib()
        if self.L is None:
            raise RuntimeError("the reference tree is needed for the reference host library")
        self.g = self.L.GmlInit(0)
        if not self.g:
            raise RuntimeError("reference GmlInit failed")
        self._keep = []

    def stop(self):
        self.L.GmlStop(self.g)

    # ---- data ----------------------------------------------------------------
    def parameters(self, size, src):
        s = ctypes.create_string_buffer(src)
        self._keep.append(s)          # the reference stores the pointer
        return self.L.GmlNewParameters(self.g, size, s)

    def mesh(self, typ, nodes, ref=None):
        """GmlNewMeshData + GmlSetDataBlock over all lines.  Vertices: float32
        (n, 4) rows (x, y, z, unused); elements: int32 (n, k) rows."""
        n = len(nodes)
        idx = self.L.GmlNewMeshData(self.g, typ, n)
        if not idx:
            raise RuntimeError("GmlNewMeshData failed")
        a = np.ascontiguousarray(nodes, np.float32 if typ == GmlVertices else np.int32)
        r = np.ascontiguousarray(np.zeros(n, np.int32) if ref is None else ref, np.int32)
        stride = a.shape[1] * 4
        ok = self.L.GmlSetDataBlock(self.g, typ, 0, n - 1, _p(a), a.ctypes.data + (n - 1) * stride,
                                    _p(r), r.ctypes.data + (n - 1) * 4)
        if ok != 1:
            raise RuntimeError("GmlSetDataBlock failed")
        return idx

    def solution(self, typ, nitm, otyp, name):
        s = ctypes.create_string_buffer(name)
        self._keep.append(s)          # the reference stores the pointer
        idx = self.L.GmlNewSolutionData(self.g, typ, nitm, otyp, s)
        if not idx:
            raise RuntimeError("GmlNewSolutionData failed")
        return idx

    def mesh_info(self, typ):
        n, i = ctypes.c_int(), ctypes.c_int()
        self.L.GmlGetMeshInfo(self.g, typ, ctypes.byref(n), ctypes.byref(i))
        return n.value, i.value

    def link_info(self, src, dst):
        v = [ctypes.c_int() for _ in range(4)]
        ok = self.L.GmlGetLinkInfo(self.g, src, dst, *[ctypes.byref(x) for x in v])
        return (ok,) + tuple(x.value for x in v)

    def set_lines(self, idx, rows):
        """GmlSetDataLine over every line of a raw (solution) datatype: row i
        of `rows` (any dtype, one line's bytes) is passed by address."""
        a = np.ascontiguousarray(rows)
        step = a.strides[0]
        for i in range(len(a)):
            r = self.L.GmlSetDataLine(ctypes.c_size_t(self.g), ctypes.c_int(idx), ctypes.c_int(i),
                                      ctypes.c_void_p(a.ctypes.data + i * step))
            if r != 1:
                raise RuntimeError("reference GmlSetDataLine returned %d" % r)

    def get_lines(self, idx, n, fmt):
        """GmlGetDataLine over lines 0..n-1 (line 0 downloads the buffer).
        fmt: 'ii' for (int, int, ref), 'iii', 'iiii' ..., 'ddd' for vertices."""
        out = []
        for i in range(n):
            if fmt.startswith("d"):
                v = [ctypes.c_double() for _ in fmt] + [ctypes.c_int()]
            else:
                v = [ctypes.c_int() for _ in fmt] + [ctypes.c_int()]
            self.L.GmlGetDataLine(ctypes.c_size_t(self.g), ctypes.c_int(idx), ctypes.c_int(i),
                                  *[ctypes.byref(x) for x in v])
            out.append([x.value for x in v])
        return np.array(out)

    # ---- kernels ---------------------------------------------------------------
    def compile(self, src, name, msh, dats):
        """dats: (data index, flags) pairs, or (data index, flags, link
        index) triplets; the link index is 0 (NULL in the examples) unless
        given.  The reference reads all three as ints (gmlib3.c:2238-2244)."""
        s = ctypes.create_string_buffer(src)
        nm = ctypes.create_string_buffer(name)
        self._keep += [s, nm]
        args = []
        for item in dats:
            d, f = item[0], item[1]
            lk = item[2] if len(item) > 2 else 0
            args += [ctypes.c_int(d), ctypes.c_int(f), ctypes.c_int(lk)]
        k = self.L.GmlCompileKernel(ctypes.c_size_t(self.g), s, nm, ctypes.c_int(msh),
                                    ctypes.c_int(len(dats)), *args)
        if k <= 0:
            raise RuntimeError("reference GmlCompileKernel(%s) failed" % name.decode())
        return k

    def launch(self, k):
        r = self.L.GmlLaunchKernel(self.g, k)
        if r != 1:
            raise RuntimeError("reference GmlLaunchKernel returned %d" % r)

    def reduce(self, idx, op):
        v = ctypes.c_double()
        r = self.L.GmlReduceVector(self.g, idx, op, ctypes.byref(v))
        if r != 1:
            raise RuntimeError("reference GmlReduceVector returned %d" % r)
        return v.value


def program_sources():
    L = lib()
    return [L.refhost_program_source(i).decode() for i in range(L.refhost_nprograms())]


def kernel_objects(name):
    """Indices (creation order) of the kernel objects of that name: a
    high-degree twin carries its base kernel's name."""
    L = lib()
    return [i for i in range(L.refhost_nkernels()) if L.refhost_kernel_name(i).decode() == name]


def kernel_signature(k):
    """Argument names of kernel object k, from its program source."""
    L = lib()
    name = L.refhost_kernel_name(k).decode()
    src = L.refhost_program_source(L.refhost_kernel_program(k)).decode()
    m = re.search(r"__kernel\s+void\s+%s\s*\((.*?)\)\s*\{" % re.escape(name), src, re.S)
    names = []
    for p in m.group(1).split(","):
        p = p.strip()
        a = re.search(r"\(\s*\*\s*(\w+)\s*\)", p)
        names.append(a.group(1) if a else re.findall(r"\w+", p)[-1])
    return names


def kernel_buffers(k):
    """{argument name: bytes of its buffer} bound to kernel object k (value
    arguments are left out)."""
    L = lib()
    ptr = (ctypes.c_void_p * 64)()
    siz = (ctypes.c_size_t * 64)()
    n = L.refhost_kernel_args(k, ptr, siz, 64)
    if n < 0:
        raise KeyError(k)
    names = kernel_signature(k)
    out = {}
    for i in range(n):
        if ptr[i]:
            out[names[i]] = ctypes.string_at(ptr[i], siz[i])
    return out


def program_of(k):
    L = lib()
    return L.refhost_program_source(L.refhost_kernel_program(k)).decode()
