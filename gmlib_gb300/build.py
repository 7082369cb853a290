"""Build libgmlib3.so in-tree for sm_103a.

The library is C99 host code (gcc) plus CUDA kernels (nvcc, one -gencode for
sm_103a), linked into gmlib_gb300/libgmlib3.so.  NVRTC is linked dynamically;
the CUDA runtime statically, so the library does not depend on the runtime
shipped with any Python package.  Translation units are compiled in parallel;
a unit is rebuilt when it or any header is newer than its object.

Usage:  python -m gmlib_gb300.build  [--force]
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(ROOT, "_build", "gmlib3")
LIB = os.path.join(PKG, "libgmlib3.so")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

C_SOURCES = ["gmlib3.c", "gml_tables.c", "gml_topo.c", "gml_codegen.c",
             "gml_dialect.c", "gml_ext.c", "gml_native.c", "gml_linalg.c",
             "gml_solver.c", "gml_problem.c", "gml_batch.c", "gml_serve.c",
             "gml_hostcopy.c", "gml_meshio.c"]
CU_SOURCES = ["gml_device.cu", "gml_reduce.cu", "gml_linalg_kernels.cu",
              "gml_mesh_kernels.cu", "gml_solver_kernels.cu", "gml_scan.cu"]
EMBEDDED = ["gml_cl.h", "gml_toolkit.h"]


def _cuda_libdirs():
    dirs = []
    for d in ("lib64", "targets/sbsa-linux/lib", "targets/x86_64-linux/lib", "lib"):
        p = os.path.join(CUDA_HOME, d)
        if os.path.isdir(p) and p not in dirs:
            dirs.append(p)
    return dirs


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".h")]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def _stale(obj, srcs):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(s) > t for s in srcs if os.path.exists(s))


def _embed():
    """Write the device headers used by NVRTC as C string literals."""
    out = os.path.join(BUILD, "gml_embedded.c")
    srcs = [os.path.join(CSRC, f) for f in EMBEDDED]
    if not _stale(out, srcs + [__file__]):
        return out
    lines = ["/* generated by gmlib_gb300/build.py from the NVRTC headers */"]
    for f in EMBEDDED:
        name = "gml_embedded_" + f[len("gml_"):].replace(".", "_")
        with open(os.path.join(CSRC, f), "r") as fh:
            text = fh.read()
        esc = []
        for line in text.split("\n"):
            line = line.replace("\\", "\\\\").replace('"', '\\"')
            esc.append('"' + line + '\\n"')
        lines.append("const char *%s =\n%s;" % (name, "\n".join(esc)))
    with open(out, "w") as fh:
        fh.write("\n".join(lines) + "\n")
    return out


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n%s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def build(force=False, verbose=False, defines=(), out=None, objdir=None):
    """Compile and link the library.  defines: extra -D macros for the CUDA
    sources (tuning variants); out / objdir: alternate library path and
    object directory for such variants."""
    lib = out or LIB
    bdir = objdir or BUILD
    os.makedirs(bdir, exist_ok=True)
    emb = _embed()
    hdrs = _headers()
    jobs, objs = [], []
    cflags = ["-O2", "-fPIC", "-std=gnu11", "-Wall", "-Wno-unused-function",
              "-I" + INCLUDE, "-I" + CSRC, "-I" + os.path.join(CUDA_HOME, "include")]
    for f in C_SOURCES + [emb]:
        src = f if os.path.isabs(f) else os.path.join(CSRC, f)
        obj = os.path.join(bdir, os.path.basename(f) + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs):
            jobs.append(["gcc"] + cflags + ["-c", src, "-o", obj])
    nvflags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                      "-I" + INCLUDE, "-I" + CSRC] + ["-D" + d for d in defines]
    for f in CU_SOURCES:
        src = os.path.join(CSRC, f)
        obj = os.path.join(bdir, f + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs):
            jobs.append([NVCC] + nvflags + ["-c", src, "-o", obj])
    if jobs:
        with ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            outs = list(ex.map(_run, jobs))
        if verbose:
            for o in outs:
                if o.strip():
                    print(o)
    # the cl2h tool of the CMake package (cmake/GMlibConfig.cmake, compile_cl)
    cl2h_src = os.path.join(CSRC, "cl2h.c")
    cl2h = os.path.join(PKG, "cl2h")
    if out is None and (force or _stale(cl2h, [cl2h_src])):
        jobs_host = [["gcc", "-O2", "-std=gnu11", "-Wall", cl2h_src, "-o", cl2h]]
        for j in jobs_host:
            _run(j)
    if jobs or force or not os.path.exists(lib):
        libdirs = _cuda_libdirs()
        link = [NVCC] + ARCH + ["-shared", "-o", lib] + objs
        for d in libdirs:
            link += ["-L" + d, "-Xlinker", "-rpath=" + d]
        link += ["-cudart", "static", "-lnvrtc", "-lpthread", "-ldl", "-lrt", "-lm"]
        _run(link)
    return lib

if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
