"""Build recipe of the oracle (test infrastructure).

  oracle/liboracle.so       the C restatement (oracle.c), gcc -O2 -fopenmp
  oracle/_ref/librefcl.so   the reference's own kernel bodies and toolkit
                            (sources/toolkit.cl, examples/*/ *.cl, P2Quality
                            included) compiled as C++ against
                            oracle/refcl/cl_host.h, from where they lie in the
                            reference tree
  oracle/_ref/librefhost.so the reference's host library, sources/gmlib3.c,
                            compiled unmodified against the OpenCL stand-in
                            header oracle/refhost/CL/opencl.h, its .cl library
                            kernels turned into headers by this project's cl2h
                            (the reference's compile_cl() step), linked with the
                            host-CPU OpenCL runtime oracle/refhost/mockcl.cpp

The two _ref libraries are built only where the reference tree exists: the
directory named by GML_REFERENCE_ROOT, else a `reference` directory beside
the repository.  Nothing from the reference is copied: its files are read
where they lie.

Usage: python -m oracle.build [--force]
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
REF_ROOT = os.environ.get("GML_REFERENCE_ROOT") or os.path.join(os.path.dirname(REPO), "reference")
LIB = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")
REF_LIB = os.path.join(REF_DIR, "librefcl.so")
HOST_LIB = os.path.join(REF_DIR, "librefhost.so")
HOST_GEN = os.path.join(REF_DIR, "refhost_gen")
HOST_JIT = os.path.join(REF_DIR, "refhost_jit")
# the reference's library kernels, embedded as C strings by cl2h (sources/CMakeLists.txt)
HOST_CL = ("addvec", "multdiagmatvec", "multmatvec", "normvec", "scalevec", "reduce", "toolkit")


def _stale(out, srcs):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs if os.path.exists(s))


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n%s\n%s" % (" ".join(cmd), r.stdout))


def build_oracle(force=False):
    names = ("oracle.c", "oracle_mesh.c", "oracle_linalg.c", "baseline.c")
    srcs = [os.path.join(HERE, f) for f in names + ("oracle.h",)]
    if force or _stale(LIB, srcs):
        _run(["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-std=gnu11"]
             + [os.path.join(HERE, f) for f in names] + ["-o", LIB, "-lm"])
    return LIB


def reference_available():
    return os.path.exists(os.path.join(REF_ROOT, "sources", "toolkit.cl"))


def build_refcl(force=False):
    """Compile the reference kernel bodies as C++ (only where the reference
    tree is present)."""
    if not reference_available():
        return None
    os.makedirs(REF_DIR, exist_ok=True)
    src = os.path.join(HERE, "refcl", "refcl.cpp")
    hdr = os.path.join(HERE, "refcl", "cl_host.h")
    deps = [src, hdr,
            os.path.join(REF_ROOT, "sources", "toolkit.cl"),
            os.path.join(REF_ROOT, "examples", "MeshQuality", "compute_quality.cl"),
            os.path.join(REF_ROOT, "examples", "NodeSmoothing", "scatter.cl"),
            os.path.join(REF_ROOT, "examples", "NodeSmoothing", "gather.cl"),
            os.path.join(REF_ROOT, "examples", "P2Quality", "quality.cl"),
            os.path.join(REPO, "tests", "kernels", "toolkit_table.cl")]
    if force or _stale(REF_LIB, deps):
        _run(["g++", "-O2", "-fPIC", "-shared", "-fopenmp", "-std=c++17",
              "-fsingle-precision-constant", "-ffp-contract=off",
              "-I" + os.path.join(HERE, "refcl"), "-I" + os.path.join(REF_ROOT, "sources"),
              "-I" + os.path.join(REF_ROOT, "examples"), "-I" + os.path.join(REPO, "tests", "kernels"),
              src, "-o", REF_LIB])
    return REF_LIB


def build_refhost(force=False):
    """Compile the reference's unmodified host library against the OpenCL
    stand-in and the host-CPU runtime (only where the reference tree is
    present)."""
    if not reference_available():
        return None
    os.makedirs(HOST_GEN, exist_ok=True)
    os.makedirs(HOST_JIT, exist_ok=True)
    rsrc = os.path.join(REF_ROOT, "sources")
    mock = os.path.join(HERE, "refhost", "mockcl.cpp")
    stub = os.path.join(HERE, "refhost", "CL", "opencl.h")
    clc = os.path.join(HERE, "refhost", "clc_host.hpp")
    cl2h_src = os.path.join(REPO, "gmlib_gb300", "csrc", "cl2h.c")
    cl2h = os.path.join(REF_DIR, "cl2h")
    deps = [mock, stub, clc, cl2h_src, os.path.join(rsrc, "gmlib3.c"), os.path.join(rsrc, "gmlib3.h")]
    deps += [os.path.join(rsrc, n + ".cl") for n in HOST_CL]
    if not (force or _stale(HOST_LIB, deps)):
        return HOST_LIB
    _run(["gcc", "-O2", cl2h_src, "-o", cl2h])
    for n in HOST_CL:
        _run([cl2h, os.path.join(rsrc, n + ".cl"), os.path.join(HOST_GEN, n + ".h"), n])
    obj = os.path.join(REF_DIR, "refhost_gmlib3.o")
    _run(["gcc", "-O2", "-fPIC", "-std=gnu99", "-w", "-c", os.path.join(rsrc, "gmlib3.c"),
          "-I" + os.path.join(HERE, "refhost"), "-I" + HOST_GEN, "-o", obj])
    _run(["g++", "-O2", "-fPIC", "-shared", "-fopenmp", "-std=c++17", "-Wl,-Bsymbolic",
          '-DREFHOST_HDR_DIR="%s"' % os.path.join(HERE, "refhost"),
          "-I" + os.path.join(HERE, "refhost"), mock, obj, "-o", HOST_LIB, "-ldl", "-lm"])
    return HOST_LIB


def build(force=False):
    build_oracle(force)
    build_refcl(force)
    build_refhost(force)


if __name__ == "__main__":
    build("--force" in sys.argv)
    print(LIB)
