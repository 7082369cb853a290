"""Build recipe of the oracle (test infrastructure).

  oracle/liboracle.so     the C restatement (oracle.c), gcc -O2 -fopenmp
  oracle/_ref/librefcl.so the reference's own kernel bodies and toolkit
                          (sources/toolkit.cl, examples/*/ *.cl, P2Quality
                          included) compiled as
                          C++ against oracle/refcl/cl_host.h, from where they
                          lie in the reference tree; built only where that
                          tree exists (it is not shipped anywhere else).

Usage: python -m oracle.build [--force]
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_ROOT = os.environ.get("GML_REFERENCE_ROOT", "/root/reference")
LIB = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")
REF_LIB = os.path.join(REF_DIR, "librefcl.so")


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
            os.path.join(REF_ROOT, "examples", "P2Quality", "quality.cl")]
    if force or _stale(REF_LIB, deps):
        _run(["g++", "-O2", "-fPIC", "-shared", "-fopenmp", "-std=c++17",
              "-fsingle-precision-constant", "-ffp-contract=off",
              "-I" + os.path.join(HERE, "refcl"), "-I" + os.path.join(REF_ROOT, "sources"),
              "-I" + os.path.join(REF_ROOT, "examples"),
              src, "-o", REF_LIB])
    return REF_LIB


def build(force=False):
    build_oracle(force)
    build_refcl(force)


if __name__ == "__main__":
    build("--force" in sys.argv)
    print(LIB)
