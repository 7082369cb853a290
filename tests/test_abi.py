"""The C-ABI library loads without a GPU and exports every entry point that
include/*.h declares; C programs written against gmlib3.h compile and link
unchanged."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")


def declared(header):
    with open(os.path.join(INCLUDE, header)) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = text.split("internal helpers")[0]
    names = re.findall(r"^\s*[A-Za-z_][\w\s\*]*?\b(Gmlx?\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def exported(path):
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True).stdout
    return {line.split()[-1] for line in out.splitlines() if " T " in line}


@pytest.mark.parametrize("header", ["gmlib3.h", "gmlib3_gb300.h"])
def test_every_declared_symbol_is_exported(G, header):
    names = declared(header)
    assert len(names) > 10
    syms = exported(G.LIB_PATH)
    missing = [n for n in names if n not in syms and not n.startswith("GmlImport")
               and not n.startswith("GmlExport")]
    assert not missing, missing


def test_library_loads_without_gpu(G):
    h = ctypes.CDLL(G.LIB_PATH)
    h.GmlGetWallClock.restype = ctypes.c_double
    assert h.GmlGetWallClock() > 1e9


def test_python_signatures_cover_header(G):
    names = declared("gmlib3.h") + declared("gmlib3_gb300.h")
    for n in names:
        if n in ("GmlImportMesh", "GmlExportSolution"):
            continue
        assert n in G.SIGNATURES, n


def test_c_program_links_against_header(G, tmp_path):
    """A C99 program using the variadic API builds against include/gmlib3.h
    and libgmlib3.so, with no OpenCL header anywhere."""
    src = os.path.join(ROOT, "tests", "c", "mesh_quality.c")
    exe = tmp_path / "mesh_quality"
    r = subprocess.run(["gcc", "-std=c99", "-O2", "-Wall", "-I" + INCLUDE, src, "-o", str(exe),
                        G.LIB_PATH, "-Wl,-rpath," + os.path.dirname(G.LIB_PATH), "-lm"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
