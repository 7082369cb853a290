"""The reference's build-side interface: the cl2h tool and the CMake package
(find_package(GMlib), the GM.3 target, compile_cl).  CPU only."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "gmlib_gb300")
CL2H = os.path.join(PKG, "cl2h")
CMAKE_DIR = os.path.join(PKG, "cmake")


def compile_and_print(tmp_path, header, name):
    src = tmp_path / "show.c"
    src.write_text('#include <stdio.h>\n#include "%s"\nint main(void) { fputs(%s, stdout); '
                   'return 0; }\n' % (header, name))
    exe = tmp_path / "show"
    subprocess.run(["gcc", "-I", str(tmp_path), str(src), "-o", str(exe)], check=True)
    return subprocess.run([str(exe)], check=True, stdout=subprocess.PIPE).stdout


@pytest.mark.parametrize("text", [
    "qal = CalVol(VerCrd[0], VerCrd[1], VerCrd[2], VerCrd[3]);\n",
    "#define SQ(x) ((x) * \\\n            (x))\nres = SQ(2.f);",        # continuation, no final newline
    'const char *s = "quoted \\"text\\"";\n\n',
])
def test_cl2h_embeds_the_body(tmp_path, text):
    """The header declares char *<name> holding "\\n", the body, and one more
    line, like the reference tool's headers."""
    cl = tmp_path / "body.cl"
    cl.write_bytes(text.encode())
    subprocess.run([CL2H, str(cl), str(tmp_path / "body.h"), "body"], check=True)
    assert (tmp_path / "body.h").read_text().startswith('char *body = "\\n" \\\n')
    got = compile_and_print(tmp_path, "body.h", "body").decode()
    assert got == "\n" + text + "\n"


def test_cl2h_usage(tmp_path):
    r = subprocess.run([CL2H, "only-one-arg"], stdout=subprocess.PIPE)
    assert r.returncode != 0 and b"Usage" in r.stdout


@pytest.mark.skipif(shutil.which("cmake") is None, reason="cmake not installed")
def test_cmake_package(tmp_path):
    """A caller's CMake project, written as for the reference, configures,
    builds and runs against this package."""
    proj = tmp_path / "app"
    proj.mkdir()
    (proj / "CMakeLists.txt").write_text(
        "cmake_minimum_required(VERSION 3.18)\n"
        "project(app C)\n"
        "find_package(GMlib 3 REQUIRED)\n"
        "compile_cl(body)\n"
        "include_directories(${CMAKE_CURRENT_BINARY_DIR} ${GMlib_INCLUDE_DIRS})\n"
        "add_executable(app app.c ${CMAKE_CURRENT_BINARY_DIR}/body.h)\n"
        "target_link_libraries(app ${GMlib_LIBRARIES})\n")
    (proj / "body.cl").write_text("qal = 1.f;\n")
    (proj / "app.c").write_text(
        '#include <stdio.h>\n#include "gmlib3.h"\n#include "body.h"\n'
        "int main(void) { size_t (*init)(int) = GmlInit; "
        'printf("%d %s", init != 0, body); return 0; }\n')
    build = tmp_path / "build"
    subprocess.run(["cmake", "-S", str(proj), "-B", str(build), "-DGMlib_DIR=" + CMAKE_DIR],
                   check=True, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    subprocess.run(["cmake", "--build", str(build)], check=True, stdout=subprocess.PIPE,
                   stderr=subprocess.STDOUT)
    out = subprocess.run([str(build / "app")], check=True, stdout=subprocess.PIPE).stdout
    assert out.decode() == "1 \nqal = 1.f;\n\n"
    # a request for another major version is refused
    (proj / "CMakeLists.txt").write_text(
        "cmake_minimum_required(VERSION 3.18)\nproject(app C)\nfind_package(GMlib 4 REQUIRED)\n")
    r = subprocess.run(["cmake", "-S", str(proj), "-B", str(tmp_path / "b4"),
                        "-DGMlib_DIR=" + CMAKE_DIR], stdout=subprocess.PIPE,
                       stderr=subprocess.STDOUT)
    assert r.returncode != 0
