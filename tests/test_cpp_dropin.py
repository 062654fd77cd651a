"""The C++ Eikonal class (include/Eikonal.h): the reference's test programs
restated in C++ against it.  Compiling and linking runs everywhere; running
needs the GPU."""
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

LIB_DIR = os.path.join(ROOT, "sci-solver_eikonal_gb300")
SRC = os.path.join(ROOT, "tests", "cpp", "eikonal_cpp_test.cc")


def _build(tmp_path):
    exe = str(tmp_path / "eikonal_cpp_test")
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe,
           "-L", LIB_DIR, "-leikonal_gb300", "-Wl,-rpath," + LIB_DIR]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "warning" not in r.stderr, r.stderr
    return exe


def _write_fixtures(d):
    g = np.load(os.path.join(GOLDEN, "meshes.npz"))
    for name in ("sphere8", "sphere13", "sphere334", "CubeMesh_size16"):
        xyz, tets = g[name + "_xyz"], g[name + "_tets"]
        with open(os.path.join(d, name + ".node"), "w") as f:
            f.write(f"{xyz.shape[0]} 3 0 0\n")
            for i, p in enumerate(xyz):
                f.write(f"{i} {repr(float(p[0]))} {repr(float(p[1]))} {repr(float(p[2]))}\n")
        with open(os.path.join(d, name + ".ele"), "w") as f:
            f.write(f"{tets.shape[0]} 4 0\n")
            for i, t in enumerate(tets):
                f.write(f"{i} {t[0]} {t[1]} {t[2]} {t[3]}\n")
    for name in ("sphere_74verts", "SquareMesh_size16"):
        xyz, faces = g[name + "_xyz"], g[name + "_faces"]
        with open(os.path.join(d, name + ".ply"), "w") as f:
            f.write("ply\nformat ascii 1.0\n")
            f.write(f"element vertex {xyz.shape[0]}\nproperty float x\nproperty float y\nproperty float z\n")
            f.write(f"element face {faces.shape[0]}\nproperty list uchar int vertex_indices\nend_header\n")
            for p in xyz:
                f.write(f"{repr(float(p[0]))} {repr(float(p[1]))} {repr(float(p[2]))}\n")
            for t in faces:
                f.write(f"3 {t[0]} {t[1]} {t[2]}\n")


def test_cpp_class_compiles_and_links(tmp_path):
    _build(tmp_path)


@pytest.mark.gpu
def test_cpp_reference_tests_pass(need_gpu, tmp_path):
    exe = _build(tmp_path)
    _write_fixtures(str(tmp_path))
    r = subprocess.run([exe, str(tmp_path)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr


def test_cpp_exit_codes_like_the_reference(tmp_path):
    """With EIKONAL_GB300_EXIT_ON_ERROR the class ends the process with the
    reference's codes (src/test/3d/3D-sanity.cc expects status 1 for a missing
    mesh file); the mesh read fails before any GPU work, so this runs anywhere."""
    src = tmp_path / "exit_test.cc"
    src.write_text('#include "Eikonal.h"\n'
                   'int main(int argc, char** argv) {\n'
                   '  Eikonal data(argv[1][0] == \'2\');\n'
                   '  data.filename_ = "notarealfile";\n'
                   '  data.solveEikonal();\n'
                   '  return 7;\n'
                   '}\n')
    exe = str(tmp_path / "exit_test")
    cmd = ["g++", "-std=c++17", "-DEIKONAL_GB300_EXIT_ON_ERROR", "-I", os.path.join(ROOT, "include"), str(src),
           "-o", exe, "-L", LIB_DIR, "-leikonal_gb300", "-Wl,-rpath," + LIB_DIR]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    for dim in ("2", "3"):
        r = subprocess.run([exe, dim], capture_output=True, text=True, timeout=60)
        assert r.returncode == 1, (dim, r.returncode, r.stderr)
        assert "notarealfile" in r.stderr
