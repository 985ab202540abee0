"""C++ case drivers written against the reference-named classes of
include/gpupfem2/gpupfem2.hpp (the reference's Poisson2D and Poisson3D flows), built with
g++ and run."""
import os
import subprocess

import pytest

import gpupfem2_gb300 as g
from gpupfem2_gb300 import meshgen as mg

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _build(tmp_path, name):
    exe = os.path.join(tmp_path, name)
    cuda_home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    lib_dir = os.path.dirname(g.LIB_PATH)
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), "-I",
                        os.path.join(cuda_home, "include"), os.path.join(ROOT, "tests", "cpp", name + ".cpp"),
                        "-o", exe, "-L", lib_dir, "-lpf2", "-L", os.path.join(cuda_home, "lib64"), "-lcudart",
                        "-Wl,-rpath," + lib_dir], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_poisson_driver(cuda, tmp_path):
    exe = _build(tmp_path, "poisson_case")
    xy, tri = mg.unit_square(64)
    mesh = os.path.join(tmp_path, "square.dat")
    mg.write_dat(mesh, xy, tri)
    r = subprocess.run([exe, mesh], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    fields = dict(kv.split("=") for kv in r.stdout.split())
    assert fields["cg_converged"] == "1" and fields["gmres_converged"] == "1"
    assert float(fields["max_error"]) < 3e-4


def test_poisson3d_driver(cuda, tmp_path):
    exe = _build(tmp_path, "poisson3d_case")
    xyz, tet = mg.box_tets(20, 10, 6)
    mesh = os.path.join(tmp_path, "box.dat")
    mg.write_dat3(mesh, xyz, tet)
    out = os.path.join(tmp_path, "solution.vtu")
    r = subprocess.run([exe, mesh, out], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    fields = dict(kv.split("=") for kv in r.stdout.split())
    assert fields["cg_converged"] == "1" and int(fields["cg_iterations"]) < 1000
    assert abs(float(fields["min"]) + 2.0) < 1e-6 and abs(float(fields["max"]) - 3.0) < 1e-6
    assert 'Name="solution"' in open(out).read()
