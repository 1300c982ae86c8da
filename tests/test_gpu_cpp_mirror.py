"""The C++ face (include/dolfinx_gb300.hpp) on a GPU: tests/cpp_host_example.cpp
assembles and solves P1 Poisson on a 4^3 x 6 box through it (matrix,
diagonal, vector, lifting, set_bc, FP64 CG, FP32-inner refinement), then
takes a(u, u) and the Neumann vector of 1 on the boundary, whose entries sum
to the boundary's area, and assembles the interior penalty on its
macro-element pattern (zero on a linear function) and lifts through it."""

import os
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpp_mirror_assembles_and_solves(cuda, capi, tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    libdir = os.path.dirname(capi.LIB_PATH)
    cuda_home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    exe = str(tmp_path / "cpp_host")
    build = subprocess.run(
        [cxx, "-std=c++20", "-O2", "-I", os.path.join(ROOT, "include"), "-I",
         os.path.join(cuda_home, "include"), os.path.join(ROOT, "tests", "cpp_host_example.cpp"),
         "-o", exe, "-L", libdir, "-ldfxgpu", f"-Wl,-rpath,{libdir}", "-L",
         os.path.join(cuda_home, "lib64"), "-lcudart",
         f"-Wl,-rpath,{os.path.join(cuda_home, 'lib64')}"],
        capture_output=True, text=True, timeout=300)
    if build.returncode != 0:
        pytest.skip("could not build the C++ example here: " + build.stderr[-300:])
    run = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, run.stdout + run.stderr
    dev = [line.split()[1:] for line in run.stdout.splitlines() if line.startswith("device ")]
    got = {d[0]: d[1:] for d in dev}
    cg_iters, cg_status = map(int, got["cg"])
    assert cg_status == 0 and cg_iters > 0
    inner, outer, ir_status = map(int, got["ir"])
    assert ir_status == 0 and inner > 0
    assert float(got["energy"][0]) > 0.0
    assert abs(float(got["boundary_area"][0]) - 6.0) < 1e-12
    assert float(got["penalty_linear"][0]) < 1e-10
    assert got["penalty_lifting_ok"] == ["1"]
