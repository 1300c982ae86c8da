"""The device counterpart of the per-cell kernel ABI (fem/kernel.h:18-27):
include/dfx_cell_kernel.cuh templates the cell loops around a caller's own
element functor. tests/user_kernel_example.cu is such a caller (P1 Poisson
with a per-cell coefficient, and a constant load). On CPU it must compile
with nvcc against the public headers alone; on a GPU its matrix and vector
must equal the library's built-in forms."""

import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def build_example(out_dir) -> str:
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    lib = os.path.join(str(out_dir), "libuser_kernel.so")
    r = subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++20",
                        "-shared", "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "user_kernel_example.cu"), "-o", lib],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return lib


def test_user_kernel_example_compiles(tmp_path):
    lib = build_example(tmp_path)
    assert os.path.getsize(lib) > 0


@pytest.mark.gpu
def test_user_kernel_matches_builtin_forms(cuda, capi, oracle, tmp_path):
    import torch

    from dolfinx_gb300 import fem, la

    from gpu_util import assert_close, problem

    L = C.CDLL(build_example(tmp_path))
    L.user_assemble_p1_poisson.argtypes = [C.c_int32] + [C.c_void_p] * 8
    L.user_assemble_p1_load.argtypes = [C.c_int32] + [C.c_void_p] * 6
    m, V, kappa, f, rp, cols = problem(oracle, (7, 5, 6), 1, seed=51)
    X = V.tabulate_dof_coordinates()
    nodes = np.flatnonzero(np.isclose(X[:, 2], 0)).astype(np.int32)
    bc = fem.dirichletbc(0.0, nodes, V)
    a = fem.poisson_form(V, kappa)
    ref = fem.MatrixAssembler(a, [bc], diagonal=0.0).assemble()
    A = la.MatrixCSR(ref.row_ptr, ref.cols, torch.zeros_like(ref.vals), 1)
    xd, x = m.device("cuda")
    dm = V.dofmap_device()
    kap = torch.from_numpy(kappa).cuda()
    markers = fem.bc_markers(V, [bc])
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    csr = A.csr()
    stream = torch.cuda.current_stream().cuda_stream
    rc = L.user_assemble_p1_poisson(m.num_cells, xd.data_ptr(), x.data_ptr(), dm.data_ptr(),
                                    kap.data_ptr(), markers.data_ptr(), C.addressof(csr),
                                    status.data_ptr(), stream)
    torch.cuda.synchronize()
    assert rc == 0 and int(status.item()) == 0
    assert_close(A.vals.cpu().numpy(), ref.vals.cpu().numpy())
    c = torch.tensor([2.5], dtype=torch.float64, device="cuda")
    b = torch.zeros(V.num_dofs, dtype=torch.float64, device="cuda")
    rc = L.user_assemble_p1_load(m.num_cells, xd.data_ptr(), x.data_ptr(), dm.data_ptr(),
                                 c.data_ptr(), b.data_ptr(), stream)
    torch.cuda.synchronize()
    assert rc == 0
    bref = fem.assemble_vector(fem.source_form(V, 2.5))
    assert_close(b.cpu().numpy(), bref.cpu().numpy())
