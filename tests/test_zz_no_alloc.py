"""The allocation-free CG entry point, dfx_cg_solve_noalloc.

Some callers may not allocate device or pinned memory once running (hosts
that capture their work into CUDA graphs after setting up their own memory
pool, plugins whose host owns all allocations, real-time loops). For them
the library offers a CG solve whose scratch is a fixed array inside the
library. This file runs last (its name sorts last) so that a failure here
leaves every other test already run; it must pass both alone in a fresh
process, where the first call sets the array up, and after the other tests.
"""

import ctypes as C

import numpy as np
import pytest
import torch

from gpu_util import assert_close, problem

pytestmark = pytest.mark.gpu


def _system(oracle, n):
    from dolfinx_gb300 import fem

    m, V, kappa, f, rp, cols = problem(oracle, n, 2, seed=41)
    X = V.tabulate_dof_coordinates()
    bnd = np.flatnonzero(np.isclose(X[:, 0], 0) | np.isclose(X[:, 0], 1)).astype(np.int32)
    bc = fem.dirichletbc(0.0, bnd, V)
    a = fem.poisson_form(V, kappa)
    A = fem.assemble_matrix(a, bcs=[bc])
    b = fem.RhsAssembler(fem.source_form(V, f), a, [bc]).assemble()
    return A, b


def _noalloc(capi, A, b, dinv, x):
    info = capi.CgInfo()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = capi.lib().dfx_cg_solve_noalloc(C.byref(A.csr()), C.c_void_p(b.data_ptr()),
                                         C.c_void_p(x.data_ptr()), C.c_void_p(dinv.data_ptr()),
                                         1e-10, 100000, 20, C.byref(info), stream)
    capi.check(rc)
    return info


def test_noalloc_cg_matches_workspace_cg(cuda, oracle, capi):
    from dolfinx_gb300 import la

    A, b = _system(oracle, (10, 9, 8))
    ref = la.CGSolver(A, jacobi=True)
    x_ref = torch.zeros_like(b)
    r_ref = ref.solve(b, x_ref, rtol=1e-10)
    # Two calls in a row: the second starts from the first call's leftover
    # scratch contents.
    for _ in range(2):
        x = torch.zeros_like(b)
        info = _noalloc(capi, A, b, ref.dinv, x)
        torch.cuda.synchronize()
        assert info.status == 0
        assert info.iterations == r_ref.iterations
        assert_close(x.cpu().numpy(), x_ref.cpu().numpy(), rtol=1e-12)


def test_noalloc_cg_rejects_oversized_systems(cuda, oracle, capi):
    from dolfinx_gb300 import la

    n = 524288 + 1
    A = la.MatrixCSR(torch.arange(n + 1, dtype=torch.int64).cuda(),
                     torch.arange(n, dtype=torch.int32).cuda(),
                     torch.ones(n, dtype=torch.float64).cuda())
    b = torch.ones(n, dtype=torch.float64).cuda()
    x = torch.zeros_like(b)
    with pytest.raises(capi.DfxError, match="at most 524288 unknowns"):
        _noalloc(capi, A, b, b, x)
