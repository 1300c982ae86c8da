"""GPU parity: assembly, lifting, set_bc, set_diagonal against the oracle.
Tolerance: 1e-12 relative to the largest entry (FP64; summation order
differs from the sequential reference loop)."""

import numpy as np
import pytest
import torch

from gpu_util import assert_close, problem

pytestmark = pytest.mark.gpu


def boundary_nodes(V):
    X = V.tabulate_dof_coordinates()
    return np.flatnonzero(np.isclose(X, 0).any(1) | np.isclose(X, 1).any(1)).astype(np.int32)


@pytest.mark.parametrize("mode", ["atomic", "coloured"])
@pytest.mark.parametrize("deg,k2", [(1, 0.0), (2, 0.0), (1, 3.5), (2, 3.5)])
def test_poisson_matrix(cuda, oracle, capi, deg, k2, mode):
    from dolfinx_gb300 import fem

    m, V, kappa, f, rp, cols = problem(oracle, (5, 4, 6), deg)
    a = fem.poisson_form(V, kappa, k2=k2)
    bnd = boundary_nodes(V)
    bc = fem.dirichletbc(0.0, bnd, V)
    A = fem.assemble_matrix(a, bcs=[bc], mode=mode)
    mk = np.zeros(V.num_nodes, np.int8)
    mk[bnd] = 1
    ref = oracle.assemble_matrix(0, deg, m.cells, m.x, V.dofmap, rp, cols, kappa=kappa, k2=k2,
                                 bc_markers=mk)
    oracle.set_diagonal(1, rp, cols, ref, bnd)
    np.testing.assert_array_equal(A.row_ptr.cpu().numpy(), rp)
    np.testing.assert_array_equal(A.cols.cpu().numpy(), cols)
    assert_close(A.vals.cpu().numpy(), ref)


def test_matrix_without_slot_map_and_without_bcs(cuda, oracle, capi):
    from dolfinx_gb300 import fem

    m, V, kappa, f, rp, cols = problem(oracle, (3, 5, 4), 2, seed=3)
    a = fem.poisson_form(V, kappa)
    A = fem.assemble_matrix(a, use_slot_map=False)
    ref = oracle.assemble_matrix(0, 2, m.cells, m.x, V.dofmap, rp, cols, kappa=kappa)
    assert_close(A.vals.cpu().numpy(), ref)
    # accumulate semantics: assembling again doubles (test_assembler.py:124-165)
    asm = fem.MatrixAssembler(a, A=A)
    asm.assemble(zero=False)
    assert_close(A.vals.cpu().numpy(), 2 * ref)


def test_coloured_mode_is_deterministic(cuda, oracle, capi):
    from dolfinx_gb300 import fem

    m, V, kappa, f, rp, cols = problem(oracle, (6, 6, 6), 2, seed=4)
    a = fem.poisson_form(V, kappa)
    A1 = fem.assemble_matrix(a, mode="coloured").vals.cpu().numpy()
    A2 = fem.assemble_matrix(a, mode="coloured").vals.cpu().numpy()
    np.testing.assert_array_equal(A1, A2)


@pytest.mark.parametrize("mode", ["atomic", "coloured"])
def test_elasticity_matrix(cuda, oracle, capi, mode):
    from dolfinx_gb300 import fem

    m, V, E, f, rp, cols = problem(oracle, (4, 2, 2), 2, seed=5, bs=3)
    E = 1e3 * E
    a = fem.elasticity_form(V, E, nu=0.3)
    X = V.tabulate_dof_coordinates()
    clamp = np.flatnonzero(np.isclose(X[:, 0], 0)).astype(np.int32)
    bc = fem.dirichletbc(np.zeros(3), clamp, V)
    A = fem.assemble_matrix(a, bcs=[bc], mode=mode)
    mk = np.zeros(V.num_dofs, np.int8)
    mk[bc.dofs] = 1
    ref = oracle.assemble_matrix(1, 2, m.cells, m.x, V.dofmap, rp, cols, kappa=E, nu=0.3,
                                 bc_markers=mk)
    oracle.set_diagonal(3, rp, cols, ref, bc.dofs)
    assert_close(A.vals.cpu().numpy(), ref)


@pytest.mark.parametrize("mode", ["atomic", "coloured"])
@pytest.mark.parametrize("deg", [1, 2])
def test_source_vector(cuda, oracle, capi, deg, mode):
    from dolfinx_gb300 import fem

    m, V, kappa, f, rp, cols = problem(oracle, (4, 5, 3), deg, seed=6)
    b = fem.assemble_vector(fem.source_form(V, f), mode=mode)
    ref = oracle.assemble_vector(0, deg, m.cells, m.x, V.dofmap, V.num_nodes, f=f)
    assert_close(b.cpu().numpy(), ref)


def test_body_force_vector(cuda, oracle, capi):
    from dolfinx_gb300 import fem

    m, V, E, f, rp, cols = problem(oracle, (4, 2, 2), 2, bs=3)
    b = fem.assemble_vector(fem.body_force_form(V, (0.5, 0.0, -1.0)))
    ref = oracle.assemble_vector(1, 2, m.cells, m.x, V.dofmap, V.num_nodes,
                                 fvec=np.array([0.5, 0.0, -1.0]))
    assert_close(b.cpu().numpy(), ref)


@pytest.mark.parametrize("mode", ["atomic", "coloured"])
@pytest.mark.parametrize("deg,bs", [(1, 1), (2, 1), (2, 3)])
def test_lifting_and_set_bc(cuda, oracle, capi, deg, bs, mode):
    from dolfinx_gb300 import fem

    m, V, kappa, f, rp, cols = problem(oracle, (3, 4, 3), deg, seed=8, bs=bs)
    rng = np.random.default_rng(9)
    X = V.tabulate_dof_coordinates()
    nodes = np.flatnonzero(np.isclose(X[:, 0], 0) | np.isclose(X[:, 2], 1)).astype(np.int32)
    gfull = rng.standard_normal(V.num_dofs)
    x0 = rng.standard_normal(V.num_dofs)
    bc = fem.dirichletbc(gfull, nodes, V)
    a = (fem.poisson_form(V, kappa, k2=0.7) if bs == 1 else fem.elasticity_form(V, kappa, 0.3))
    b0 = rng.standard_normal(V.num_dofs)
    b = torch.from_numpy(b0.copy()).cuda()
    x0d = torch.from_numpy(x0).cuda()
    fem.apply_lifting(b, [a], [[bc]], x0=[x0d], alpha=-0.5, mode=mode)
    mk = np.zeros(V.num_dofs, np.int8)
    mk[bc.dofs] = 1
    g = np.zeros(V.num_dofs)
    g[bc.dofs] = gfull[bc.dofs]
    ref = oracle.apply_lifting(b0.copy(), 0 if bs == 1 else 1, deg, m.cells, m.x, V.dofmap, mk, g,
                               kappa=kappa, k2=0.7, nu=0.3, x0=x0, alpha=-0.5)
    assert_close(b.cpu().numpy(), ref)
    fem.set_bc(b, [bc], x0=x0d, alpha=2.0)
    ref = oracle.set_bc(ref, bc.dofs, g, x0=x0, alpha=2.0)
    assert_close(b.cpu().numpy(), ref)


@pytest.mark.parametrize("mode", ["atomic", "coloured"])
@pytest.mark.parametrize("deg,bs,shape", [(2, 1, (9, 8, 7)), (1, 1, (12, 9, 8)),
                                          (2, 3, (8, 8, 6))])
def test_lifting_over_several_scan_ranges(cuda, oracle, capi, deg, bs, shape, mode):
    """Lifting compacts the constrained cells of each 2048-cell scan range in
    shared memory: meshes of 2,304-5,184 cells span two or three ranges, and
    constraints on one face only leave most batches partly filled."""
    from dolfinx_gb300 import fem

    m, V, kappa, f, rp, cols = problem(oracle, shape, deg, seed=11, bs=bs)
    rng = np.random.default_rng(12)
    X = V.tabulate_dof_coordinates()
    nodes = np.flatnonzero(np.isclose(X[:, 1], 1)).astype(np.int32)
    gfull = rng.standard_normal(V.num_dofs)
    bc = fem.dirichletbc(gfull, nodes, V)
    a = (fem.poisson_form(V, kappa) if bs == 1 else fem.elasticity_form(V, kappa, 0.3))
    b0 = rng.standard_normal(V.num_dofs)
    b = torch.from_numpy(b0.copy()).cuda()
    fem.apply_lifting(b, [a], [[bc]], mode=mode)
    mk = np.zeros(V.num_dofs, np.int8)
    mk[bc.dofs] = 1
    g = np.zeros(V.num_dofs)
    g[bc.dofs] = gfull[bc.dofs]
    ref = oracle.apply_lifting(b0.copy(), 0 if bs == 1 else 1, deg, m.cells, m.x, V.dofmap, mk, g,
                               kappa=kappa, nu=0.3)
    assert_close(b.cpu().numpy(), ref)
    assert np.abs(b.cpu().numpy() - b0).max() > 0  # the constraint did lift


def test_entry_not_in_sparsity(cuda, oracle, capi):
    from dolfinx_gb300 import fem, la

    m, V, kappa, f, rp, cols = problem(oracle, (2, 2, 2), 1)
    a = fem.poisson_form(V, kappa)
    # a diagonal-only pattern cannot hold the element matrices
    n = V.num_nodes
    A = la.MatrixCSR(torch.arange(n + 1, dtype=torch.int64).cuda(),
                     torch.arange(n, dtype=torch.int32).cuda(),
                     torch.zeros(n, dtype=torch.float64).cuda())
    with pytest.raises(capi.DfxError, match="Entry not in sparsity"):
        fem.MatrixAssembler(a, A=A)
    with pytest.raises(capi.DfxError, match="Entry not in sparsity"):
        fem.MatrixAssembler(a, A=A, use_slot_map=False).assemble()
