"""Value parity at the benchmark configurations (GPU): the P2 Poisson
64^3 x 6 matrix and right-hand side (1.57M cells, seed-0 lognormal kappa,
uniform f, u = 0 on x = 0 and x = 1) against the oracle at 1e-12, and the
P1 16^3 x 6 configuration with its exact inputs (kappa = 1,
f = sin(pi x) sin(pi y) sin(pi z) interpolated into P1, u = 0 on the whole
boundary) through assembly and Jacobi-PCG to rtol 1e-10; and the vector P2
elasticity system of the 4 x 1 x 1 box on 96 x 24 x 24 x 6 tetrahedra
(331,776 cells, 3x3 blocks, E lognormal(log 1e3, 0.5) from seed 3, nu = 0.3,
body force (0, 0, -1), clamped at x = 0) against the oracle at 1e-12."""

import numpy as np
import pytest
import torch

from gpu_util import assert_close

pytestmark = pytest.mark.gpu


def _boundary(V, test):
    X = V.tabulate_dof_coordinates()
    return np.flatnonzero(test(X)).astype(np.int32)


def _oracle_system(oracle, m, V, kappa, f, bnd):
    rp, cols = oracle.sparsity(V.num_nodes, V.dofmap)
    mk = np.zeros(V.num_nodes, np.int8)
    mk[bnd] = 1
    A = oracle.assemble_matrix(0, V.degree, m.cells, m.x, V.dofmap, rp, cols, kappa=kappa,
                               bc_markers=mk)
    oracle.set_diagonal(1, rp, cols, A, bnd)
    b = oracle.assemble_vector(0, V.degree, m.cells, m.x, V.dofmap, V.num_nodes, f=f)
    oracle.apply_lifting(b, 0, V.degree, m.cells, m.x, V.dofmap, mk, np.zeros(V.num_nodes),
                         kappa=kappa)
    oracle.set_bc(b, bnd, np.zeros(V.num_nodes))
    return rp, cols, A, b


def test_p2_64_matrix_and_rhs_match_oracle(cuda, oracle):
    from dolfinx_gb300 import fem, mesh

    m = mesh.create_unit_cube(64, 64, 64)
    V = fem.functionspace(m, ("Lagrange", 2))
    rng = np.random.default_rng(0)
    kappa = np.exp(rng.normal(0.0, 1.0, m.num_cells))
    f = rng.uniform(-1.0, 1.0, m.num_nodes)
    bnd = _boundary(V, lambda X: np.isclose(X[:, 0], 0.0) | np.isclose(X[:, 0], 1.0))
    bc = fem.dirichletbc(0.0, bnd, V)
    a = fem.poisson_form(V, kappa)
    A = fem.assemble_matrix(a, bcs=[bc])
    b = fem.RhsAssembler(fem.source_form(V, f), a, [bc]).assemble()
    rp, cols, Ar, br = _oracle_system(oracle, m, V, kappa, f, bnd)
    np.testing.assert_array_equal(A.row_ptr.cpu().numpy(), rp)
    np.testing.assert_array_equal(A.cols.cpu().numpy(), cols)
    assert_close(A.vals.cpu().numpy(), Ar, rtol=1e-12)
    assert_close(b.cpu().numpy(), br, rtol=1e-12)


def test_p1_16_exact_inputs_through_cg(cuda, oracle):
    from dolfinx_gb300 import fem, la, mesh

    m = mesh.create_unit_cube(16, 16, 16)
    V = fem.functionspace(m, ("Lagrange", 1))
    assert (m.num_cells, V.num_nodes) == (24576, 4913)
    x = m.x
    f = np.sin(np.pi * x[:, 0]) * np.sin(np.pi * x[:, 1]) * np.sin(np.pi * x[:, 2])
    bnd = _boundary(V, lambda X: np.any(np.isclose(X, 0.0) | np.isclose(X, 1.0), axis=1))
    assert bnd.size == 17 ** 3 - 15 ** 3 == 1538
    bc = fem.dirichletbc(0.0, bnd, V)
    a = fem.poisson_form(V, 1.0)
    A = fem.assemble_matrix(a, bcs=[bc])
    b = fem.RhsAssembler(fem.source_form(V, f), a, [bc]).assemble()
    rp, cols, Ar, br = _oracle_system(oracle, m, V, None, f, bnd)
    assert A.nnz == rp[-1] == 66961
    assert_close(A.vals.cpu().numpy(), Ar, rtol=1e-12)
    assert_close(b.cpu().numpy(), br, rtol=1e-12)
    xg, res = la.cg(A, b, rtol=1e-10)
    dinv = 1.0 / Ar[[np.searchsorted(cols[rp[i]:rp[i + 1]], i) + rp[i] for i in range(V.num_nodes)]]
    xo, its = oracle.cg(rp, cols, Ar, br, dinv=dinv, rtol=1e-10)
    assert res.status == 0 and abs(res.iterations - abs(its)) <= 2
    r = br - oracle.spmv(rp, cols, Ar, xg.cpu().numpy())
    assert np.linalg.norm(r) / np.linalg.norm(br) < 1e-10 * 1.0001
    assert np.linalg.norm(xg.cpu().numpy() - xo) / np.linalg.norm(xo) < 1e-8


def test_elasticity_96x24x24_matrix_and_rhs_match_oracle(cuda, oracle):
    from dolfinx_gb300 import fem, mesh

    m = mesh.create_box(((0.0, 0.0, 0.0), (4.0, 1.0, 1.0)), (96, 24, 24))
    V = fem.functionspace(m, ("Lagrange", 2, (3,)))
    assert (m.num_cells, V.num_dofs) == (331776, 1390179)
    rng = np.random.default_rng(3)
    E = np.exp(rng.normal(np.log(1e3), 0.5, m.num_cells))
    X = V.tabulate_dof_coordinates()
    clamp = np.flatnonzero(np.isclose(X[:, 0], 0.0)).astype(np.int32)
    bc = fem.dirichletbc(np.zeros(3), clamp, V)
    a = fem.elasticity_form(V, torch.from_numpy(E).cuda(), 0.3)
    A = fem.assemble_matrix(a, bcs=[bc])
    b = fem.RhsAssembler(fem.body_force_form(V, (0.0, 0.0, -1.0)), a, [bc]).assemble()
    rp, cols = oracle.sparsity(V.num_nodes, V.dofmap)
    np.testing.assert_array_equal(A.row_ptr.cpu().numpy(), rp)
    np.testing.assert_array_equal(A.cols.cpu().numpy(), cols)
    assert A.nnz == 12957697
    mk = np.zeros(V.num_dofs, np.int8)
    mk[bc.dofs] = 1
    Ar = oracle.assemble_matrix(1, 2, m.cells, m.x, V.dofmap, rp, cols, kappa=E, nu=0.3,
                                bc_markers=mk)
    oracle.set_diagonal(3, rp, cols, Ar, bc.dofs)
    assert_close(A.vals.cpu().numpy(), Ar, rtol=1e-12)
    br = oracle.assemble_vector(1, 2, m.cells, m.x, V.dofmap, V.num_nodes,
                                fvec=np.array([0.0, 0.0, -1.0]))
    oracle.apply_lifting(br, 1, 2, m.cells, m.x, V.dofmap, mk, np.zeros(V.num_dofs),
                         kappa=E, nu=0.3)
    oracle.set_bc(br, bc.dofs, np.zeros(V.num_dofs))
    assert_close(b.cpu().numpy(), br, rtol=1e-12)
