"""Exterior-facet integrals and functionals against the oracle, which
integrates on the facets by quadrature (the GPU uses closed-form triangle
integrals). Tolerance: 1e-12 relative to the largest entry (FP64)."""

import numpy as np
import pytest
import torch

from gpu_util import assert_close, problem

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("deg", [1, 2])
@pytest.mark.parametrize("g_kind", ["const", "p1"])
def test_facet_vector(cuda, oracle, capi, deg, g_kind):
    from dolfinx_gb300 import fem

    m, V, kappa, f, rp, cols = problem(oracle, (5, 4, 6), deg, seed=31)
    g = 2.5 if g_kind == "const" else f
    b = fem.assemble_vector(fem.facet_source_form(V, g))
    fac = m.exterior_facets()
    ref = oracle.assemble_vector_facets(deg, fac, m.cells, m.x, V.dofmap, V.num_nodes,
                                        g=None if g_kind == "const" else f, g_const=2.5)
    assert_close(b.cpu().numpy(), ref)
    if g_kind == "const":
        assert abs(b.sum().item() - 2.5 * 6.0) < 1e-12


@pytest.mark.parametrize("deg", [1, 2])
@pytest.mark.parametrize("with_bc", [False, True])
@pytest.mark.parametrize("slot_map", [True, False])
def test_facet_mass(cuda, oracle, capi, deg, with_bc, slot_map):
    from dolfinx_gb300 import fem

    m, V, alpha, f, rp, cols = problem(oracle, (4, 5, 3), deg, seed=32)
    bcs, mk = [], None
    if with_bc:
        X = V.tabulate_dof_coordinates()
        nodes = np.flatnonzero(np.isclose(X[:, 2], 0)).astype(np.int32)
        bcs = [fem.dirichletbc(0.0, nodes, V)]
        mk = np.zeros(V.num_nodes, np.int8)
        mk[nodes] = 1
    a = fem.facet_mass_form(V, alpha)
    A = fem.MatrixAssembler(a, bcs, diagonal=0.0, use_slot_map=slot_map).assemble()
    ref = oracle.assemble_matrix_facets(deg, m.exterior_facets(), m.cells, m.x, V.dofmap, rp,
                                        cols, alpha=alpha, bc_markers=mk)
    assert_close(A.vals.cpu().numpy(), ref)


@pytest.mark.parametrize("deg", [1, 2])
def test_cell_plus_facet_form(cuda, oracle, capi, deg):
    """A form with a cell and an exterior-facet part (Helmholtz + Robin):
    one matrix, equal to the two oracle loops added."""
    from dolfinx_gb300 import fem, la

    m, V, kappa, f, rp, cols = problem(oracle, (5, 5, 4), deg, seed=33)
    a = fem.poisson_form(V, kappa, k2=0.5) + fem.facet_mass_form(V, 3.0)
    A = fem.assemble_matrix(a)
    ref = oracle.assemble_matrix(0, deg, m.cells, m.x, V.dofmap, rp, cols, kappa=kappa, k2=0.5)
    ref = oracle.assemble_matrix_facets(deg, m.exterior_facets(), m.cells, m.x, V.dofmap, rp,
                                        cols, alpha_const=3.0, vals=ref)
    assert_close(A.vals.cpu().numpy(), ref)
    # Robin problem: cell source + facet source, solved by CG
    L = fem.source_form(V, f) + fem.facet_source_form(V, 1.0)
    b = fem.assemble_vector(L)
    x, res = la.cg(A, b, rtol=1e-10)
    bh = b.cpu().numpy()
    r = bh - oracle.spmv(rp, cols, ref, x.cpu().numpy())
    assert np.linalg.norm(r) / np.linalg.norm(bh) < 1e-9


@pytest.mark.parametrize("deg", [1, 2])
@pytest.mark.parametrize("k2", [0.0, 1.5])
def test_assemble_scalar(cuda, oracle, capi, deg, k2):
    from dolfinx_gb300 import fem

    m, V, kappa, f, rp, cols = problem(oracle, (6, 5, 4), deg, seed=34)
    u = np.random.default_rng(35).standard_normal(V.num_nodes)
    ud = torch.from_numpy(u).cuda()
    energy = fem.assemble_scalar(fem.functional(fem.poisson_form(V, kappa, k2=k2), ud))
    ref = oracle.assemble_scalar(0, deg, m.cells, m.x, V.dofmap, u, kappa=kappa, k2=k2)
    assert abs(energy - ref) <= 1e-12 * abs(ref)
    got = fem.assemble_scalar(fem.functional(fem.source_form(V, f), ud))
    ref = oracle.assemble_scalar(1, deg, m.cells, m.x, V.dofmap, u, f=f)
    # L(u) sums terms of both signs: compare against the sum of magnitudes
    scale = oracle.assemble_scalar(1, deg, m.cells, m.x, V.dofmap, np.abs(u), f=np.abs(f))
    assert abs(got - ref) <= 1e-12 * scale
    # a(u, u) equals u^T A u of the assembled matrix
    A = fem.assemble_matrix(fem.poisson_form(V, kappa, k2=k2))
    uAu = float(ud @ A.matvec(ud))
    assert abs(energy - uAu) <= 1e-12 * abs(uAu)


def test_empty_facet_domain_and_functional_of_zero(cuda, oracle, capi):
    from dolfinx_gb300 import fem

    m, V, kappa, f, rp, cols = problem(oracle, (2, 2, 2), 2, seed=36)
    none = np.zeros((0, 2), np.int32)
    b = fem.assemble_vector(fem.facet_source_form(V, 1.0, facets=none))
    assert torch.count_nonzero(b) == 0
    A = fem.assemble_matrix(fem.facet_mass_form(V, 1.0, facets=none))
    assert torch.count_nonzero(A.vals) == 0
    zero = torch.zeros(V.num_dofs, dtype=torch.float64, device="cuda")
    assert fem.assemble_scalar(fem.functional(fem.poisson_form(V, kappa), zero)) == 0.0


# ---------------------------------------------------------------- interior facets
def _quad_area_sum(m, quads):
    x = m.x[m.cells[quads[:, 0]]]  # (nf, 4, 3)
    fv = np.array([[1, 2, 3], [0, 2, 3], [0, 1, 3], [0, 1, 2]])[quads[:, 1]]
    p = np.take_along_axis(x, fv[:, :, None], axis=1)
    n = np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0])
    return 0.5 * np.linalg.norm(n, axis=1).sum()


@pytest.mark.parametrize("deg", [1, 2])
@pytest.mark.parametrize("g_kind", ["const", "p1"])
def test_interior_facet_vector(cuda, oracle, capi, deg, g_kind):
    """int_F avg(g) avg(v) dS against the oracle's facet quadrature; with
    g = 1 the entries sum to the total interior facet area."""
    from dolfinx_gb300 import fem

    m, V, kappa, f, rp, cols = problem(oracle, (4, 3, 5), deg, seed=41)
    g = 1.0 if g_kind == "const" else f
    b = fem.assemble_vector(fem.interior_facet_source_form(V, g))
    quads = m.interior_facets()
    ref = oracle.assemble_vector_interior_facets(deg, quads, m.cells, m.x, V.dofmap,
                                                 V.num_nodes, g=None if g_kind == "const" else f,
                                                 g_const=1.0)
    assert_close(b.cpu().numpy(), ref)
    if g_kind == "const":
        total = _quad_area_sum(m, quads)
        assert abs(b.sum().item() - total) < 1e-11 * total


@pytest.mark.parametrize("deg", [1, 2])
@pytest.mark.parametrize("with_bc", [False, True])
def test_interior_penalty_matrix(cuda, oracle, capi, deg, with_bc):
    """The continuous interior penalty matrix against the oracle (its own
    quadrature and pull-back into the second cell), on the pattern with the
    facets' macro-element couplings; symmetric, and zero on polynomials of
    the space's degree (their gradients do not jump)."""
    from dolfinx_gb300 import fem

    m, V, gamma, f, _, _ = problem(oracle, (4, 4, 3), deg, seed=42)
    quads = m.interior_facets()
    rp, cols = V.sparsity_with_interior_facets(quads)
    bcs, mk = [], None
    if with_bc:
        X = V.tabulate_dof_coordinates()
        nodes = np.flatnonzero(np.isclose(X[:, 0], 0)).astype(np.int32)
        bcs = [fem.dirichletbc(0.0, nodes, V)]
        mk = np.zeros(V.num_nodes, np.int8)
        mk[nodes] = 1
    a = fem.interior_penalty_form(V, gamma)
    A = fem.MatrixAssembler(a, bcs, diagonal=0.0).assemble()
    np.testing.assert_array_equal(A.row_ptr.cpu().numpy(), rp)
    np.testing.assert_array_equal(A.cols.cpu().numpy(), cols)
    ref = oracle.assemble_matrix_interior_facets(deg, quads, m.cells, m.x, V.dofmap, rp, cols,
                                                 gamma=gamma, bc_markers=mk)
    assert_close(A.vals.cpu().numpy(), ref)
    if not with_bc:
        import scipy.sparse as sp

        M = sp.csr_matrix((A.vals.cpu().numpy(), cols, rp), shape=(V.num_nodes,) * 2)
        assert abs(M - M.T).max() <= 1e-12 * abs(M).max()
        X = V.tabulate_dof_coordinates()
        u = 1.0 + 2 * X[:, 0] - X[:, 1] + 0.5 * X[:, 2]
        if deg == 2:
            u = u + X[:, 0] * X[:, 1] - 2 * X[:, 2] ** 2
        assert np.abs(M @ u).max() <= 1e-10 * abs(M).max() * np.abs(u).max()


@pytest.mark.parametrize("deg", [1, 2])
def test_facet_lifting(cuda, oracle, capi, deg):
    """apply_lifting through exterior-facet (Robin mass) and interior-facet
    (penalty) terms: b = -A_F g restricted to the constrained columns, with
    A_F the facet matrix assembled without boundary conditions."""
    from dolfinx_gb300 import fem

    m, V, gamma, f, _, _ = problem(oracle, (4, 3, 4), deg, seed=43)
    quads = m.interior_facets()
    rp, cols = V.sparsity_with_interior_facets(quads)
    X = V.tabulate_dof_coordinates()
    nodes = np.flatnonzero(np.isclose(X[:, 1], 0)).astype(np.int32)
    gvals = np.zeros(V.num_nodes)
    gvals[nodes] = np.sin(3 * X[nodes, 0]) + X[nodes, 2]
    bc = fem.dirichletbc(gvals, nodes, V)
    for form, ref_matrix in (
            (fem.facet_mass_form(V, 2.0),
             lambda: oracle.assemble_matrix_facets(deg, m.exterior_facets(), m.cells, m.x,
                                                   V.dofmap, rp, cols, alpha_const=2.0)),
            (fem.interior_penalty_form(V, gamma),
             lambda: oracle.assemble_matrix_interior_facets(deg, quads, m.cells, m.x, V.dofmap,
                                                            rp, cols, gamma=gamma))):
        b = torch.zeros(V.num_dofs, dtype=torch.float64, device="cuda")
        fem.apply_lifting(b, [form], [[bc]])
        import scipy.sparse as sp

        M = sp.csr_matrix((ref_matrix(), cols, rp), shape=(V.num_nodes,) * 2)
        assert_close(b.cpu().numpy(), -(M @ gvals))


def test_poisson_with_interior_penalty_solves(cuda, oracle, capi):
    """A cell form plus the interior penalty, non-homogeneous Dirichlet data:
    assemble, lift through both terms, set_bc and CG; the solution satisfies
    the oracle's assembled system."""
    from dolfinx_gb300 import fem, la

    m, V, kappa, f, _, _ = problem(oracle, (5, 4, 4), 2, seed=44)
    quads = m.interior_facets()
    rp, cols = V.sparsity_with_interior_facets(quads)
    X = V.tabulate_dof_coordinates()
    nodes = np.flatnonzero(np.isclose(X[:, 0], 0) | np.isclose(X[:, 0], 1)).astype(np.int32)
    gvals = np.zeros(V.num_nodes)
    gvals[nodes] = 1.0 + X[nodes, 1] ** 2
    bc = fem.dirichletbc(gvals, nodes, V)
    a = fem.poisson_form(V, kappa) + fem.interior_penalty_form(V, 0.1)
    A = fem.assemble_matrix(a, bcs=[bc])
    b = fem.assemble_vector(fem.source_form(V, f))
    fem.apply_lifting(b, [a], [[bc]])
    fem.set_bc(b, [bc])
    x, res = la.cg(A, b, rtol=1e-11)
    mk = np.zeros(V.num_nodes, np.int8)
    mk[nodes] = 1
    Ar = oracle.assemble_matrix(0, 2, m.cells, m.x, V.dofmap, rp, cols, kappa=kappa,
                                bc_markers=mk)
    Ar = oracle.assemble_matrix_interior_facets(2, quads, m.cells, m.x, V.dofmap, rp, cols,
                                                gamma_const=0.1, bc_markers=mk, vals=Ar)
    oracle.set_diagonal(1, rp, cols, Ar, nodes)
    assert_close(A.vals.cpu().numpy(), Ar)
    # The oracle's right-hand side: source, lifting of the cell term and of
    # the penalty (-A_full g on constrained columns), then the BC values.
    import scipy.sparse as sp

    br = oracle.assemble_vector(0, 2, m.cells, m.x, V.dofmap, V.num_nodes, f=f)
    oracle.apply_lifting(br, 0, 2, m.cells, m.x, V.dofmap, mk, gvals, kappa=kappa)
    P = sp.csr_matrix((oracle.assemble_matrix_interior_facets(2, quads, m.cells, m.x, V.dofmap,
                                                               rp, cols, gamma_const=0.1),
                       cols, rp), shape=(V.num_nodes,) * 2)
    br -= P @ gvals
    oracle.set_bc(br, nodes, gvals)
    assert_close(b.cpu().numpy(), br)
    r = br - oracle.spmv(rp, cols, Ar, x.cpu().numpy())
    assert res.status == 0 and np.linalg.norm(r) / np.linalg.norm(br) < 1e-11 * 1.001
