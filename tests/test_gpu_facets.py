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
