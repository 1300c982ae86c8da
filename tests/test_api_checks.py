"""Argument checks of the Python API, on the host (no GPU): every vector that
a kernel would read or write through a raw pointer is checked for device,
dtype, contiguity and length before the call, and Dirichlet dofs for range,
so that a wrong argument raises instead of reaching the GPU."""

import numpy as np
import pytest
import torch


def _csr(n=4, bs=1, dtype=torch.float64):
    from dolfinx_gb300 import la

    rp = torch.arange(n + 1, dtype=torch.int64)
    cols = torch.arange(n, dtype=torch.int32)
    return la.MatrixCSR(rp, cols, torch.ones(n * bs * bs, dtype=dtype), bs)


def test_check_vec_names_the_problem(capi):
    from dolfinx_gb300 import la

    cuda0 = torch.device("cuda", 0)
    with pytest.raises(TypeError, match="x must be a torch tensor"):
        la._check_vec(np.zeros(3), 3, torch.float64, cuda0, "x")
    with pytest.raises(ValueError, match=r"x must be on a CUDA device \(got cpu\)"):
        la._check_vec(torch.zeros(3, dtype=torch.float64), 3, torch.float64, cuda0, "x")


def test_matrix_rejects_host_vectors_and_bad_types(capi):
    from dolfinx_gb300 import la

    A = _csr()
    x = torch.zeros(4, dtype=torch.float64)
    with pytest.raises(ValueError, match="must be on"):
        A.mult(x, torch.zeros(4, dtype=torch.float64))
    with pytest.raises(ValueError, match="must be on"):
        A.matvec(x)
    with pytest.raises(TypeError, match="row_ptr must be int64"):
        la.MatrixCSR(torch.zeros(2, dtype=torch.int32), torch.zeros(1, dtype=torch.int32),
                     torch.zeros(1, dtype=torch.float64))
    with pytest.raises(TypeError, match="float64 or float32"):
        la.MatrixCSR(torch.zeros(2, dtype=torch.int64), torch.zeros(1, dtype=torch.int32),
                     torch.zeros(1, dtype=torch.int64))
    with pytest.raises(TypeError, match="expand_blocks needs float64"):
        _csr(dtype=torch.float32).expand_blocks()


def test_inner_product_rejects_host_vectors(capi):
    from dolfinx_gb300 import la

    a = torch.ones(5, dtype=torch.float64)
    with pytest.raises(ValueError, match="a must be on a CUDA device"):
        la.inner_product(a, a)


def test_dirichlet_dofs_must_lie_in_the_space(capi):
    from dolfinx_gb300 import fem, mesh

    V = fem.functionspace(mesh.create_unit_cube(2, 2, 2), ("Lagrange", 1), device="cpu")
    n = V.num_nodes
    with pytest.raises(ValueError, match=rf"\[0, {n}\)"):
        fem.dirichletbc(0.0, np.array([0, n]), V)
    with pytest.raises(ValueError, match="Dirichlet dofs"):
        fem.dirichletbc(0.0, np.array([-1, 2]), V)
    with pytest.raises(ValueError, match="Dirichlet dofs"):
        fem.dirichletbc(0.0, np.array([2 ** 33]), V)  # would wrap in int32
    bc = fem.dirichletbc(0.0, np.array([3, 1, 3]), V)
    assert bc.dofs.tolist() == [1, 3]
    assert fem.dirichletbc(0.0, np.zeros(0, np.int32), V).dofs.size == 0
    with pytest.raises(ValueError, match="constant or a full dof vector"):
        fem.dirichletbc(np.zeros(n + 1), np.array([1]), V)
    with pytest.raises(ValueError, match="x must be on"):
        bc.set(torch.zeros(n, dtype=torch.float64))


def test_forms_check_their_space(capi):
    from dolfinx_gb300 import fem, mesh

    m = mesh.create_unit_cube(2, 2, 2)
    V1 = fem.functionspace(m, ("Lagrange", 1), device="cpu")
    V3 = fem.functionspace(m, ("Lagrange", 2, (3,)), device="cpu")
    with pytest.raises(ValueError, match="vector P2"):
        fem.elasticity_form(V1)
    with pytest.raises(ValueError, match="vector P2"):
        fem.body_force_form(V1)
    with pytest.raises(ValueError, match="scalar space"):
        fem.facet_source_form(V3)
    with pytest.raises(ValueError, match="scalar space"):
        fem.facet_mass_form(V3)


def test_coefficients_and_facets_are_sized_for_the_mesh(capi):
    from dolfinx_gb300 import fem, mesh

    m = mesh.create_unit_cube(2, 2, 2)
    V = fem.functionspace(m, ("Lagrange", 2), device="cpu")
    with pytest.raises(ValueError, match=rf"kappa \(per cell\) must be a constant or {m.num_cells}"):
        fem.poisson_form(V, np.ones(m.num_cells - 1))
    with pytest.raises(ValueError, match=rf"f \(per geometry node\).* {m.num_nodes} values"):
        fem.source_form(V, np.ones(V.num_nodes))  # P2 nodes, not geometry nodes
    with pytest.raises(ValueError, match="alpha"):
        fem.facet_mass_form(V, np.ones(3))
    with pytest.raises(ValueError, match="local facet < 4"):
        fem.facet_source_form(V, 1.0, facets=np.array([[0, 4]]))
    with pytest.raises(ValueError, match=rf"cell < {m.num_cells}"):
        fem.facet_mass_form(V, 1.0, facets=np.array([[m.num_cells, 0]]))
    with pytest.raises(ValueError, match="cell <"):
        fem.facet_mass_form(V, 1.0, facets=np.array([[-1, 0]]))
    # well-formed ones build (the space is on the host here)
    assert fem.poisson_form(V, np.ones(m.num_cells)).kappa.numel() == m.num_cells
    assert fem.source_form(V, np.ones(m.num_nodes)).f.numel() == m.num_nodes
    assert fem.facet_source_form(V, 1.0, facets=np.zeros((0, 2), np.int32)).facets.shape == (0, 2)
    assert fem.facet_mass_form(V, 2.0).facets.shape == (m.exterior_facets().shape[0], 2)


def test_matrix_shapes_are_checked(capi):
    from dolfinx_gb300 import fem, la, mesh

    rp = torch.arange(5, dtype=torch.int64)
    cols = torch.arange(4, dtype=torch.int32)
    with pytest.raises(ValueError, match="need 36 values"):
        la.MatrixCSR(rp, cols, torch.zeros(4, dtype=torch.float64), 3)
    with pytest.raises(ValueError, match="1-D"):
        la.MatrixCSR(rp.reshape(5, 1), cols, torch.zeros(4, dtype=torch.float64))
    V = fem.functionspace(mesh.create_unit_cube(2, 2, 2), ("Lagrange", 1), device="cpu")
    with pytest.raises(ValueError, match=rf"the space needs {V.num_nodes}x{V.num_nodes}"):
        fem.MatrixAssembler(fem.poisson_form(V), A=_csr(4))
    n = V.num_nodes
    A = la.MatrixCSR(torch.arange(n + 1, dtype=torch.int64), torch.arange(n, dtype=torch.int32),
                     torch.zeros(n, dtype=torch.float64))
    with pytest.raises(ValueError, match="CUDA device"):
        fem.MatrixAssembler(fem.poisson_form(V), A=A)
