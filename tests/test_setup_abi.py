"""CPU tests of the product library: it loads, exports every symbol that
include/dfx_gpu.h declares, and its host set-up (box mesh + RCM order,
dofmaps, sparsity, colouring) is bit-identical to the oracle."""

import ctypes as C

import numpy as np
import pytest


def test_library_exports_header_symbols(capi):
    lib = capi.lib()
    names = capi.declared_symbols()
    assert len(names) >= 20
    for name in names:
        assert hasattr(lib, name), name
    assert lib.dfx_abi_version() == 1


@pytest.mark.parametrize("n", [(1, 1, 1), (2, 3, 4), (7, 5, 6), (16, 16, 16)])
def test_mesh_matches_oracle(capi, oracle, n):
    from dolfinx_gb300 import mesh

    m = mesh.create_box(((0, 0, 0), (1.5, 1, 2)), n)
    cells, x = oracle.create_box_tet(*n, p1=(1.5, 1, 2))
    np.testing.assert_array_equal(m.cells, cells)
    np.testing.assert_array_equal(m.x, x)


@pytest.mark.parametrize("deg", [1, 2])
@pytest.mark.parametrize("n", [(2, 3, 4), (9, 8, 7)])
def test_dofmap_and_sparsity_match_oracle(capi, oracle, n, deg):
    from dolfinx_gb300 import fem, mesh

    m = mesh.create_unit_cube(*n)
    V = fem.functionspace(m, ("Lagrange", deg), device="cpu")
    dm, nn = oracle.dofmap_tet(m.cells, deg)
    assert V.num_nodes == nn
    np.testing.assert_array_equal(V.dofmap, dm)
    rp, cols = V.sparsity()
    rp0, cols0 = oracle.sparsity(nn, dm)
    np.testing.assert_array_equal(rp, rp0)
    np.testing.assert_array_equal(cols, cols0)


def test_colouring_is_valid(capi):
    from dolfinx_gb300 import fem, mesh

    m = mesh.create_unit_cube(6, 5, 4)
    V = fem.functionspace(m, ("Lagrange", 2), device="cpu")
    order, off = V.colouring()
    order = order.numpy()
    assert sorted(order.tolist()) == list(range(m.num_cells))
    for k in range(off.size - 1):
        cells = order[off[k]:off[k + 1]]
        d = V.dofmap[cells].ravel()
        assert np.unique(d).size == d.size, f"colour {k} shares a dof"


def test_invalid_box_is_rejected(capi):
    from dolfinx_gb300 import mesh

    with pytest.raises(capi.DfxError, match="At least one cell"):
        mesh.create_box(((0, 0, 0), (1, 1, 1)), (0, 1, 1))
    with pytest.raises(capi.DfxError, match="p\\[0\\] < p\\[1\\]"):
        mesh.create_box(((0, 0, 0), (1, 0, 1)), (1, 1, 1))


@pytest.mark.parametrize("n", [(1, 1, 1), (3, 2, 4), (6, 5, 7)])
def test_exterior_facets_match_oracle(capi, oracle, n):
    from dolfinx_gb300 import mesh

    m = mesh.create_unit_cube(*n)
    np.testing.assert_array_equal(m.exterior_facets(), oracle.exterior_facets(m.cells))


def test_exterior_facets_of_no_cells(capi):
    import ctypes as C

    nf = C.c_int32(-1)
    out = np.zeros(2, np.int32)
    cells = np.zeros(4, np.int32)
    capi.check(capi.lib().dfx_exterior_facets_tet(0, cells.ctypes.data, out.ctypes.data,
                                                  C.byref(nf)))
    assert nf.value == 0
