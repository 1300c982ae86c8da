"""The CPU oracle against the reference's own code (golden vectors written
by tests/golden/make_golden.py from oracle/_ref) and against the
properties the reference's tests pin (cpp/test/matrix.cpp,
python/test/unit/fem/test_fem_pipeline.py, test_symmetry.py,
test_custom_assembler.py)."""

import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "reference_golden.npz")


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


@pytest.mark.parametrize("n", [(1, 1, 1), (2, 2, 2), (3, 2, 4), (5, 4, 3)])
def test_dual_graph_and_rcm_match_reference(oracle, golden, n):
    tag = "%dx%dx%d" % n
    raw, _ = oracle.box_tet_raw(*n)
    off, adj = oracle.dual_graph_tet(raw)
    np.testing.assert_array_equal(off, golden[f"dual_off_{tag}"])
    np.testing.assert_array_equal(adj, golden[f"dual_adj_{tag}"])
    r = oracle.reorder_rcm(off, adj)
    np.testing.assert_array_equal(r, golden[f"rcm_{tag}"])


@pytest.mark.parametrize("tag,n,kind", [("p2", (2, 2, 2), 0), ("el", (2, 1, 1), 1)])
def test_insert_and_spmv_match_reference(oracle, golden, tag, n, kind):
    cells, x = oracle.create_box_tet(*n)
    dm, nn = oracle.dofmap_tet(cells, 2)
    rp, cols = oracle.sparsity(nn, dm)
    np.testing.assert_array_equal(rp, golden[f"csr_rowptr_{tag}"])
    np.testing.assert_array_equal(cols, golden[f"csr_cols_{tag}"])
    bs = 3 if kind == 1 else 1
    # Replay the reference's insertion with the oracle's CSR search: the
    # oracle's assembly inserts with the same lower_bound semantics.
    rng = np.random.default_rng(7)
    vals = np.zeros(cols.size * bs * bs)
    for c in range(cells.shape[0]):
        Ae = rng.standard_normal((10 * bs) ** 2).reshape(10 * bs, 10 * bs)
        for i in range(10):
            row = dm[c, i]
            for j in range(10):
                p = rp[row] + np.searchsorted(cols[rp[row]:rp[row + 1]], dm[c, j])
                vals[p * bs * bs:(p + 1) * bs * bs] += Ae[bs * i:bs * i + bs,
                                                          bs * j:bs * j + bs].ravel()
    np.testing.assert_array_equal(vals, golden[f"csr_vals_{tag}"])
    y = golden[f"spmv_y0_{tag}"].copy()
    oracle.spmv(rp, cols, vals, golden[f"spmv_x_{tag}"], bs=bs, y=y)
    np.testing.assert_array_equal(y, golden[f"spmv_y_{tag}"])


def test_c1_counts(oracle):
    cells, x = oracle.create_box_tet(16, 16, 16)
    dm, n = oracle.dofmap_tet(cells, 1)
    rp, cols = oracle.sparsity(n, dm)
    assert cells.shape[0] == 24576 and n == 4913 and cols.size == 66961
    # P1 dofmap == geometry dofmap (both first-appearance numbered)
    np.testing.assert_array_equal(dm, cells)


def test_p2_laplacian_kills_constants(oracle):
    # cpp/test/matrix.cpp:66-120: P2 Laplacian on a 12^3 x 6 box, A 1 = 0
    cells, x = oracle.create_box_tet(12, 12, 12)
    dm, n = oracle.dofmap_tet(cells, 2)
    rp, cols = oracle.sparsity(n, dm)
    A = oracle.assemble_matrix(0, 2, cells, x, dm, rp, cols)
    y = oracle.spmv(rp, cols, A, np.ones(n))
    assert np.abs(y).max() < 1e-13


@pytest.mark.parametrize("deg", [1, 2])
def test_element_symmetry_and_row_sums(oracle, deg):
    rng = np.random.default_rng(1)
    coords = rng.standard_normal((4, 3))
    Ae = oracle.kernel_poisson(deg, coords, kappa=2.5, k2=0.0)
    np.testing.assert_allclose(Ae, Ae.T, rtol=0, atol=1e-13 * np.abs(Ae).max())
    np.testing.assert_allclose(Ae.sum(axis=1), 0.0, atol=1e-13 * np.abs(Ae).max())
    # mass part: sum of all entries = k2 * |T|
    M = oracle.kernel_poisson(deg, coords, kappa=0.0, k2=1.0)
    vol = abs(np.linalg.det((coords[1:] - coords[0]).T)) / 6
    assert abs(M.sum() - vol) < 1e-13 * vol


def test_elasticity_rigid_motions(oracle):
    rng = np.random.default_rng(2)
    coords = rng.standard_normal((4, 3))
    Ae = oracle.kernel_elasticity(coords, E=3.0, nu=0.3)
    np.testing.assert_allclose(Ae, Ae.T, atol=1e-12 * np.abs(Ae).max())
    # P2 nodes
    e = [(2, 3), (1, 3), (1, 2), (0, 3), (0, 2), (0, 1)]
    X = np.vstack([coords, [(coords[a] + coords[b]) / 2 for a, b in e]])
    for rig in [np.tile([1.0, 0, 0], 10), np.cross([0, 0, 1.0], X).ravel()]:
        assert np.abs(Ae @ rig).max() < 1e-11 * np.abs(Ae).max()


def test_rhs_total_is_volume(oracle):
    # python/test/unit/fem/test_custom_assembler.py:162: sum(b) = |Omega| for f = 1
    for deg in (1, 2):
        cells, x = oracle.create_box_tet(3, 2, 2)
        dm, n = oracle.dofmap_tet(cells, deg)
        b = oracle.assemble_vector(0, deg, cells, x, dm, n)
        assert abs(b.sum() - 1.0) < 1e-13


@pytest.mark.parametrize("deg", [1, 2])
def test_pipeline_reproduces_polynomial(oracle, deg):
    # python/test/unit/fem/test_fem_pipeline.py:55-108: u = y^p is exact in P_p
    cells, x = oracle.create_box_tet(4, 3, 5)
    dm, n = oracle.dofmap_tet(cells, deg)
    rp, cols = oracle.sparsity(n, dm)
    # dof coordinates
    X = np.empty((n, 3))
    e = np.array([[2, 3], [1, 3], [1, 2], [0, 3], [0, 2], [0, 1]])
    xc = x[cells]
    X[dm[:, :4].ravel()] = xc.reshape(-1, 3)
    if deg == 2:
        X[dm[:, 4:].ravel()] = (0.5 * (xc[:, e[:, 0]] + xc[:, e[:, 1]])).reshape(-1, 3)
    u = X[:, 1] ** deg
    f_p1 = np.full(x.shape[0], -2.0 if deg == 2 else 0.0)  # -div grad y^2 = -2
    bnd = np.flatnonzero(np.isclose(X, 0).any(1) | np.isclose(X, 1).any(1))
    mk = np.zeros(n, np.int8)
    mk[bnd] = 1
    g = np.zeros(n)
    g[bnd] = u[bnd]
    A = oracle.assemble_matrix(0, deg, cells, x, dm, rp, cols, bc_markers=mk)
    oracle.set_diagonal(1, rp, cols, A, bnd.astype(np.int32))
    b = oracle.assemble_vector(0, deg, cells, x, dm, n, f=f_p1)
    oracle.apply_lifting(b, 0, deg, cells, x, dm, mk, g)
    oracle.set_bc(b, bnd.astype(np.int32), g)
    d = np.zeros(n)
    d = oracle.spmv(rp, cols, A, np.ones(n))  # just exercise; compute diagonal below
    diag = np.array([A[rp[i] + np.searchsorted(cols[rp[i]:rp[i + 1]], i)] for i in range(n)])
    uh, it = oracle.cg(rp, cols, A, b, dinv=1.0 / diag, rtol=1e-12)
    assert it > 0
    assert np.abs(uh - u).max() < 1e-9


def test_q4_action_exact_on_linears(oracle):
    """Q4 on perturbed trilinear hexahedra: the space holds the physical
    linear functions and 5^3 Gauss-Legendre integrates their stiffness rows
    exactly, so A u vanishes at interior nodes for linear u, A 1 = 0, and
    u^T A u = kappa |grad u|^2 vol(cube) = kappa."""
    from dolfinx_gb300 import matrix_free as mf

    dims = (2, 3, 2)
    v = mf.hex_box_vertices(*dims, perturb=0.05, seed=3)
    xyz = mf.node_coordinates(v, *dims)
    bnd = mf.boundary_mask(*dims)
    n = xyz.shape[0]
    assert n == 9 * 13 * 9
    one = np.ones(n)
    assert np.abs(oracle.q4_action(dims, v, one, apply_bc=False)).max() < 1e-12
    u = 0.3 + 1.0 * xyz[:, 0] - 2.0 * xyz[:, 1] + 0.5 * xyz[:, 2]
    y = oracle.q4_action(dims, v, u, kappa=1.7, apply_bc=False)
    assert np.abs(y[~bnd]).max() < 1e-11
    x = xyz[:, 0]
    e = x @ oracle.q4_action(dims, v, x, kappa=1.7, apply_bc=False)
    assert abs(e - 1.7) < 1e-12
    # With the boundary rows set to the identity the operator stays symmetric.
    rng = np.random.default_rng(0)
    a, b = rng.standard_normal(n), rng.standard_normal(n)
    a[bnd] = 0.0
    b[bnd] = 0.0
    assert abs(a @ oracle.q4_action(dims, v, b) - b @ oracle.q4_action(dims, v, a)) < 1e-11


def _dof_coords(x, cells, dm, n, deg):
    X = np.empty((n, 3))
    e = np.array([[2, 3], [1, 3], [1, 2], [0, 3], [0, 2], [0, 1]])
    xc = x[cells]
    X[dm[:, :4].ravel()] = xc.reshape(-1, 3)
    if deg == 2:
        X[dm[:, 4:].ravel()] = (0.5 * (xc[:, e[:, 0]] + xc[:, e[:, 1]])).reshape(-1, 3)
    return X


@pytest.mark.parametrize("n", [(1, 1, 1), (3, 2, 4)])
def test_exterior_facets_count_and_orientation(oracle, n):
    # every boundary square of the box is split into two triangles
    cells, x = oracle.create_box_tet(*n)
    fac = oracle.exterior_facets(cells)
    nx, ny, nz = n
    assert fac.shape[0] == 4 * (nx * ny + ny * nz + nx * nz)
    # each exterior facet lies on a face of the unit cube
    loc = np.array([[1, 2, 3], [0, 2, 3], [0, 1, 3], [0, 1, 2]])
    v = x[cells[fac[:, 0][:, None], loc[fac[:, 1]]]]  # (nf, 3, 3)
    on = (np.isclose(v, 0) | np.isclose(v, 1)).all(1).any(1)
    assert on.all()


@pytest.mark.parametrize("n", [(1, 1, 1), (3, 2, 4)])
def test_interior_facets_pair_cells_on_one_triangle(oracle, n):
    # 6 tetrahedra per box cell, 4 facets each: every facet not on the
    # boundary is shared by exactly two distinct cells, on the same triangle
    cells, x = oracle.create_box_tet(*n)
    fi = oracle.interior_facets(cells)
    nx, ny, nz = n
    assert 2 * fi.shape[0] == 24 * nx * ny * nz - 4 * (nx * ny + ny * nz + nx * nz)
    loc = np.array([[1, 2, 3], [0, 2, 3], [0, 1, 3], [0, 1, 2]])
    t0 = np.sort(cells[fi[:, 0][:, None], loc[fi[:, 1]]], axis=1)
    t1 = np.sort(cells[fi[:, 2][:, None], loc[fi[:, 3]]], axis=1)
    np.testing.assert_array_equal(t0, t1)
    assert (fi[:, 0] < fi[:, 2]).all()
    assert (np.diff(fi[:, 0] * 4 + fi[:, 1]) > 0).all()
    # no triangle appears twice
    assert np.unique(t0, axis=0).shape[0] == fi.shape[0]


@pytest.mark.parametrize("deg", [1, 2])
def test_facet_vector_totals(oracle, deg):
    # sum_i b_i = \int_Gamma g ds: g = 1 gives the surface area of the box,
    # g = x gives 3 on the unit cube (faces x=1: 1, y,z faces: 1/2 each)
    cells, x = oracle.create_box_tet(3, 2, 4, p1=(1.5, 1.0, 2.0))
    dm, n = oracle.dofmap_tet(cells, deg)
    fac = oracle.exterior_facets(cells)
    b = oracle.assemble_vector_facets(deg, fac, cells, x, dm, n)
    assert abs(b.sum() - 2 * (1.5 * 1 + 1 * 2 + 1.5 * 2)) < 1e-12
    if deg == 2:  # P2 vertex functions integrate to zero on a triangle
        assert np.abs(b[dm[:, :4].ravel()]).max() < 1e-14
    cells, x = oracle.create_box_tet(3, 3, 2)
    dm, n = oracle.dofmap_tet(cells, deg)
    fac = oracle.exterior_facets(cells)
    b = oracle.assemble_vector_facets(deg, fac, cells, x, dm, n, g=x[:, 0].copy())
    assert abs(b.sum() - 3.0) < 1e-12


@pytest.mark.parametrize("deg", [1, 2])
def test_facet_mass_totals(oracle, deg):
    # 1^T M 1 = alpha |Gamma|; the facet mass is symmetric
    cells, x = oracle.create_box_tet(2, 3, 2)
    dm, n = oracle.dofmap_tet(cells, deg)
    rp, cols = oracle.sparsity(n, dm)
    fac = oracle.exterior_facets(cells)
    M = oracle.assemble_matrix_facets(deg, fac, cells, x, dm, rp, cols, alpha_const=2.5)
    assert abs(M.sum() - 2.5 * 6.0) < 1e-12
    import scipy.sparse as sp
    S = sp.csr_matrix((M, cols, rp), shape=(n, n))
    assert abs(S - S.T).max() < 1e-15


@pytest.mark.parametrize("deg", [1, 2])
def test_functionals_on_polynomials(oracle, deg):
    # a(1, 1) = k2 |Omega|; a(x, x) = \int kappa for linear x; L(1) = \int f
    cells, x = oracle.create_box_tet(3, 2, 2)
    dm, n = oracle.dofmap_tet(cells, deg)
    X = _dof_coords(x, cells, dm, n, deg)
    kappa = np.exp(np.random.default_rng(1).normal(0, 1, cells.shape[0]))
    one = np.ones(n)
    assert abs(oracle.assemble_scalar(0, deg, cells, x, dm, one, k2=3.0) - 3.0) < 1e-13
    vol = np.abs(np.linalg.det(x[cells[:, 1:]] - x[cells[:, :1]])) / 6
    ref = (kappa * vol).sum()
    got = oracle.assemble_scalar(0, deg, cells, x, dm, X[:, 0].copy(), kappa=kappa)
    assert abs(got - ref) < 1e-13 * ref
    f = 1.0 + x[:, 1]  # \int (1 + y) dx = 1.5
    assert abs(oracle.assemble_scalar(1, deg, cells, x, dm, one, f=f) - 1.5) < 1e-13


@pytest.mark.parametrize("tag", ["p1", "p2"])
def test_sparsity_matches_reference(oracle, golden, tag, capi):
    """The cell sparsity pattern of the reference's own SparsityPattern
    (la/SparsityPattern.cpp, compiled from its sources on one rank) against
    the oracle and the product's host builder, bit for bit."""
    import ctypes as C

    dm = golden[f"sp_dofmap_{tag}"]
    rp_ref, cols_ref = golden[f"sp_rowptr_{tag}"], golden[f"sp_cols_{tag}"]
    n = rp_ref.size - 1
    rp, cols = oracle.sparsity(n, dm)
    np.testing.assert_array_equal(rp, rp_ref)
    np.testing.assert_array_equal(cols, cols_ref)
    rp2 = np.empty(n + 1, np.int64)
    nnz = C.c_int64(0)
    L = capi.lib()
    capi.check(L.dfx_sparsity_create(n, dm.shape[0], dm.shape[1], dm.ctypes.data, rp2.ctypes.data,
                                     None, C.byref(nnz)))
    cols2 = np.empty(nnz.value, np.int32)
    capi.check(L.dfx_sparsity_create(n, dm.shape[0], dm.shape[1], dm.ctypes.data, rp2.ctypes.data,
                                     cols2.ctypes.data, C.byref(nnz)))
    np.testing.assert_array_equal(rp2, rp_ref)
    np.testing.assert_array_equal(cols2, cols_ref)


def test_threaded_step_matches_serial_oracle(oracle):
    """The threaded full step behind the CPU baseline (colour-class cell
    loops, row-split Jacobi-PCG) gives the serial oracle's matrix and
    right-hand side, independently of the thread count, and solves to the
    requested residual."""
    cells, x = oracle.create_box_tet(6, 5, 4)
    dm, nn = oracle.dofmap_tet(cells, 2)
    rp, cols = oracle.sparsity(nn, dm)
    rng = np.random.default_rng(5)
    kappa = np.exp(rng.normal(0, 1, cells.shape[0]))
    f = rng.uniform(-1, 1, x.shape[0])
    X = np.zeros((nn, 3))
    X[dm[:, :4]] = x[cells]
    for e, (a, b) in enumerate(((2, 3), (1, 3), (1, 2), (0, 3), (0, 2), (0, 1))):
        X[dm[:, 4 + e]] = 0.5 * (x[cells[:, a]] + x[cells[:, b]])
    bnd = np.flatnonzero(np.isclose(X[:, 0], 0) | np.isclose(X[:, 0], 1)).astype(np.int32)
    order, off = oracle.colour_cells(dm, nn)
    # no two cells of a colour share a dof
    for k in range(off.size - 1):
        d = dm[order[off[k]:off[k + 1]]].ravel()
        assert np.unique(d).size == d.size
    assert np.array_equal(np.sort(order), np.arange(cells.shape[0]))
    runs = [oracle.poisson_step_threaded(2, cells, x, dm, nn, bnd, rp, cols, (order, off),
                                         kappa=kappa, f=f, rtol=1e-11, threads=t)
            for t in (1, 3)]
    assert np.array_equal(runs[0][2], runs[1][2]) and np.array_equal(runs[0][3], runs[1][3])
    mk = np.zeros(nn, np.int8)
    mk[bnd] = 1
    A = oracle.assemble_matrix(0, 2, cells, x, dm, rp, cols, kappa=kappa, bc_markers=mk)
    oracle.set_diagonal(1, rp, cols, A, bnd)
    b = oracle.assemble_vector(0, 2, cells, x, dm, nn, f=f)
    oracle.apply_lifting(b, 0, 2, cells, x, dm, mk, np.zeros(nn), kappa=kappa)
    oracle.set_bc(b, bnd, np.zeros(nn))
    for it, sec, vals, bt, u in runs:
        assert it > 0 and all(s >= 0 for s in sec)
        assert np.abs(vals - A).max() <= 1e-14 * np.abs(A).max()
        assert np.abs(bt - b).max() <= 1e-14 * np.abs(b).max()
        r = b - oracle.spmv(rp, cols, A, u)
        assert np.linalg.norm(r) / np.linalg.norm(b) < 1e-11 * 1.001


def test_interior_facet_pattern_and_penalty_oracle(oracle, capi):
    """The product's macro-element pattern (cells plus interior-facet macro
    elements) equals the oracle's pattern of the same elements and contains
    the cell pattern; the oracle's interior penalty is symmetric, positive
    semi-definite and zero on quadratics (P2)."""
    from dolfinx_gb300 import fem, mesh

    m = mesh.create_unit_cube(3, 4, 3)
    V = fem.functionspace(m, ("Lagrange", 2), device="cpu")
    quads = m.interior_facets()
    rp, cols = V.sparsity_with_interior_facets(quads)
    macro = np.concatenate([np.concatenate([V.dofmap, V.dofmap], axis=1),
                            np.concatenate([V.dofmap[quads[:, 0]], V.dofmap[quads[:, 2]]],
                                           axis=1)])
    rp0, cols0 = oracle.sparsity(V.num_nodes, macro)
    np.testing.assert_array_equal(rp, rp0)
    np.testing.assert_array_equal(cols, cols0)
    rpc, colsc = V.sparsity()
    for r in range(V.num_nodes):
        assert set(colsc[rpc[r]:rpc[r + 1]]) <= set(cols[rp[r]:rp[r + 1]])
    vals = oracle.assemble_matrix_interior_facets(2, quads, m.cells, m.x, V.dofmap, rp, cols)
    import scipy.sparse as sp

    M = sp.csr_matrix((vals, cols, rp), shape=(V.num_nodes,) * 2).toarray()
    assert np.abs(M - M.T).max() <= 1e-12 * np.abs(M).max()
    assert np.linalg.eigvalsh(0.5 * (M + M.T)).min() >= -1e-10 * np.abs(M).max()
    X = V.tabulate_dof_coordinates()
    u = X[:, 0] ** 2 - X[:, 1] * X[:, 2] + 3 * X[:, 1]
    assert np.abs(M @ u).max() <= 1e-11 * np.abs(M).max()
