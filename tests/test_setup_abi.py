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


# The two largest boxes are large enough for the threaded paths: the dual
# graph's bucket sort and run fill, and the level-synchronous RCM team.
@pytest.mark.parametrize("n", [(1, 1, 1), (2, 3, 4), (7, 5, 6), (16, 16, 16), (24, 24, 24),
                               (30, 20, 26)])
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


@pytest.mark.parametrize("deg", [1, 2])
@pytest.mark.parametrize("n,reorder", [((24, 24, 24), True), ((30, 20, 26), False)])
def test_dofmap_matches_oracle_on_threads(capi, oracle, n, reorder, deg):
    """Boxes with tens of thousands of cells, so the dofmap's first-appearance
    passes run on several threads; RCM order and the unordered build order
    (a different cell order, so different first appearances). Two builds
    must agree bit for bit."""
    from dolfinx_gb300 import fem, mesh

    m = mesh.create_box(((0, 0, 0), (1, 1, 1)), n, reorder=reorder)
    dm, nn = oracle.dofmap_tet(m.cells, deg)
    V = fem.functionspace(m, ("Lagrange", deg), device="cpu")
    assert V.num_nodes == nn
    np.testing.assert_array_equal(V.dofmap, dm)
    V2 = fem.functionspace(m, ("Lagrange", deg), device="cpu")
    np.testing.assert_array_equal(V2.dofmap, V.dofmap)


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


@pytest.mark.parametrize("n", [(1, 1, 1), (3, 2, 4), (6, 5, 7), (24, 24, 24)])
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


@pytest.mark.parametrize("n", [(1, 1, 1), (3, 2, 4), (6, 5, 7), (24, 24, 24)])
def test_interior_facets_match_oracle(capi, oracle, n):
    from dolfinx_gb300 import mesh

    m = mesh.create_unit_cube(*n)
    got = m.interior_facets()
    np.testing.assert_array_equal(got, oracle.interior_facets(m.cells))
    # every facet of every cell is either exterior or one side of an interior facet
    assert 2 * got.shape[0] + m.exterior_facets().shape[0] == 4 * m.num_cells
    # the cell pairs are the edges of the facet-connected dual graph
    off, adj = m.dual_graph()
    src = np.repeat(np.arange(m.num_cells), np.diff(off))
    edges = np.stack([src, adj], 1)
    edges = edges[edges[:, 0] < edges[:, 1]]
    pairs = got[:, [0, 2]]
    np.testing.assert_array_equal(np.unique(pairs, axis=0), np.unique(edges, axis=0))
    assert np.unique(pairs, axis=0).shape[0] == pairs.shape[0]


def test_interior_facets_edge_cases(capi):
    import ctypes as C

    def interior(cells):
        cells = np.ascontiguousarray(cells, np.int32)
        nc = cells.size // 4
        out = np.full((max(2 * nc, 1), 4), -7, np.int32)
        nf = C.c_int32(-1)
        capi.check(capi.lib().dfx_interior_facets_tet(nc, cells.ctypes.data, out.ctypes.data,
                                                      C.byref(nf)))
        return out[: nf.value]

    assert interior(np.zeros(4, np.int32)[:0]).shape == (0, 4)
    assert interior([[0, 1, 2, 3]]).shape == (0, 4)
    # two cells glued on the triangle {1, 2, 3}: opposite vertex 0 in cell 0,
    # opposite vertex 4 (local 3) in cell 1
    np.testing.assert_array_equal(interior([[0, 1, 2, 3], [1, 2, 3, 4]]), [[0, 0, 1, 3]])
    # the same triangle in a third cell: not an interior facet (three cells)
    assert interior([[0, 1, 2, 3], [1, 2, 3, 4], [3, 2, 1, 5]]).shape == (0, 4)
    with pytest.raises(capi.DfxError, match="negative vertex index in cell 1"):
        interior([[0, 1, 2, 3], [1, 2, -3, 4]])
    nf = C.c_int32(0)
    with pytest.raises(capi.DfxError, match="invalid interior facet arguments"):
        capi.check(capi.lib().dfx_interior_facets_tet(-1, None, None, C.byref(nf)))


def test_autotuner_table_host_logic(capi):
    """The autotuner's table is host state: choices are keyed per workload
    (form kind, degree, mass term, cells, mode; matrix shape), validated
    against the candidates, and forgotten by dfx_tune_clear. Empty forms and
    matrices reach it without a GPU."""
    import ctypes as C

    L = capi.lib()
    capi.check(L.dfx_tune_clear())
    f = capi.Form(capi.FORM_POISSON, 2, 0, 0, None, None, None, None, 1.0, 0.0, 0.3, None,
                  (C.c_double * 3)())
    v = C.c_int32(0)

    def cpb(form, mode):
        capi.check(L.dfx_get_cells_per_block(C.byref(form), mode, C.byref(v)))
        return v.value

    assert cpb(f, 0) == 32 and cpb(f, 1) == 32
    capi.check(L.dfx_set_cells_per_block(C.byref(f), 0, 64))
    assert cpb(f, 0) == 64 and cpb(f, 1) == 32  # modes are separate workloads
    f.k2 = 1.0
    assert cpb(f, 0) == 32  # the mass term is part of the key
    assert L.dfx_set_cells_per_block(C.byref(f), 0, 48) == capi.DFX_ERR_INVALID
    e = capi.Form(capi.FORM_ELASTICITY, 2, 0, 0, None, None, None, None, 1.0, 0.0, 0.3, None,
                  (C.c_double * 3)())
    assert cpb(e, 0) == 4
    assert L.dfx_set_cells_per_block(C.byref(e), 0, 64) == capi.DFX_ERR_INVALID
    capi.check(L.dfx_set_cells_per_block(C.byref(e), 0, 8))
    assert cpb(e, 0) == 8
    capi.check(L.dfx_set_cells_per_block(C.byref(e), 0, 0))  # back to the default
    assert cpb(e, 0) == 4
    A = capi.Csr(0, 0, 1, capi.F64, 0, None, None, None)
    capi.check(L.dfx_get_spmv_lanes(C.byref(A), C.byref(v)))
    assert v.value == 4  # mean row length 0
    capi.check(L.dfx_set_spmv_lanes(C.byref(A), 16))
    capi.check(L.dfx_get_spmv_lanes(C.byref(A), C.byref(v)))
    assert v.value == 16
    assert L.dfx_set_spmv_lanes(C.byref(A), 3) == capi.DFX_ERR_INVALID
    capi.check(L.dfx_tune_clear())
    f.k2 = 0.0
    assert cpb(f, 0) == 32
    capi.check(L.dfx_get_spmv_lanes(C.byref(A), C.byref(v)))
    assert v.value == 4


def test_device_sparsity_workspace_is_sized_by_the_problem(capi):
    L = capi.lib()
    small = L.dfx_sparsity_device_workspace_bytes(100, 50, 10)
    big = L.dfx_sparsity_device_workspace_bytes(100000, 50000, 10)
    assert 0 < small < big
    assert big >= 50000 * 10 * 4  # the dof -> cell transpose
    assert L.dfx_sparsity_device_workspace_bytes(-1, 0, 4) == 0


def test_device_mesh_workspaces_are_sized_by_the_problem(capi):
    """Workspace sizes of the device box mesh, dual graph and RCM (host
    functions): growing with the problem, 0 for invalid sizes and for boxes
    whose cell indices overflow int32."""
    L = capi.lib()
    box = L.dfx_mesh_create_box_tet_device_workspace_bytes
    assert 0 < box(2, 2, 2, 1) < box(64, 64, 64, 1)
    assert box(64, 64, 64, 0) < box(64, 64, 64, 1)  # no dual graph, no ordering
    nc = 6 * 64 ** 3
    assert box(64, 64, 64, 1) >= 4 * nc * 4 * 2  # the box's cells and the reordered cells
    assert box(0, 1, 1, 1) == 0 and box(448, 448, 448, 1) == 0
    dual = L.dfx_mesh_dual_graph_tet_device_workspace_bytes
    assert 0 < dual(10, 20) < dual(10000, 3000)
    assert dual(10000, 3000) >= 2 * 4 * 10000 * 4  # facet lists and twins
    assert dual(-1, 0) == 0
    rcm = L.dfx_graph_reorder_rcm_device_workspace_bytes
    assert 0 < rcm(0) < rcm(1000) < rcm(10 ** 6)
    assert rcm(-1) == 0


def test_device_mesh_entries_check_arguments_on_the_host(capi):
    """Arguments are checked before any device work, so these calls need no
    GPU: an empty box, inverted corners, a NULL output, a short workspace."""
    import ctypes as C

    L = capi.lib()
    p0 = np.zeros(3)
    p1 = np.ones(3)
    buf = C.c_void_p(256)  # never dereferenced: each call fails its checks first
    assert L.dfx_mesh_create_box_tet_device(0, 1, 1, p0.ctypes.data, p1.ctypes.data, 1, buf, buf,
                                            buf, 1 << 30, None) == capi.DFX_ERR_INVALID
    assert L.dfx_mesh_create_box_tet_device(1, 1, 1, p1.ctypes.data, p0.ctypes.data, 1, buf, buf,
                                            buf, 1 << 30, None) == capi.DFX_ERR_INVALID
    assert L.dfx_mesh_create_box_tet_device(1, 1, 1, p0.ctypes.data, p1.ctypes.data, 1, None, buf,
                                            buf, 1 << 30, None) == capi.DFX_ERR_INVALID
    assert L.dfx_mesh_create_box_tet_device(4, 4, 4, p0.ctypes.data, p1.ctypes.data, 1, buf, buf,
                                            buf, 16, None) == capi.DFX_ERR_INVALID
    assert L.dfx_graph_reorder_rcm_device(10, buf, buf, buf, buf, 16, None) == \
        capi.DFX_ERR_INVALID
    assert L.dfx_mesh_dual_graph_tet_device(10, buf, 40, buf, buf, buf, 16, None) == \
        capi.DFX_ERR_INVALID


_THREADS_SCRIPT = r"""
import sys
import numpy as np
sys.path.insert(0, sys.argv[1])
from dolfinx_gb300 import fem, mesh
m = mesh.create_box(((0, 0, 0), (1, 1, 1)), (26, 22, 20))
V = fem.functionspace(m, ("Lagrange", 2), device="cpu")
np.savez(sys.argv[2], cells=m.cells, x=m.x, dofmap=V.dofmap, facets=m.exterior_facets(),
         interior=m.interior_facets())
"""


def test_host_setup_is_independent_of_the_thread_count(capi, tmp_path):
    """Mesh (dual-graph sort), dofmap (first appearance), exterior and
    interior facets built with 1, 3, 7 and 16 host threads are identical: the GPU host has a
    different core count from the machine the parity tests ran on."""
    import os
    import subprocess
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    script = tmp_path / "build_mesh.py"
    script.write_text(_THREADS_SCRIPT)
    out = {}
    for t in (1, 3, 7, 16):
        f = tmp_path / f"t{t}.npz"
        env = dict(os.environ, DFX_NUM_THREADS=str(t))
        subprocess.run([sys.executable, str(script), root, str(f)], check=True, env=env,
                       timeout=300)
        out[t] = np.load(f)
    for t in (3, 7, 16):
        for k in ("cells", "x", "dofmap", "facets", "interior"):
            np.testing.assert_array_equal(out[t][k], out[1][k])


def _dof_coordinates_numpy(m, V):
    """The dof points restated with numpy: vertices, then edge midpoints
    0.5 (a + b) in Basix edge order, zero for nodes that no cell holds."""
    edges = np.array([[2, 3], [1, 3], [1, 2], [0, 3], [0, 2], [0, 1]])
    X = np.zeros((V.num_nodes, 3))
    xc = m.x[m.cells]
    X[V.dofmap[:, :4].ravel()] = xc.reshape(-1, 3)
    if V.degree == 2:
        X[V.dofmap[:, 4:].ravel()] = (0.5 * (xc[:, edges[:, 0]] + xc[:, edges[:, 1]])).reshape(-1, 3)
    return X


@pytest.mark.parametrize("deg", [1, 2])
@pytest.mark.parametrize("n", [(1, 1, 1), (3, 4, 2), (20, 18, 16)])
def test_dof_coordinates_match_numpy(capi, n, deg):
    from dolfinx_gb300 import fem, mesh

    m = mesh.create_box(((-1.0, 0.25, 0.0), (2.0, 1.0, 3.5)), n)
    V = fem.functionspace(m, ("Lagrange", deg), device="cpu")
    X = V.tabulate_dof_coordinates()
    assert X.shape == (V.num_nodes, 3)
    np.testing.assert_array_equal(X, _dof_coordinates_numpy(m, V))
    if deg == 1:
        np.testing.assert_array_equal(X[V.dofmap], m.x[m.cells])


def test_dof_coordinates_checks_indices(capi):
    L = capi.lib()
    cells = np.array([[0, 1, 2, 3]], np.int32)
    x = np.zeros((4, 3))
    X = np.full((4, 3), 7.0)
    dm = np.array([[0, 1, 2, 4]], np.int32)  # node 4 of 4
    assert L.dfx_tabulate_dof_coordinates_tet(1, cells.ctypes.data, 4, x.ctypes.data,
                                              dm.ctypes.data, 1, 4,
                                              X.ctypes.data) == capi.DFX_ERR_INVALID
    assert (X == 7.0).all()  # nothing written
    assert L.dfx_tabulate_dof_coordinates_tet(1, cells.ctypes.data, 3, x.ctypes.data,
                                              dm.ctypes.data, 1, 5,
                                              X.ctypes.data) == capi.DFX_ERR_INVALID
    assert L.dfx_tabulate_dof_coordinates_tet(1, cells.ctypes.data, 4, x.ctypes.data,
                                              dm.ctypes.data, 3, 5,
                                              X.ctypes.data) == capi.DFX_ERR_UNSUPPORTED
    assert L.dfx_tabulate_dof_coordinates_tet(0, None, 0, None, None, 2, 0, None) == capi.DFX_OK


@pytest.mark.parametrize("deg", [1, 2])
@pytest.mark.parametrize("n", [(1, 1, 1), (3, 4, 2), (7, 7, 7), (20, 9, 13)])
def test_facet_closure_dofs_are_the_boundary_dofs(capi, n, deg):
    """The dofs on the exterior facets of a unit box are exactly the dofs
    whose point lies on its surface (a coordinate at 0 or 1)."""
    from dolfinx_gb300 import fem, mesh

    m = mesh.create_unit_cube(*n)
    V = fem.functionspace(m, ("Lagrange", deg), device="cpu")
    got = fem.locate_dofs_facets(V, m.exterior_facets())
    X = V.tabulate_dof_coordinates()
    ref = np.flatnonzero(np.isclose(X, 0.0).any(1) | np.isclose(X, 1.0).any(1))
    np.testing.assert_array_equal(got, ref)
    assert got.dtype == np.int32
    assert fem.locate_dofs_facets(V, np.zeros((0, 2), np.int32)).size == 0


# The two largest meshes take the threaded bucket sort with several threads.
@pytest.mark.parametrize("n,reorder", [((1, 1, 1), True), ((3, 2, 4), True), ((7, 5, 6), False),
                                       ((24, 24, 24), True), ((30, 20, 26), False)])
def test_dual_graph_matches_oracle(capi, oracle, n, reorder):
    from dolfinx_gb300 import mesh

    m = mesh.create_box(((0, 0, 0), (1, 1, 1)), n, reorder=reorder)
    off, adj = m.dual_graph()
    off0, adj0 = oracle.dual_graph_tet(m.cells.astype(np.int64))
    np.testing.assert_array_equal(off, off0)
    np.testing.assert_array_equal(adj, adj0)
    # each interior facet joins two cells: 4 nc - (boundary facets) = 2 edges
    nb = 4 * (n[0] * n[1] + n[1] * n[2] + n[0] * n[2])
    assert off[-1] == 4 * m.num_cells - nb


def test_dual_graph_rejects_bad_cells(capi):
    cells = np.array([[0, 1, 2, 7]], np.int32)
    off = np.empty(2, np.int32)
    adj = np.empty(4, np.int32)
    assert capi.lib().dfx_mesh_dual_graph_tet(1, cells.ctypes.data, 5, off.ctypes.data,
                                              adj.ctypes.data) == capi.DFX_ERR_INVALID
    assert capi.lib().dfx_mesh_dual_graph_tet(0, None, 0, off.ctypes.data, None) == capi.DFX_OK
    assert off[0] == 0


def _random_graph(n, deg, seed, components=1):
    """A symmetric graph without self-loops or repeated edges, adjacency in
    random order, in `components` parts: many equal degrees, so the RCM tie
    order is exercised."""
    rng = np.random.default_rng(seed)
    part = n // components
    src, dst = [], []
    for c in range(components):
        lo, hi = c * part, (c + 1) * part if c < components - 1 else n
        m = (hi - lo) * deg // 2
        a = rng.integers(lo, hi, m)
        b = rng.integers(lo, hi, m)
        keep = a != b
        src.append(a[keep])
        dst.append(b[keep])
    a, b = np.concatenate(src), np.concatenate(dst)
    e = np.unique(np.stack([np.minimum(a, b), np.maximum(a, b)], 1), axis=0)
    u = np.concatenate([e[:, 0], e[:, 1]])
    v = np.concatenate([e[:, 1], e[:, 0]])
    order = rng.permutation(u.size)
    u, v = u[order], v[order]
    idx = np.argsort(u, kind="stable")
    off = np.zeros(n + 1, np.int32)
    np.add.at(off, u + 1, 1)
    return np.cumsum(off).astype(np.int32), v[idx].astype(np.int32)


@pytest.mark.parametrize("case", ["box", "random", "random_parts", "small"])
def test_rcm_matches_reference(capi, oracle, case):
    """The threaded RCM against the reference's own compiled graph::reorder_rcm
    (and the oracle when the reference was not built): graphs large enough for
    the level-synchronous team, with many degree ties and several components."""
    from dolfinx_gb300 import graph, mesh

    if case == "box":
        off, adj = mesh.create_box(((0, 0, 0), (1, 1, 1)), (26, 22, 20), reorder=False).dual_graph()
    elif case == "random":
        off, adj = _random_graph(120000, 4, 7)
    elif case == "random_parts":
        off, adj = _random_graph(90000, 3, 8, components=5)
    else:
        off, adj = _random_graph(50, 3, 9, components=3)
    perm = graph.reorder_rcm(off, adj)
    n = off.size - 1
    assert np.array_equal(np.sort(perm), np.arange(n))
    R = oracle.ref()
    if R is not None:
        ref = np.empty(n, np.int32)
        R.ref_reorder_rcm(n, off, np.ascontiguousarray(adj, np.int32), ref)
    else:
        ref = oracle.reorder_rcm(off, adj)
    np.testing.assert_array_equal(perm, ref)


def test_rcm_rejects_bad_graphs(capi):
    from dolfinx_gb300 import graph

    with pytest.raises(capi.DfxError, match="outside the graph"):
        graph.reorder_rcm(np.array([0, 1, 2]), np.array([1, 5]))
    with pytest.raises(capi.DfxError, match="must not decrease"):
        graph.reorder_rcm(np.array([0, 2, 1, 2]), np.array([1, 2]))
    assert graph.reorder_rcm(np.array([0]), np.zeros(0)).size == 0


def test_a_plain_c_host_uses_the_abi(capi, tmp_path):
    """tests/c_host_example.c, compiled as C11 against include/dfx_gpu.h and
    linked to libdfxgpu.so, runs the host set-up through the C ABI."""
    import os
    import shutil
    import subprocess

    from dolfinx_gb300 import fem, mesh

    cc = shutil.which("gcc")
    if cc is None:
        pytest.skip("no C compiler")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    libdir = os.path.dirname(capi.LIB_PATH)
    exe = str(tmp_path / "c_host")
    subprocess.run([cc, "-std=c11", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I",
                    os.path.join(root, "include"), os.path.join(root, "tests", "c_host_example.c"),
                    "-o", exe, "-L", libdir, "-ldfxgpu", f"-Wl,-rpath,{libdir}"], check=True,
                   capture_output=True, timeout=120)
    out = subprocess.run([exe], check=True, capture_output=True, text=True, timeout=120).stdout
    V = fem.functionspace(mesh.create_unit_cube(4, 4, 4), ("Lagrange", 2), device="cpu")
    rp, cols = V.sparsity()
    assert out.split() == ["abi", "1", "cells", "384", "nodes", str(V.num_nodes), "nnz",
                           str(cols.size), "facets", "192", "interior", "672",
                           "mesh_reps", "1"]


def test_the_cpp_mirror_header_on_the_host(capi, tmp_path):
    """include/dolfinx_gb300.hpp (the C++ face of the library) compiles with
    -pedantic -Werror into tests/cpp_host_example.cpp; the host set-up,
    timings and error path run and agree with the Python path. The binary
    runs with no visible GPU, where device work must raise, not fall back."""
    import os
    import shutil
    import subprocess

    from dolfinx_gb300 import fem, mesh

    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    libdir = os.path.dirname(capi.LIB_PATH)
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    exe = str(tmp_path / "cpp_host")
    subprocess.run([cxx, "-std=c++20", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I",
                    os.path.join(root, "include"), "-I", os.path.join(cuda, "include"),
                    os.path.join(root, "tests", "cpp_host_example.cpp"), "-o", exe, "-L", libdir,
                    "-ldfxgpu", f"-Wl,-rpath,{libdir}", "-L", os.path.join(cuda, "lib64"),
                    "-lcudart", f"-Wl,-rpath,{os.path.join(cuda, 'lib64')}"],
                   check=True, capture_output=True, timeout=300)
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    out = subprocess.run([exe], check=True, capture_output=True, text=True, timeout=120,
                         env=env).stdout
    got = dict(line.split(" ", 1) for line in out.strip().splitlines())
    m = mesh.create_unit_cube(4, 4, 4)
    V = fem.functionspace(m, ("Lagrange", 2), device="cpu")
    rp, cols = V.sparsity()
    off, adj = m.dual_graph()
    assert got["cells"] == str(m.num_cells) and got["vertices"] == str(m.num_nodes)
    assert got["nodes"] == str(V.num_nodes) and got["nnz"] == str(cols.size)
    assert got["dual_edges"] == str(adj.size) and got["rcm"] == str(m.num_cells)
    assert got["coords"] == str(3 * V.num_nodes) and got["facets"] == "192"
    assert got["interior_facets"] == str(m.interior_facets().shape[0]) == "672"
    assert got["timer_reps"] == "1" and got["mesh_reps"] == "1" and got["table_has_title"] == "1"
    assert got["error"] == f"{capi.DFX_ERR_INVALID} At least one cell is required."
    assert got["device"] == f"none {capi.DFX_ERR_CUDA}"


def test_ctypes_signatures_match_the_header(capi):
    """Every function declared in include/dfx_gpu.h has a ctypes binding
    with as many arguments as its prototype (a mismatch would shift the
    arguments of a call silently)."""
    import os
    import re

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    h = open(os.path.join(root, "include", "dfx_gpu.h")).read()
    h = re.sub(r"/\*.*?\*/", "", h, flags=re.S)
    protos = {}
    for m in re.finditer(r"\b(?:int|size_t|int64_t|const char\*)\s+(dfx_[a-z0-9_]+)\s*"
                         r"\(([^;{]*?)\)\s*;", h, flags=re.S):
        args = m.group(2).strip()
        protos[m.group(1)] = 0 if args in ("", "void") else args.count(",") + 1
    assert set(protos) == set(capi.declared_symbols())
    assert set(protos) == set(capi._SIGS)
    for name, (res, args) in capi._SIGS.items():
        assert len(args) == protos[name], name
    # and each parameter's type: scalars exactly, pointers as pointers (to
    # the same scalar where ctypes names it), library handles as void*
    scalar = {"int32_t": C.c_int32, "int64_t": C.c_int64, "double": C.c_double,
              "size_t": C.c_size_t, "float": C.c_float, "int": C.c_int}
    for m in re.finditer(r"\b(?:int|size_t|int64_t|const char\*)\s+(dfx_[a-z0-9_]+)\s*"
                         r"\(([^;{]*?)\)\s*;", h, flags=re.S):
        name, params = m.group(1), m.group(2).strip()
        if params in ("", "void"):
            continue
        for p, t in zip((" ".join(a.split()) for a in params.split(",")), capi._SIGS[name][1]):
            base = p.replace("const ", "").split("*")[0].split()[0]
            if "**" in p:
                ok = getattr(t, "_type_", None) is C.c_void_p
            elif "*" in p:
                ok = t in (C.c_void_p, C.c_char_p) or (
                    hasattr(t, "_type_") and scalar.get(base, t._type_) is t._type_)
            elif base in ("dfx_operator", "dfx_batch"):
                ok = t is C.c_void_p
            else:
                ok = scalar.get(base) is t
            assert ok, (name, p, t)
    rets = {"int": C.c_int, "size_t": C.c_size_t, "int64_t": C.c_int64, "const char*": C.c_char_p}
    for m in re.finditer(r"\b(int|size_t|int64_t|const char\*)\s+(dfx_[a-z0-9_]+)\s*\(", h):
        assert capi._SIGS[m.group(2)][0] is rets[m.group(1)], m.group(2)


# ctypes structure of the binding -> (C struct name, C field names in order)
_STRUCTS = {
    "Form": ("dfx_form", ["kind", "degree", "num_cells", "num_nodes", "x_dofmap", "x", "dofmap",
                          "kappa", "kappa_const", "k2", "nu", "f", "f_const"]),
    "Csr": ("dfx_csr", ["nrows", "ncols", "bs", "dtype", "nnz", "row_ptr", "cols", "vals"]),
    "CgInfo": ("dfx_cg_info", ["iterations", "status", "rnorm0_sq", "rnorm_sq",
                               "kernel_launches"]),
    "IrInfo": ("dfx_ir_info", ["outer_iterations", "inner_iterations", "status", "reserved",
                               "rnorm0_sq", "rnorm_sq", "kernel_launches"]),
    "BatchSystem": ("dfx_batch_system", ["op32", "op64", "b", "x", "dinv", "work", "rtol",
                                         "delta", "max_iters", "mode"]),
    "Q4Mesh": ("dfx_q4_mesh", ["nx", "ny", "nz", "verts", "kappa", "edges32", "geom32",
                               "geom64"]),
}


def test_ctypes_structures_match_the_c_layout(capi, tmp_path):
    """Each ctypes Structure of the binding has the size and field offsets
    that a C compiler gives the struct of include/dfx_gpu.h (the kernels
    read these structs by value or pointer)."""
    import os
    import shutil
    import subprocess

    cc = shutil.which("gcc")
    if cc is None:
        pytest.skip("no C compiler")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    lines = ['#include "dfx_gpu.h"', "#include <stddef.h>", "#include <stdio.h>",
             "int main(void) {"]
    for py, (cs, fields) in _STRUCTS.items():
        lines.append(f'  printf("{py} size %zu\\n", sizeof({cs}));')
        for f in fields:
            lines.append(f'  printf("{py} {f} %zu\\n", offsetof({cs}, {f}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = str(tmp_path / "layout")
    subprocess.run([cc, "-std=c11", "-I", os.path.join(root, "include"), str(src), "-o", exe],
                   check=True, capture_output=True, timeout=120)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l.strip()}
    for py, (cs, fields) in _STRUCTS.items():
        T = getattr(capi, py)
        assert [f[0] for f in T._fields_] == fields, py
        assert C.sizeof(T) == got[(py, "size")], py
        for f in fields:
            assert getattr(T, f).offset == got[(py, f)], (py, f)


def test_compute_integration_domains(capi, oracle):
    """fem.compute_integration_domains: flat int32 entities per integral
    type, with the reference's IntegralType values."""
    from dolfinx_gb300 import fem, mesh

    m = mesh.create_unit_cube(3, 2, 2)
    T = fem.IntegralType
    assert [T.cell, T.exterior_facet, T.interior_facet, T.vertex, T.ridge] == list(range(5))
    cells = fem.compute_integration_domains(T.cell, m)
    assert cells.dtype == np.int32
    np.testing.assert_array_equal(cells, np.arange(m.num_cells))
    np.testing.assert_array_equal(fem.compute_integration_domains(T.cell, m, [2, 5, 7]),
                                  [2, 5, 7])
    ext = fem.compute_integration_domains(T.exterior_facet, m)
    np.testing.assert_array_equal(ext, oracle.exterior_facets(m.cells).ravel())
    inner = fem.compute_integration_domains(2, m)
    assert inner.dtype == np.int32 and inner.ndim == 1
    np.testing.assert_array_equal(inner, oracle.interior_facets(m.cells).ravel())
    with pytest.raises(ValueError, match="cell indices must lie"):
        fem.compute_integration_domains(T.cell, m, [m.num_cells])
    with pytest.raises(ValueError, match="take no entities"):
        fem.compute_integration_domains(T.interior_facet, m, [0])
    with pytest.raises(ValueError, match="ridge integration domains are not supported"):
        fem.compute_integration_domains(T.ridge, m)
