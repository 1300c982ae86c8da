"""Device-side mesh set-up against the host builders and the oracle: the box
mesh, its facet dual graph and the reverse Cuthill-McKee ordering built on
the GPU must equal the host ones bit for bit (mesh/generation.h:332-426,
mesh/graphbuild.cpp:566-905, graph/ordering.cpp:22-170)."""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _same_doubles(a, b):
    a = np.ascontiguousarray(a, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    return a.shape == b.shape and np.array_equal(a.view(np.int64), b.view(np.int64))


@pytest.mark.parametrize("reorder", [True, False])
@pytest.mark.parametrize("n", [(1, 1, 1), (2, 3, 4), (5, 3, 7), (12, 12, 12), (16, 9, 5)])
def test_box_device_equals_host(cuda, capi, n, reorder):
    from dolfinx_gb300 import mesh

    pts = ((-1.0, 0.5, 2.0), (3.0, 1.75, 2.3))
    h = mesh.create_box(pts, n, reorder=reorder)
    d = mesh.create_box(pts, n, reorder=reorder, device="cuda")
    np.testing.assert_array_equal(d.cells, h.cells)
    assert _same_doubles(d.x, h.x)
    dc, dx = d.device("cuda")
    np.testing.assert_array_equal(dc.cpu().numpy(), h.cells)


def test_box_device_equals_oracle_c2_size(cuda, capi, oracle):
    """The 64^3 x 6 unit cube of the P2 Poisson benchmark (1,572,864 cells):
    device mesh = host mesh = the oracle's restatement of the reference."""
    from dolfinx_gb300 import mesh

    d = mesh.create_unit_cube(64, 64, 64, device="cuda")
    h = mesh.create_unit_cube(64, 64, 64)
    np.testing.assert_array_equal(d.cells, h.cells)
    assert _same_doubles(d.x, h.x)
    cells, x = oracle.create_box_tet(64, 64, 64)
    np.testing.assert_array_equal(d.cells, cells.reshape(-1, 4))
    np.testing.assert_allclose(d.x, x.reshape(-1, 3), rtol=0, atol=0)


def _shuffled_mesh(n, seed):
    """A box mesh with its cells shuffled and its vertices relabelled: a
    conforming tetrahedral mesh in no particular order."""
    from dolfinx_gb300 import mesh

    m = mesh.create_unit_cube(*n, reorder=False)
    rng = np.random.default_rng(seed)
    relabel = rng.permutation(m.num_nodes).astype(np.int32)
    cells = relabel[m.cells][rng.permutation(m.num_cells)]
    return np.ascontiguousarray(cells, np.int32), m.num_nodes


@pytest.mark.parametrize("n,seed", [((1, 1, 1), 0), ((3, 4, 5), 1), ((10, 7, 6), 2),
                                    ((20, 20, 20), 3)])
def test_dual_graph_device_equals_host(cuda, capi, n, seed):
    from dolfinx_gb300 import mesh

    cells, nv = _shuffled_mesh(n, seed)
    m = mesh.Mesh(cells, np.zeros((nv, 3)))
    off_h, adj_h = m.dual_graph()
    off_d, adj_d = m.dual_graph(device="cuda")
    np.testing.assert_array_equal(off_d.cpu().numpy(), off_h)
    np.testing.assert_array_equal(adj_d.cpu().numpy(), adj_h)


def test_dual_graph_device_refuses_a_facet_of_three_cells(cuda, capi):
    """Three cells on one facet: the host lists all pairs, the device
    reports it cannot (UNSUPPORTED) instead of returning another graph."""
    from dolfinx_gb300 import mesh

    cells = np.array([[0, 1, 2, 3], [0, 1, 2, 4], [0, 1, 2, 5]], np.int32)
    m = mesh.Mesh(cells, np.zeros((6, 3)))
    off_h, adj_h = m.dual_graph()
    assert off_h.tolist() == [0, 2, 4, 6]
    with pytest.raises(capi.DfxError) as e:
        m.dual_graph(device="cuda")
    assert e.value.code == capi.DFX_ERR_UNSUPPORTED


def _random_graph(n, max_deg, seed, components=1):
    """A symmetric graph without self-loops, node degrees at most max_deg,
    in `components` disconnected parts (plus isolated nodes)."""
    rng = np.random.default_rng(seed)
    nbrs = [[] for _ in range(n)]
    part = rng.integers(0, components, n)
    for _ in range(n * max_deg // 3):
        a, b = rng.integers(0, n, 2)
        if a == b or part[a] != part[b] or b in nbrs[a]:
            continue
        if len(nbrs[a]) >= max_deg or len(nbrs[b]) >= max_deg:
            continue
        nbrs[a].append(int(b))
        nbrs[b].append(int(a))
    off = np.zeros(n + 1, np.int32)
    off[1:] = np.cumsum([len(v) for v in nbrs])
    adj = np.array([u for v in nbrs for u in v], np.int32)
    return off, adj


@pytest.mark.parametrize("n,deg,seed,parts", [(1, 4, 0, 1), (50, 4, 1, 1), (2000, 6, 2, 3),
                                              (30000, 16, 3, 2), (100000, 8, 4, 1)])
def test_rcm_device_equals_host_random_graphs(cuda, capi, n, deg, seed, parts):
    from dolfinx_gb300 import graph

    off, adj = _random_graph(n, deg, seed, parts)
    p_h = graph.reorder_rcm(off, adj)
    p_d = graph.reorder_rcm(torch.from_numpy(off).cuda(), torch.from_numpy(adj).cuda())
    np.testing.assert_array_equal(p_d.cpu().numpy(), p_h)
    assert np.array_equal(np.sort(p_h), np.arange(n))


@pytest.mark.parametrize("n", [(4, 4, 4), (24, 17, 9)])
def test_rcm_device_equals_host_dual_graphs(cuda, capi, n):
    """The ordering create_box applies: the dual graph of the unordered box."""
    from dolfinx_gb300 import graph, mesh

    m = mesh.create_unit_cube(*n, reorder=False)
    off, adj = m.dual_graph()
    p_h = graph.reorder_rcm(off, adj)
    off_d, adj_d = m.dual_graph(device="cuda")
    p_d = graph.reorder_rcm(off_d, adj_d)
    np.testing.assert_array_equal(p_d.cpu().numpy(), p_h)


def test_rcm_device_refusals(cuda, capi):
    from dolfinx_gb300 import graph

    # a node of degree 17: the degree sort of more than 16 children is not restated
    n = 18
    nb = [list(range(1, 18))] + [[0] for _ in range(17)]
    off = np.zeros(n + 1, np.int32)
    off[1:] = np.cumsum([len(v) for v in nb])
    adj = np.array([u for v in nb for u in v], np.int32)
    with pytest.raises(capi.DfxError) as e:
        graph.reorder_rcm(torch.from_numpy(off).cuda(), torch.from_numpy(adj).cuda())
    assert e.value.code == capi.DFX_ERR_UNSUPPORTED
    # an edge that points outside the graph
    off = np.array([0, 1, 2], np.int32)
    adj = np.array([1, 5], np.int32)
    with pytest.raises(capi.DfxError) as e:
        graph.reorder_rcm(torch.from_numpy(off).cuda(), torch.from_numpy(adj).cuda())
    assert e.value.code == capi.DFX_ERR_INVALID


def test_function_space_on_device_mesh(cuda, capi):
    """A device mesh feeds the device dofmap without a host round trip of
    its cells; the dofmap equals the host mesh's."""
    from dolfinx_gb300 import fem, mesh

    d = mesh.create_unit_cube(9, 7, 8, device="cuda")
    h = mesh.create_unit_cube(9, 7, 8)
    Vd = fem.functionspace(d, ("Lagrange", 2))
    Vh = fem.functionspace(h, ("Lagrange", 2), device="cpu")
    np.testing.assert_array_equal(Vd.dofmap, Vh.dofmap)
    assert Vd.num_dofs == Vh.num_dofs
