"""Randomised parity of the threaded host set-up: seeded box shapes (odd and
lopsided, some large enough for every thread team), RCM order on or off, and
1 to 8 host threads, so chunk and level boundaries fall in different places.
Each build is compared with the oracle (mesh, dual graph, P1/P2 dofmaps,
exterior facets) and with the reference's compiled RCM where it was built."""

import os

import numpy as np
import pytest


def _shapes():
    rng = np.random.default_rng(2024)
    out = [tuple(int(v) for v in rng.integers(1, 9, 3)) for _ in range(8)]
    out += [(41, 7, 23), (5, 61, 19), (29, 31, 17)]  # 40K-100K cells: threaded paths
    return out


@pytest.fixture
def threads_env():
    old = os.environ.get("DFX_NUM_THREADS")
    yield
    if old is None:
        os.environ.pop("DFX_NUM_THREADS", None)
    else:
        os.environ["DFX_NUM_THREADS"] = old


@pytest.mark.parametrize("i,n", list(enumerate(_shapes())))
def test_random_box_matches_oracle(capi, oracle, threads_env, i, n):
    from dolfinx_gb300 import fem, graph, mesh

    threads = (1, 2, 3, 5, 8)[i % 5]
    reorder = i % 3 != 2
    os.environ["DFX_NUM_THREADS"] = str(threads)
    p1 = (1.0 + 0.25 * i, 1.0, 0.5 + 0.1 * i)
    m = mesh.create_box(((0.0, 0.0, 0.0), p1), n, reorder=reorder)
    cells, x = oracle.create_box_tet(*n, p1=p1, reorder=reorder)
    np.testing.assert_array_equal(m.cells, cells)
    np.testing.assert_array_equal(m.x, x)
    off, adj = m.dual_graph()
    off0, adj0 = oracle.dual_graph_tet(m.cells.astype(np.int64))
    np.testing.assert_array_equal(off, off0)
    np.testing.assert_array_equal(adj, adj0)
    perm = graph.reorder_rcm(off, adj)
    R = oracle.ref()
    if R is not None:
        ref = np.empty(off.size - 1, np.int32)
        R.ref_reorder_rcm(off.size - 1, off, adj, ref)
    else:
        ref = oracle.reorder_rcm(off, adj)
    np.testing.assert_array_equal(perm, ref)
    for deg in (1, 2):
        V = fem.functionspace(m, ("Lagrange", deg), device="cpu")
        dm, nn = oracle.dofmap_tet(m.cells, deg)
        assert V.num_nodes == nn
        np.testing.assert_array_equal(V.dofmap, dm)
    np.testing.assert_array_equal(m.exterior_facets(), oracle.exterior_facets(m.cells))
    np.testing.assert_array_equal(m.interior_facets(), oracle.interior_facets(m.cells))
