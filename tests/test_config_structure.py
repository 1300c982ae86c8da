"""Structure parity at the benchmark sizes (CPU): the product's host set-up
-- box mesh with RCM cell order, first-appearance dofmap, CSR sparsity --
of the P1 16^3, P2 64^3 and vector-P2 96x24x24 configurations, bit for bit
against the oracle and against the SHA-256 digests that
tests/golden/make_structure_hashes.py recorded from it."""

import hashlib
import json
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                      "config_structure.json")
CONFIGS = {
    "c1_p1_unit_cube_16": ((16, 16, 16), (1.0, 1.0, 1.0), 1),
    "c2_p2_unit_cube_64": ((64, 64, 64), (1.0, 1.0, 1.0), 2),
    "c3_p2_box_96x24x24": ((96, 24, 24), (4.0, 1.0, 1.0), 2),
}


def digest(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def product_structure(n, p1, degree):
    from dolfinx_gb300 import fem, mesh

    m = mesh.create_box(((0.0, 0.0, 0.0), p1), n)
    V = fem.functionspace(m, ("Lagrange", degree), device="cpu")
    rp, cols = V.sparsity()
    return m, V, rp, cols


@pytest.mark.parametrize("name", sorted(CONFIGS))
def test_structure_matches_golden_digests(capi, name):
    ref = json.load(open(GOLDEN))[name]
    m, V, rp, cols = product_structure(*CONFIGS[name])
    assert (m.num_cells, V.num_nodes, int(rp[-1])) == (ref["num_cells"], ref["num_nodes"],
                                                        ref["nnz"])
    assert digest(m.cells.astype(np.int32)) == ref["cells"]
    assert digest(m.x.astype(np.float64)) == ref["x"]
    assert digest(V.dofmap.astype(np.int32)) == ref["dofmap"]
    assert digest(np.asarray(rp, np.int64)) == ref["row_ptr"]
    assert digest(np.asarray(cols, np.int32)) == ref["cols"]


def test_p2_64_structure_matches_oracle(capi, oracle):
    """The headline configuration, array for array against the oracle."""
    m, V, rp, cols = product_structure(*CONFIGS["c2_p2_unit_cube_64"])
    cells, x = oracle.create_box_tet(64, 64, 64)
    np.testing.assert_array_equal(m.cells, cells)
    np.testing.assert_array_equal(m.x, x)
    dm, nn = oracle.dofmap_tet(cells, 2)
    assert V.num_nodes == nn == 2146689
    np.testing.assert_array_equal(V.dofmap, dm)
    rp0, cols0 = oracle.sparsity(nn, dm)
    np.testing.assert_array_equal(rp, rp0)
    np.testing.assert_array_equal(cols, cols0)
    assert rp0[-1] == 60859905
