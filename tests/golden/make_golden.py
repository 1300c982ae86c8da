"""Write the golden vectors of tests/golden/ from the reference's own code.

Runs where the DOLFINx source tree is available: it builds
oracle/_ref/libdfxref.so from the reference's graph/ordering.cpp,
common/sort.h and la/matrix_csr_impl.h, and oracle/_ref/libdfxref_la.so
from its la/SparsityPattern.cpp and common/IndexMap.cpp (oracle/Makefile,
target `ref`), and records their outputs on small seeded inputs. The test-suite then checks
the oracle restatement against these files on any machine.

    python tests/golden/make_golden.py
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402


def main():
    O.build(with_ref=True)
    R = O.ref()
    assert R is not None, "reference pieces did not build"
    out = {}
    # 1. Facet sort of the dual graph (common/sort.h sort_by_perm) and RCM
    #    (graph/ordering.cpp) on raw box meshes.
    for (nx, ny, nz) in [(1, 1, 1), (2, 2, 2), (3, 2, 4), (5, 4, 3)]:
        raw, _ = O.box_tet_raw(nx, ny, nz)
        nc = raw.shape[0]
        fac = np.array([[1, 2, 3], [0, 2, 3], [0, 1, 3], [0, 1, 2]])
        keys = np.sort(raw[:, fac], axis=2).reshape(-1, 3)
        cols = [np.ascontiguousarray(keys[:, k]) for k in range(3)]
        perm = np.empty(4 * nc, np.int32)
        R.ref_sort_by_perm3(4 * nc, cols[0], cols[1], cols[2], perm)
        # Dual graph built from the reference permutation, as
        # mesh/graphbuild.cpp does after its sort.
        edges = []
        i = 0
        while i < perm.size:
            j = i + 1
            while j < perm.size and (keys[perm[j]] == keys[perm[i]]).all():
                j += 1
            for a in range(i, j):
                for b in range(a + 1, j):
                    edges.append((perm[a] // 4, perm[b] // 4))
            i = j
        cnt = np.zeros(nc + 1, np.int32)
        for a, b in edges:
            cnt[a + 1] += 1
            cnt[b + 1] += 1
        off = np.cumsum(cnt).astype(np.int32)
        adj = np.empty(off[-1], np.int32)
        pos = off[:-1].copy()
        for a, b in edges:
            adj[pos[a]] = b
            pos[a] += 1
            adj[pos[b]] = a
            pos[b] += 1
        r = np.empty(nc, np.int32)
        R.ref_reorder_rcm(nc, off, adj, r)
        tag = f"{nx}x{ny}x{nz}"
        out[f"facet_perm_{tag}"] = perm
        out[f"dual_off_{tag}"] = off
        out[f"dual_adj_{tag}"] = adj
        out[f"rcm_{tag}"] = r
    # 2. insert_csr (add) and spmv on a P2 Poisson matrix of a 2x2x2 box
    #    and a vector P2 elasticity matrix of a 2x1x1 box (bs 3).
    for tag, (n, deg, kind) in {"p2": ((2, 2, 2), 2, 0), "el": ((2, 1, 1), 2, 1)}.items():
        cells, x = O.create_box_tet(*n)
        dm, nn = O.dofmap_tet(cells, deg)
        rp, cols = O.sparsity(nn, dm)
        bs = 3 if kind == 1 else 1
        rng = np.random.default_rng(7)
        vals = np.zeros(cols.size * bs * bs)
        for c in range(cells.shape[0]):
            Ae = rng.standard_normal((10 * bs) ** 2)
            rc = R.ref_insert_csr_add(bs, vals, cols.size, cols, rp, nn, Ae, 10, dm[c].copy(), 10,
                                      dm[c].copy())
            assert rc == 0
        xv = rng.standard_normal(nn * bs)
        y = rng.standard_normal(nn * bs)
        y0 = y.copy()
        R.ref_spmv(nn, bs, rp, cols, vals, nn, xv, y)
        out[f"csr_vals_{tag}"] = vals
        out[f"spmv_x_{tag}"] = xv
        out[f"spmv_y0_{tag}"] = y0
        out[f"spmv_y_{tag}"] = y
        out[f"csr_rowptr_{tag}"] = rp
        out[f"csr_cols_{tag}"] = cols
    # 3. The cell sparsity pattern from the reference's own SparsityPattern
    #    (la/SparsityPattern.cpp, one rank) for P1 and P2 dofmaps.
    assert O.ref_la() is not None, "reference sparsity pattern did not build"
    for tag, (n, deg) in {"p1": ((3, 4, 5), 1), "p2": ((4, 3, 2), 2)}.items():
        cells, x = O.create_box_tet(*n)
        dm, nn = O.dofmap_tet(cells, deg)
        rp, cols = O.ref_sparsity(nn, dm)
        out[f"sp_dofmap_{tag}"] = dm
        out[f"sp_rowptr_{tag}"] = rp
        out[f"sp_cols_{tag}"] = cols
    np.savez_compressed(os.path.join(HERE, "reference_golden.npz"), **out)
    print("wrote", len(out), "arrays")


if __name__ == "__main__":
    main()
