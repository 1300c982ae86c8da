"""Write tests/golden/config_structure.json: SHA-256 digests of the mesh,
dofmap and sparsity of the benchmark configurations, computed by the
oracle (the CPU restatement of the reference's box generation, RCM order,
first-appearance dofmap and SparsityPattern, itself pinned to the
reference's compiled ordering and sparsity code by the golden vectors of
make_golden.py). The test-suite checks the product's host and device
set-up against these digests at full size, so a change of numbering is
caught without rerunning the oracle.

    python tests/golden/make_structure_hashes.py
"""

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

# name -> (hexahedra per direction, box upper corner, Lagrange degree)
CONFIGS = {
    "c1_p1_unit_cube_16": ((16, 16, 16), (1.0, 1.0, 1.0), 1),
    "c2_p2_unit_cube_64": ((64, 64, 64), (1.0, 1.0, 1.0), 2),
    "c3_p2_box_96x24x24": ((96, 24, 24), (4.0, 1.0, 1.0), 2),
}


def digest(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def structure(n, p1, degree):
    cells, x = O.create_box_tet(*n, p1=p1)
    dm, nn = O.dofmap_tet(cells, degree)
    rp, cols = O.sparsity(nn, dm)
    return {"cells": digest(cells.astype(np.int32)), "x": digest(x.astype(np.float64)),
            "dofmap": digest(dm.astype(np.int32)), "row_ptr": digest(rp.astype(np.int64)),
            "cols": digest(cols.astype(np.int32)), "num_cells": int(cells.shape[0]),
            "num_nodes": int(nn), "nnz": int(rp[-1])}


def main():
    O.build(with_ref=False)
    out = {name: structure(*cfg) for name, cfg in CONFIGS.items()}
    with open(os.path.join(HERE, "config_structure.json"), "w") as fh:
        json.dump(out, fh, indent=1, sort_keys=True)
        fh.write("\n")
    for name, d in out.items():
        print(name, d["num_cells"], d["num_nodes"], d["nnz"])


if __name__ == "__main__":
    main()
