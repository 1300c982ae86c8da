"""Graph tools of the host set-up, mirroring ``dolfinx.graph``: the reverse
Cuthill-McKee ordering that ``mesh.create_box`` applies to the facet dual
graph (graph::reorder_rcm, cpp/dolfinx/graph/ordering.cpp:148-170)."""

from __future__ import annotations

import numpy as np

from . import _capi


def reorder_rcm(offsets: np.ndarray, adjacency: np.ndarray) -> np.ndarray:
    """The reverse Cuthill-McKee permutation of a graph given as (offsets,
    adjacency): perm[old] = new. Roots and degree ties follow the
    reference's George-Liu search and sort order exactly."""
    off = np.ascontiguousarray(offsets, np.int32)
    adj = np.ascontiguousarray(adjacency, np.int32)
    n = off.size - 1
    if n < 0 or adj.size < off[-1]:
        raise ValueError("offsets must have n+1 entries and adjacency offsets[-1]")
    perm = np.empty(max(n, 1), np.int32)
    _capi.check(_capi.lib().dfx_graph_reorder_rcm(n, off.ctypes.data, adj.ctypes.data,
                                                  perm.ctypes.data))
    return perm[:n]
