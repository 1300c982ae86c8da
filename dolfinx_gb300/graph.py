"""Graph tools of the host set-up, mirroring ``dolfinx.graph``: the reverse
Cuthill-McKee ordering that ``mesh.create_box`` applies to the facet dual
graph (graph::reorder_rcm, cpp/dolfinx/graph/ordering.cpp:148-170)."""

from __future__ import annotations

import numpy as np

from . import _capi


def reorder_rcm(offsets, adjacency):
    """The reverse Cuthill-McKee permutation of a graph given as (offsets,
    adjacency): perm[old] = new. Roots and degree ties follow the
    reference's George-Liu search and sort order exactly. CUDA tensors are
    ordered on the device (nodes of degree at most 16) and give a CUDA
    tensor; arrays are ordered on host threads."""
    try:
        import torch
    except ImportError:  # pragma: no cover
        torch = None
    if torch is not None and isinstance(offsets, torch.Tensor) and offsets.is_cuda:
        return _reorder_rcm_device(offsets, adjacency)
    off = np.ascontiguousarray(offsets, np.int32)
    adj = np.ascontiguousarray(adjacency, np.int32)
    n = off.size - 1
    if n < 0 or adj.size < off[-1]:
        raise ValueError("offsets must have n+1 entries and adjacency offsets[-1]")
    perm = np.empty(max(n, 1), np.int32)
    _capi.check(_capi.lib().dfx_graph_reorder_rcm(n, off.ctypes.data, adj.ctypes.data,
                                                  perm.ctypes.data))
    return perm[:n]


def _reorder_rcm_device(offsets, adjacency):
    import torch

    from .la import _ptr, _stream

    off = offsets.to(torch.int32).contiguous()
    adj = adjacency.to(torch.int32).contiguous()
    n = off.numel() - 1
    if n < 0 or adj.device != off.device:
        raise ValueError("offsets must have n+1 entries and sit with adjacency on one device")
    if n > 0 and int(off[-1]) > adj.numel():
        raise ValueError("adjacency must hold offsets[-1] entries")
    perm = torch.empty(max(n, 1), dtype=torch.int32, device=off.device)
    L = _capi.lib()
    wb = int(L.dfx_graph_reorder_rcm_device_workspace_bytes(n))
    work = torch.empty(max(wb, 1), dtype=torch.uint8, device=off.device)
    _capi.check(L.dfx_graph_reorder_rcm_device(n, _ptr(off), _ptr(adj) if adj.numel() else None,
                                               _ptr(perm), _ptr(work), wb, _stream()))
    return perm[:n]
