"""Mesh creation, mirroring ``dolfinx.mesh.create_box`` / ``create_unit_cube``
for tetrahedral boxes (cpp/dolfinx/mesh/generation.h:104-134, 380-426).

The cells are RCM-reordered and the geometry nodes numbered exactly as
DOLFINx does on one rank. The work runs in the host part of libdfxgpu, or
with ``device="cuda"`` on the GPU (the same mesh bit for bit).
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _capi


class CellType:
    tetrahedron = "tetrahedron"


@dataclass
class Mesh:
    """Tetrahedral mesh: ``cells`` (nc, 4) geometry node indices, ``x`` (nv, 3)."""

    cells: np.ndarray
    x: np.ndarray
    _dev: dict = field(default_factory=dict, repr=False)

    @property
    def num_cells(self) -> int:
        return int(self.cells.shape[0])

    @property
    def num_nodes(self) -> int:
        return int(self.x.shape[0])

    def exterior_facets(self) -> np.ndarray:
        """(num_facets, 2) int32 (cell, local facet) pairs of the boundary,
        sorted (mesh::exterior_facet_indices + compute_integration_domains,
        cpp/dolfinx/mesh/utils.cpp:61-89, cpp/dolfinx/fem/utils.h:155-162);
        local facet f is the triangle opposite vertex f. Cached."""
        if "facets" not in self._dev:
            out = np.empty((4 * self.num_cells, 2), np.int32)
            nf = C.c_int32(0)
            _capi.check(_capi.lib().dfx_exterior_facets_tet(self.num_cells, self.cells.ctypes.data,
                                                            out.ctypes.data, C.byref(nf)))
            self._dev["facets"] = out[: nf.value].copy()
        return self._dev["facets"]

    def interior_facets(self) -> np.ndarray:
        """(num_facets, 4) int32 (cell0, local facet0, cell1, local facet1)
        of the facets shared by two cells: the integration domain of an
        interior-facet integral (fem::compute_integration_domains,
        cpp/dolfinx/fem/utils.cpp:223-254). (cell0, facet0) < (cell1,
        facet1) within a row; rows sorted. Cached."""
        if "interior_facets" not in self._dev:
            out = np.empty((2 * self.num_cells, 4), np.int32)
            nf = C.c_int32(0)
            cells = np.ascontiguousarray(self.cells, np.int32)
            _capi.check(_capi.lib().dfx_interior_facets_tet(self.num_cells, cells.ctypes.data,
                                                            out.ctypes.data, C.byref(nf)))
            self._dev["interior_facets"] = out[: nf.value].copy()
        return self._dev["interior_facets"]

    def dual_graph(self, device=None):
        """(offsets, adjacency) int32 of the facet-connected dual graph
        (mesh::build_local_dual_graph, cpp/dolfinx/mesh/graphbuild.cpp:566-905):
        the cells that share a facet with each cell. With a CUDA `device`
        the graph is built there and returned as device tensors."""
        if device is not None and _is_cuda(device):
            return dual_graph_device(self.device(device)[0], self.num_nodes)
        nc = self.num_cells
        off = np.empty(nc + 1, np.int32)
        adj = np.empty(max(4 * nc, 1), np.int32)
        cells = np.ascontiguousarray(self.cells, np.int32)
        _capi.check(_capi.lib().dfx_mesh_dual_graph_tet(nc, cells.ctypes.data, self.num_nodes,
                                                        off.ctypes.data, adj.ctypes.data))
        return off, adj[: off[-1]].copy()

    def device(self, device="cuda"):
        """(x_dofmap, x) as device tensors (cached)."""
        import torch

        key = str(device)
        if key not in self._dev:
            self._dev[key] = (torch.from_numpy(self.cells).to(device),
                              torch.from_numpy(self.x).to(device))
        return self._dev[key]


def _is_cuda(device) -> bool:
    import torch

    return torch.device(device).type == "cuda"


def _work(nbytes: int, device):
    import torch

    return torch.empty(max(int(nbytes), 1), dtype=torch.uint8, device=device)


def dual_graph_device(cells, num_vertices: int):
    """Device (offsets, adjacency) int32 tensors of the facet dual graph of
    device cells (num_cells, 4); see Mesh.dual_graph."""
    import torch

    from .la import _ptr, _stream

    nc = int(cells.shape[0])
    cells = cells.contiguous()
    off = torch.empty(nc + 1, dtype=torch.int32, device=cells.device)
    adj = torch.empty(max(4 * nc, 1), dtype=torch.int32, device=cells.device)
    L = _capi.lib()
    wb = int(L.dfx_mesh_dual_graph_tet_device_workspace_bytes(nc, int(num_vertices)))
    work = _work(wb, cells.device)
    _capi.check(L.dfx_mesh_dual_graph_tet_device(nc, _ptr(cells), int(num_vertices), _ptr(off),
                                                 _ptr(adj), _ptr(work), wb, _stream()))
    return off, adj[: int(off[-1])]


def create_box(points, n, cell_type=CellType.tetrahedron, reorder: bool = True,
               device=None) -> Mesh:
    """device: None or a CPU device builds on host threads; a CUDA device
    builds the same mesh on the GPU (and keeps its device copy)."""
    if cell_type != CellType.tetrahedron:
        raise ValueError("only tetrahedral boxes are on the GPU hot path")
    nx, ny, nz = (int(v) for v in n)
    p0 = np.ascontiguousarray(points[0], np.float64)
    p1 = np.ascontiguousarray(points[1], np.float64)
    nc = 6 * nx * ny * nz
    nv = (nx + 1) * (ny + 1) * (nz + 1)
    if device is not None and _is_cuda(device):
        return _create_box_device(nx, ny, nz, p0, p1, reorder, device)
    cells = np.empty((nc, 4), np.int32)
    x = np.empty((nv, 3), np.float64)
    _capi.check(_capi.lib().dfx_mesh_create_box_tet(nx, ny, nz, p0.ctypes.data, p1.ctypes.data,
                                                    int(reorder), cells.ctypes.data, x.ctypes.data))
    return Mesh(cells, x)


def _create_box_device(nx, ny, nz, p0, p1, reorder, device) -> Mesh:
    import torch

    from .la import _ptr, _stream

    if min(nx, ny, nz) < 1:
        raise _capi.DfxError(_capi.DFX_ERR_INVALID, "At least one cell is required.")
    L = _capi.lib()
    wb = int(L.dfx_mesh_create_box_tet_device_workspace_bytes(nx, ny, nz, int(reorder)))
    if wb == 0:
        raise _capi.DfxError(_capi.DFX_ERR_INVALID, "mesh too large for int32 cell indices")
    nc = 6 * nx * ny * nz
    nv = (nx + 1) * (ny + 1) * (nz + 1)
    cells = torch.empty((nc, 4), dtype=torch.int32, device=device)
    x = torch.empty((nv, 3), dtype=torch.float64, device=device)
    work = _work(wb, device)
    _capi.check(L.dfx_mesh_create_box_tet_device(nx, ny, nz, p0.ctypes.data, p1.ctypes.data,
                                                 int(reorder), _ptr(cells), _ptr(x), _ptr(work),
                                                 wb, _stream()))
    del work
    m = Mesh(cells.cpu().numpy(), x.cpu().numpy())
    m._dev[str(device)] = (cells, x)
    return m


def create_unit_cube(nx, ny, nz, cell_type=CellType.tetrahedron, reorder: bool = True,
                     device=None) -> Mesh:
    return create_box(((0.0, 0.0, 0.0), (1.0, 1.0, 1.0)), (nx, ny, nz), cell_type, reorder,
                      device)
