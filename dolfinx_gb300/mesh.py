"""Mesh creation, mirroring ``dolfinx.mesh.create_box`` / ``create_unit_cube``
for tetrahedral boxes (cpp/dolfinx/mesh/generation.h:104-134, 380-426).

The cells are RCM-reordered and the geometry nodes numbered exactly as
DOLFINx does on one rank; the work runs in the host part of libdfxgpu.
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

    def dual_graph(self) -> tuple[np.ndarray, np.ndarray]:
        """(offsets, adjacency) int32 of the facet-connected dual graph
        (mesh::build_local_dual_graph, cpp/dolfinx/mesh/graphbuild.cpp:566-905):
        the cells that share a facet with each cell."""
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


def create_box(points, n, cell_type=CellType.tetrahedron, reorder: bool = True) -> Mesh:
    if cell_type != CellType.tetrahedron:
        raise ValueError("only tetrahedral boxes are on the GPU hot path")
    nx, ny, nz = (int(v) for v in n)
    p0 = np.ascontiguousarray(points[0], np.float64)
    p1 = np.ascontiguousarray(points[1], np.float64)
    nc = 6 * nx * ny * nz
    nv = (nx + 1) * (ny + 1) * (nz + 1)
    cells = np.empty((nc, 4), np.int32)
    x = np.empty((nv, 3), np.float64)
    _capi.check(_capi.lib().dfx_mesh_create_box_tet(nx, ny, nz, p0.ctypes.data, p1.ctypes.data,
                                                    int(reorder), cells.ctypes.data, x.ctypes.data))
    return Mesh(cells, x)


def create_unit_cube(nx, ny, nz, cell_type=CellType.tetrahedron, reorder: bool = True) -> Mesh:
    return create_box(((0.0, 0.0, 0.0), (1.0, 1.0, 1.0)), (nx, ny, nz), cell_type, reorder)
