"""Matrix-free Q4 Poisson operator and its CG, mirroring the matrix-free
demo (cpp/demo/poisson_matrix_free/main.cpp: the action lambda 201-222 and
the CG of 84-132; the form M = action(a, u) in poisson.py:33-46) on a
structured hexahedral mesh of the unit cube with Lagrange Q4 and
Gauss-Legendre 5^3 quadrature.

The element action is applied by sum factorisation in libdfxgpu (one CTA
per cell, 8 colours of cells that share no node). Nodes are the
Gauss-Lobatto-Legendre points of each cell, numbered lexicographically on
the (4n+1)^3 lattice; the boundary rows are the identity (homogeneous
Dirichlet on the whole boundary, the BC rows of the demo's action).
"""

from __future__ import annotations

import ctypes as C
import numpy as np
import torch

from . import _capi
from .la import CGResult, _check_vec, _ptr, _stream


def hex_box_vertices(nx: int, ny: int | None = None, nz: int | None = None,
                     perturb: float = 0.05, seed: int = 0) -> np.ndarray:
    """Vertices ((nx+1)(ny+1)(nz+1), 3) of a structured hex mesh of the unit
    cube, x fastest. Interior vertices move by U(-perturb h, +perturb h) per
    coordinate (h the cell size in that direction) from a seeded generator;
    boundary vertices stay, so the domain stays the unit cube."""
    ny = nx if ny is None else ny
    nz = nx if nz is None else nz
    z, y, x = np.meshgrid(np.linspace(0, 1, nz + 1), np.linspace(0, 1, ny + 1),
                          np.linspace(0, 1, nx + 1), indexing="ij")
    v = np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1)
    if perturb:
        rng = np.random.default_rng(seed)
        noise = rng.uniform(-perturb, perturb, size=v.shape) * np.array([1 / nx, 1 / ny, 1 / nz])
        k, j, i = np.meshgrid(np.arange(nz + 1), np.arange(ny + 1), np.arange(nx + 1),
                              indexing="ij")
        interior = ((i > 0) & (i < nx) & (j > 0) & (j < ny) & (k > 0) & (k < nz)).ravel()
        v[interior] += noise[interior]
    return v


def gll_points() -> np.ndarray:
    """The five Gauss-Lobatto-Legendre points on [0, 1] (the Q4 nodes of a
    cell edge)."""
    s = np.sqrt(3.0 / 7.0)
    return np.array([0.0, 0.5 * (1 - s), 0.5, 0.5 * (1 + s), 1.0])


def node_coordinates(verts, nx: int, ny: int | None = None, nz: int | None = None) -> np.ndarray:
    """Physical coordinates ((4nx+1)(4ny+1)(4nz+1), 3) of the Q4 nodes: the
    GLL points of each cell mapped by the cell's trilinear map (the map of a
    shared face depends only on that face's vertices, so neighbours agree)."""
    ny = nx if ny is None else ny
    nz = nx if nz is None else nz
    V = np.asarray(verts, np.float64).reshape(nz + 1, ny + 1, nx + 1, 3)
    g = gll_points()
    NX, NY, NZ = 4 * nx + 1, 4 * ny + 1, 4 * nz + 1
    # Cell index and local coordinate of every lattice line.
    def split(N, n):
        idx = np.arange(N)
        c = np.minimum(idx // 4, n - 1)
        return c, g[idx - 4 * c]
    ci, X = split(NX, nx)
    cj, Y = split(NY, ny)
    ck, Z = split(NZ, nz)
    out = np.zeros((NZ, NY, NX, 3))
    for v in range(8):
        bx, by, bz = v & 1, (v >> 1) & 1, (v >> 2) & 1
        wx = X if bx else 1 - X
        wy = Y if by else 1 - Y
        wz = Z if bz else 1 - Z
        corner = V[ck[:, None, None] + bz, cj[None, :, None] + by, ci[None, None, :] + bx]
        out += (wz[:, None, None] * wy[None, :, None] * wx[None, None, :])[..., None] * corner
    return out.reshape(-1, 3)


def boundary_mask(nx: int, ny: int, nz: int) -> np.ndarray:
    """True at the Q4 nodes on the boundary of the box (lexicographic)."""
    NX, NY, NZ = 4 * nx + 1, 4 * ny + 1, 4 * nz + 1
    K, J, I = np.meshgrid(np.arange(NZ), np.arange(NY), np.arange(NX), indexing="ij")
    return ((I == 0) | (J == 0) | (K == 0) | (I == NX - 1) | (J == NY - 1)
            | (K == NZ - 1)).ravel()


class Q4Laplacian:
    """y = A u for a(u, v) = int kappa grad u . grad v on Q4 hexahedra, with
    identity rows on the boundary. Vertex coordinates stay resident in HBM."""

    def __init__(self, verts, nx: int, ny: int | None = None, nz: int | None = None,
                 kappa: float = 1.0, device="cuda", cache_edges: bool = True,
                 cache_geometry=(torch.float64,)):
        """cache_edges: keep the cells' FP32 edge vectors in HBM (36 floats
        per cell) for the FP32 action instead of forming them from the FP64
        vertices in every application (same results, bitwise).
        cache_geometry: the precisions (torch.float64, torch.float32) whose
        action reads the geometric factor of every quadrature point from HBM
        (750 values per cell: 6 KB in FP64, 3 KB in FP32) instead of forming
        the Jacobian, its adjugate and determinant at each point; results
        agree to rounding. FP64 only by default: at 64^3 cells the FP64
        action took 6.56 ms against 10.07 ms (FP64-pipe bound), while the
        FP32 action took 0.411 ms with the cache against 0.394 ms without
        (its extra 786 MB cost more than the instructions it saves)."""
        ny = nx if ny is None else ny
        nz = nx if nz is None else nz
        v = torch.as_tensor(np.ascontiguousarray(verts, np.float64))
        if v.shape != ((nx + 1) * (ny + 1) * (nz + 1), 3):
            raise ValueError(f"verts must be ({(nx + 1) * (ny + 1) * (nz + 1)}, 3), "
                             f"got {tuple(v.shape)}")
        self.verts = v.to(device)
        self.dims = (nx, ny, nz)
        self.kappa = float(kappa)
        self._mesh = _capi.Q4Mesh(nx, ny, nz, self.verts.data_ptr(), self.kappa, None, None,
                                  None)
        self.n = int(_capi.lib().dfx_q4_num_dofs(C.byref(self._mesh)))
        self.edges = None
        if cache_edges:
            self.edges = torch.empty(36 * nx * ny * nz, dtype=torch.float32, device=device)
            _capi.check(_capi.lib().dfx_q4_edges(C.byref(self._mesh), _ptr(self.edges),
                                                 _stream()))
            self._mesh.edges32 = self.edges.data_ptr()
        self.geom = {}
        if cache_geometry is True:
            cache_geometry = (torch.float64, torch.float32)
        for dt, cdt, field in ((torch.float32, _capi.F32, "geom32"),
                               (torch.float64, _capi.F64, "geom64")):
            if cache_geometry and dt in tuple(cache_geometry):
                g = torch.empty(750 * nx * ny * nz, dtype=dt, device=device)
                _capi.check(_capi.lib().dfx_q4_geometry(C.byref(self._mesh), cdt, _ptr(g),
                                                        _stream()))
                self.geom[dt] = g
                setattr(self._mesh, field, g.data_ptr())

    def mesh(self):
        return self._mesh

    def apply(self, u: torch.Tensor, y: torch.Tensor) -> None:
        if u.dtype not in (torch.float64, torch.float32):
            raise TypeError("u must be float64 or float32")
        _check_vec(u, self.n, u.dtype, self.verts.device, "u")
        _check_vec(y, self.n, u.dtype, self.verts.device, "y")
        dt = _capi.F64 if u.dtype == torch.float64 else _capi.F32
        _capi.check(_capi.lib().dfx_q4_action(C.byref(self._mesh), dt, _ptr(u), _ptr(y),
                                              _stream()))

    def apply_tc(self, u: torch.Tensor, y: torch.Tensor) -> None:
        """FP32 action with the basis contractions on the tensor cores
        (tcgen05, TF32 words split hi + lo); same operator as apply()."""
        _check_vec(u, self.n, torch.float32, self.verts.device, "u")
        _check_vec(y, self.n, torch.float32, self.verts.device, "y")
        _capi.check(_capi.lib().dfx_q4_action_tc(C.byref(self._mesh), _ptr(u), _ptr(y),
                                                 _stream()))

    def check_tc(self) -> None:
        """Raises if a tensor-core launch stopped early (its MMA wait ran out)."""
        _capi.check(_capi.lib().dfx_q4_tc_check(_stream()))

    def __call__(self, u: torch.Tensor) -> torch.Tensor:
        y = torch.empty_like(u)
        self.apply(u, y)
        return y


class MatrixFreeCG:
    """CG on the Q4 action (unpreconditioned, as the demo's). mode "fp64":
    FP64 throughout; mode "mixed": FP32 action and vectors with residual
    replacement by the FP64 action whenever |r| has dropped by `delta`;
    mode "mixed_tc": "mixed" with the tensor-core FP32 action."""

    def __init__(self, op: Q4Laplacian, mode: str = "mixed", delta: float = 0.1,
                 graph_iters: int = 20):
        self.op = op
        self.mode = {"fp64": 0, "mixed": 1, "mixed_tc": 2}[mode]
        self.delta = float(delta)
        self.graph_iters = graph_iters
        wb = int(_capi.lib().dfx_q4_cg_workspace_bytes(op.n, self.mode))
        self.work = torch.empty(wb, dtype=torch.uint8, device=op.verts.device)

    def solve(self, b: torch.Tensor, x: torch.Tensor, rtol: float = 1e-10,
              max_iters: int = 100000, raise_on_fail: bool = True) -> CGResult:
        _check_vec(b, self.op.n, torch.float64, self.op.verts.device, "b")
        _check_vec(x, self.op.n, torch.float64, self.op.verts.device, "x")
        info = _capi.CgInfo()
        rc = _capi.lib().dfx_q4_cg_solve(C.byref(self.op.mesh()), _ptr(b), _ptr(x), float(rtol),
                                         int(max_iters), int(self.mode), self.delta,
                                         int(self.graph_iters), _ptr(self.work),
                                         self.work.numel(), C.byref(info), _stream())
        if raise_on_fail:
            _capi.check(rc)
        return CGResult(info.iterations, info.status, info.rnorm0_sq, info.rnorm_sq,
                        info.kernel_launches)
