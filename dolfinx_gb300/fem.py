"""Finite-element front end mirroring ``dolfinx.fem`` for the GPU hot path.

Names, argument meaning and accumulate semantics follow the reference's
Python layer (python/dolfinx/fem/assemble.py:111-493,
python/dolfinx/fem/bcs.py) and C++ assemblers (cpp/dolfinx/fem/assembler.h).
The bilinear/linear forms are the built-in element kernels of libdfxgpu
(Poisson/Helmholtz, linear elasticity, sources) in place of UFL + FFCx.
"""

from __future__ import annotations

import ctypes as C
import enum
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _capi
from .la import MatrixCSR, _check_vec, _ptr, _stream
from .mesh import Mesh


class FunctionSpace:
    """Lagrange P1/P2 space (scalar or vector, bs 3) on a tetrahedral mesh."""

    def __init__(self, mesh: Mesh, degree: int, bs: int = 1, device="cuda"):
        self.mesh, self.degree, self.bs = mesh, int(degree), int(bs)
        self.device = device
        self._dofmap_dev = None
        nd = 4 if degree == 1 else 10
        built = False
        if torch.device(device).type == "cuda" and mesh.num_cells > 0:
            # the numbering on the device (bit-identical to the host builder)
            built = self._dofmap_on_device(nd)
        if not built:
            self.dofmap = np.empty((mesh.num_cells, nd), np.int32)
            n = C.c_int32(0)
            _capi.check(_capi.lib().dfx_dofmap_create_tet(mesh.num_cells,
                                                          mesh.cells.ctypes.data, self.degree,
                                                          self.dofmap.ctypes.data, C.byref(n)))
            self.num_nodes = int(n.value)
        self._sparsity = None
        self._sparsity_dev = None
        self._colouring = None

    def _dofmap_on_device(self, nd: int) -> bool:
        """dfx_dofmap_create_tet_device; False when its edge table overflows
        (the host builder then applies)."""
        m = self.mesh
        cells, _ = m.device(self.device)
        L = _capi.lib()
        wb = int(L.dfx_dofmap_device_workspace_bytes(m.num_cells, m.num_nodes, self.degree))
        work = torch.empty(wb, dtype=torch.uint8, device=self.device)
        dm = torch.empty((m.num_cells, nd), dtype=torch.int32, device=self.device)
        n = C.c_int32(0)
        rc = L.dfx_dofmap_create_tet_device(m.num_cells, _ptr(cells), m.num_nodes, self.degree,
                                            _ptr(dm), C.byref(n), _ptr(work), wb, _stream())
        if rc == _capi.DFX_ERR_UNSUPPORTED:
            return False
        _capi.check(rc)
        self.num_nodes = int(n.value)
        self._dofmap_dev = dm
        self.dofmap = dm.cpu().numpy()
        return True

    @property
    def num_dofs(self) -> int:
        """Scalar dofs (nodes x bs)."""
        return self.num_nodes * self.bs

    @property
    def ndofs_cell(self) -> int:
        return self.dofmap.shape[1]

    def dofmap_device(self) -> torch.Tensor:
        if self._dofmap_dev is None:
            self._dofmap_dev = torch.from_numpy(self.dofmap).to(self.device)
        return self._dofmap_dev

    def tabulate_dof_coordinates(self) -> np.ndarray:
        """Coordinates of the dof nodes (vertices, then edge midpoints), one
        row per node: FunctionSpace::tabulate_dof_coordinates
        (fem/FunctionSpace.h:218-330), computed on host threads."""
        X = np.zeros((self.num_nodes, 3))
        m = self.mesh
        cells = np.ascontiguousarray(m.cells, np.int32)
        x = np.ascontiguousarray(m.x, np.float64)
        dm = np.ascontiguousarray(self.dofmap, np.int32)
        _capi.check(_capi.lib().dfx_tabulate_dof_coordinates_tet(
            m.num_cells, cells.ctypes.data, x.shape[0], x.ctypes.data, dm.ctypes.data,
            self.degree, self.num_nodes, X.ctypes.data))
        return X

    def sparsity(self):
        """(row_ptr, cols) of the cell sparsity pattern on the host (cached)."""
        if self._sparsity is None:
            nd = self.ndofs_cell
            rp = np.empty(self.num_nodes + 1, np.int64)
            nnz = C.c_int64(0)
            L = _capi.lib()
            _capi.check(L.dfx_sparsity_create(self.num_nodes, self.mesh.num_cells, nd,
                                              self.dofmap.ctypes.data, rp.ctypes.data, None,
                                              C.byref(nnz)))
            cols = np.empty(nnz.value, np.int32)
            _capi.check(L.dfx_sparsity_create(self.num_nodes, self.mesh.num_cells, nd,
                                              self.dofmap.ctypes.data, rp.ctypes.data,
                                              cols.ctypes.data, C.byref(nnz)))
            self._sparsity = (rp, cols)
        return self._sparsity

    def sparsity_with_interior_facets(self, facets: np.ndarray):
        """(row_ptr, cols) on the host of the pattern of a form with cell and
        interior-facet integrals: every cell's dofs coupled with each other,
        and every interior facet's macro element -- the dofs of both its
        cells -- coupled with each other (sparsitybuild::cells and
        sparsitybuild::interior_facets, fem/sparsitybuild.h:36-75), the union
        sorted without repeats."""
        facets = np.asarray(facets, np.int32).reshape(-1, 4)
        nd = self.ndofs_cell
        # Cells as macro elements of their own dofs twice (repeats are
        # dropped), then the facets' macro elements.
        macro = np.concatenate([np.concatenate([self.dofmap, self.dofmap], axis=1),
                                np.concatenate([self.dofmap[facets[:, 0]],
                                                self.dofmap[facets[:, 2]]], axis=1)])
        macro = np.ascontiguousarray(macro, np.int32)
        ne = macro.shape[0]
        rp = np.empty(self.num_nodes + 1, np.int64)
        nnz = C.c_int64(0)
        L = _capi.lib()
        _capi.check(L.dfx_sparsity_create(self.num_nodes, ne, 2 * nd, macro.ctypes.data,
                                          rp.ctypes.data, None, C.byref(nnz)))
        cols = np.empty(nnz.value, np.int32)
        _capi.check(L.dfx_sparsity_create(self.num_nodes, ne, 2 * nd, macro.ctypes.data,
                                          rp.ctypes.data, cols.ctypes.data, C.byref(nnz)))
        return rp, cols

    def sparsity_device(self):
        """(row_ptr, cols) of the same pattern as device tensors, built on the
        device from the device dofmap (cached). Equal to ``sparsity()`` bit
        for bit; used by ``create_matrix`` for spaces on a GPU."""
        if self._sparsity_dev is None:
            nd, nc, n = self.ndofs_cell, self.mesh.num_cells, self.num_nodes
            L = _capi.lib()
            dm = self.dofmap_device()
            wb = int(L.dfx_sparsity_device_workspace_bytes(n, nc, nd))
            work = torch.empty(wb, dtype=torch.uint8, device=self.device)
            rp = torch.empty(n + 1, dtype=torch.int64, device=self.device)
            nnz = C.c_int64(0)
            _capi.check(L.dfx_sparsity_create_device(n, nc, nd, _ptr(dm), _ptr(rp), None,
                                                     C.byref(nnz), _ptr(work), wb, _stream()))
            cols = torch.empty(nnz.value, dtype=torch.int32, device=self.device)
            _capi.check(L.dfx_sparsity_create_device(n, nc, nd, _ptr(dm), _ptr(rp), _ptr(cols),
                                                     C.byref(nnz), _ptr(work), wb, _stream()))
            self._sparsity_dev = (rp, cols)
        return self._sparsity_dev

    def colouring(self, max_colours: int = 256):
        """Cell colouring for deterministic assembly: (order on device, offsets)."""
        if self._colouring is None:
            nc = self.mesh.num_cells
            order = np.empty(nc, np.int32)
            offsets = np.zeros(max_colours + 1, np.int32)
            ncol = C.c_int32(0)
            _capi.check(_capi.lib().dfx_colour_cells(nc, self.ndofs_cell, self.dofmap.ctypes.data,
                                                     self.num_nodes, order.ctypes.data,
                                                     offsets.ctypes.data, max_colours,
                                                     C.byref(ncol)))
            off = offsets[: ncol.value + 1].copy()
            self._colouring = (torch.from_numpy(order).to(self.device), off)
        return self._colouring


def functionspace(mesh: Mesh, element, device="cuda") -> FunctionSpace:
    """``functionspace(mesh, ("Lagrange", k))`` or ``("Lagrange", k, (3,))``."""
    family, degree = element[0], int(element[1])
    if family not in ("Lagrange", "P", "CG"):
        raise ValueError(f"element family {family} is not on the GPU hot path")
    bs = 1
    if len(element) > 2 and element[2]:
        bs = int(np.prod(element[2]))
    return FunctionSpace(mesh, degree, bs, device)


def locate_dofs_geometrical(V: FunctionSpace, marker) -> np.ndarray:
    """Node (block) indices whose coordinates satisfy ``marker(x)`` (x: (3, n))."""
    X = V.tabulate_dof_coordinates()
    return np.flatnonzero(marker(X.T)).astype(np.int32)


# Local dofs in the closure of local facet f (the triangle opposite vertex
# f): its three vertices, then (P2) its three edges in Basix edge order.
_FACET_CLOSURE = np.array([[1, 2, 3, 4, 5, 6], [0, 2, 3, 4, 7, 8], [0, 1, 3, 5, 7, 9],
                           [0, 1, 2, 6, 8, 9]], np.int32)


class IntegralType(enum.IntEnum):
    """Integral types with the reference's values (fem/Form.h:39-46)."""

    cell = 0
    exterior_facet = 1
    interior_facet = 2
    vertex = 3
    ridge = 4


def compute_integration_domains(integral_type: IntegralType, mesh: Mesh,
                                entities: np.ndarray | None = None) -> np.ndarray:
    """Flat int32 integration entities (fem/utils.cpp:153-275) of one rank:
    cell indices for ``cell``; (cell, local facet) pairs for
    ``exterior_facet``; (cell0, local facet0, cell1, local facet1) for
    ``interior_facet``. The meshes here number no facets, so facet
    domains cover every exterior or interior facet, sorted by cell; for
    cells, ``entities`` (sorted cell indices) selects a subset. Vertex and
    ridge domains are not supported."""
    integral_type = IntegralType(integral_type)
    if integral_type in (IntegralType.vertex, IntegralType.ridge):
        raise ValueError(f"{integral_type.name} integration domains are not supported")
    if integral_type == IntegralType.cell:
        if entities is None:
            return np.arange(mesh.num_cells, dtype=np.int32)
        cells = np.asarray(entities, np.int32).ravel()
        if cells.size and (cells.min() < 0 or cells.max() >= mesh.num_cells):
            raise ValueError(f"cell indices must lie in [0, {mesh.num_cells})")
        return cells.copy()
    if entities is not None:
        raise ValueError("facet domains take no entities: the mesh numbers no facets")
    if integral_type == IntegralType.exterior_facet:
        return mesh.exterior_facets().ravel().copy()
    return mesh.interior_facets().ravel().copy()


def locate_dofs_facets(V: FunctionSpace, facets: np.ndarray) -> np.ndarray:
    """Sorted node (block) indices in the closure of the given (cell, local
    facet) pairs. With ``V.mesh.exterior_facets()`` these are the boundary
    dofs that ``locate_dofs_topological(V, 2, exterior_facet_indices(...))``
    gives (fem/DirichletBC.cpp, mesh/utils.cpp:61-89)."""
    facets = np.asarray(facets, np.int32).reshape(-1, 2)
    local = _FACET_CLOSURE[:, : (6 if V.degree == 2 else 3)]
    dofs = V.dofmap[facets[:, :1], local[facets[:, 1]]]
    return np.unique(dofs).astype(np.int32)


class DirichletBC:
    """Dirichlet condition u = g on the given dof nodes (fem/DirichletBC.h)."""

    def __init__(self, value, dofs, V: FunctionSpace):
        self.V = V
        dofs = np.asarray(dofs).ravel()
        if dofs.size and (dofs.min() < 0 or dofs.max() >= V.num_nodes):
            # checked here: the device kernels must never see an index
            # outside the space
            raise ValueError(f"Dirichlet dofs must lie in [0, {V.num_nodes}) "
                             f"(got {dofs.min()}..{dofs.max()})")
        dofs = np.unique(dofs.astype(np.int32))
        bs = V.bs
        # _dofs0 unrolled by block size (fem/DirichletBC.h:357-359).
        self.dofs = (dofs[:, None] * bs + np.arange(bs, dtype=np.int32)[None, :]).ravel()
        self.dofs = self.dofs.astype(np.int32)
        n = V.num_dofs
        dev = V.device
        if np.isscalar(value):
            self.g_const = float(value)
            self.g = None
        else:
            val = np.asarray(value, np.float64)
            if val.size == bs:  # constant per component
                g = np.zeros(n)
                g[self.dofs] = val[self.dofs % bs]
                self.g = torch.from_numpy(g).to(dev)
            else:
                if val.size != n:
                    raise ValueError("BC value must be a constant or a full dof vector")
                self.g = torch.from_numpy(val.copy()).to(dev)
            self.g_const = 0.0
        self.dofs_dev = torch.from_numpy(self.dofs).to(dev)

    def g_full(self) -> torch.Tensor:
        if self.g is None:
            self.g = torch.full((self.V.num_dofs,), self.g_const, dtype=torch.float64,
                                device=self.V.device)
        return self.g

    def mark_dofs(self, markers: torch.Tensor) -> None:
        markers[self.dofs_dev.long()] = 1

    def set(self, x: torch.Tensor, x0: torch.Tensor | None = None, alpha: float = 1.0) -> None:
        n, dev = self.V.num_dofs, self.dofs_dev.device
        _check_vec(x, n, torch.float64, dev, "x")
        if x0 is not None:
            _check_vec(x0, n, torch.float64, dev, "x0")
        _capi.check(_capi.lib().dfx_set_bc(_ptr(x), x.numel(), _ptr(self.dofs_dev),
                                           int(self.dofs.size), _ptr(self.g), self.g_const,
                                           _ptr(x0), float(alpha), _stream()))


def dirichletbc(value, dofs, V: FunctionSpace) -> DirichletBC:
    return DirichletBC(value, dofs, V)


@dataclass
class Form:
    """A built-in form on a function space: a cell integral, or an
    exterior-facet integral when ``facets`` holds its (cell, local facet)
    domain on the device."""

    kind: int
    V: FunctionSpace
    kappa: torch.Tensor | None = None  # per-cell coefficient (kappa, E or alpha)
    kappa_const: float = 1.0
    k2: float = 0.0
    nu: float = 0.3
    f: torch.Tensor | None = None  # P1 source values on the geometry nodes
    f_const: tuple = (0.0, 0.0, 0.0)
    # (num_facets, 2) int32 exterior-facet pairs, or (num_facets, 4) interior-facet quads
    facets: torch.Tensor | None = None
    _cache: dict = field(default_factory=dict, repr=False)

    @property
    def rank(self) -> int:
        return 2 if self.kind in (_capi.FORM_POISSON, _capi.FORM_ELASTICITY,
                                  _capi.FORM_FACET_MASS, _capi.FORM_FACET_JUMP) else 1

    @property
    def interior(self) -> bool:
        """An interior-facet integral (dS)."""
        return self.facets is not None and self.facets.shape[1] == 4

    def __add__(self, other):
        return FormSum([self]) + other

    def cstruct(self) -> _capi.Form:
        V = self.V
        xd, x = V.mesh.device(V.device)
        fc = (C.c_double * 3)(*[float(v) for v in self.f_const])
        return _capi.Form(self.kind, V.degree, V.mesh.num_cells, V.mesh.num_nodes,
                          xd.data_ptr(), x.data_ptr(), V.dofmap_device().data_ptr(),
                          None if self.kappa is None else self.kappa.data_ptr(),
                          float(self.kappa_const), float(self.k2), float(self.nu),
                          None if self.f is None else self.f.data_ptr(), fc)


class FormSum:
    """Terms of one form on one space, e.g. a cell integral plus an
    exterior-facet integral (a form with dx and ds parts): assembled into
    one tensor, cell terms first."""

    def __init__(self, terms):
        self.terms = list(terms)
        self.V = self.terms[0].V
        if not all(t.V is self.V for t in self.terms):
            raise ValueError("terms on different spaces")
        if len({t.rank for t in self.terms}) != 1:
            raise ValueError("terms of different rank")

    @property
    def rank(self) -> int:
        return self.terms[0].rank

    def __add__(self, other):
        more = other.terms if isinstance(other, FormSum) else [other]
        return FormSum(self.terms + more)


def _terms(a):
    return a.terms if isinstance(a, FormSum) else [a]


def _dev(v, V, n: int, name: str):
    """A coefficient on the device: None for a constant, else n float64
    values (per cell or per geometry node; the kernels index all n)."""
    if v is None or np.isscalar(v):
        return None
    t = torch.as_tensor(np.asarray(v, np.float64)) if not torch.is_tensor(v) else v
    if t.numel() != n:
        raise ValueError(f"{name} must be a constant or {n} values (got {t.numel()})")
    return t.to(device=V.device, dtype=torch.float64).contiguous().reshape(-1)


def poisson_form(V: FunctionSpace, kappa=1.0, k2: float = 0.0) -> Form:
    """a(u,v) = int kappa grad u.grad v + k2 u v dx; kappa constant or per cell."""
    return Form(_capi.FORM_POISSON, V, kappa=_dev(kappa, V, V.mesh.num_cells, "kappa (per cell)"),
                kappa_const=float(kappa) if np.isscalar(kappa) else 1.0, k2=float(k2))


def _require_vector_p2(V: FunctionSpace) -> None:
    if V.bs != 3 or V.degree != 2:
        raise ValueError("this form needs a vector P2 space (block size 3)")


def _require_scalar(V: FunctionSpace) -> None:
    if V.bs != 1:
        raise ValueError("facet forms need a scalar space")


def elasticity_form(V: FunctionSpace, E=1.0, nu: float = 0.3) -> Form:
    """a(u,v) = int sigma(u):eps(v) dx, E constant or per cell."""
    _require_vector_p2(V)
    return Form(_capi.FORM_ELASTICITY, V, kappa=_dev(E, V, V.mesh.num_cells, "E (per cell)"),
                kappa_const=float(E) if np.isscalar(E) else 1.0, nu=float(nu))


def source_form(V: FunctionSpace, f=1.0) -> Form:
    """L(v) = int f v dx, f constant or P1 values on the geometry nodes."""
    return Form(_capi.FORM_SOURCE, V, f=_dev(f, V, V.mesh.num_nodes, "f (per geometry node)"),
                f_const=(float(f) if np.isscalar(f) else 0.0, 0.0, 0.0))


def _facets(V: FunctionSpace, facets):
    if facets is None:
        facets = V.mesh.exterior_facets()
    t = torch.as_tensor(np.asarray(facets)) if not torch.is_tensor(facets) else facets
    t = t.reshape(-1, 2) if t.numel() else t.reshape(0, 2)
    if t.numel():
        # (cell, local facet) pairs index the mesh in the kernels: checked here
        lo, hi = t.min(0).values.tolist(), t.max(0).values.tolist()
        if lo[0] < 0 or hi[0] >= V.mesh.num_cells or lo[1] < 0 or hi[1] > 3:
            raise ValueError(f"facets must be (cell < {V.mesh.num_cells}, local facet < 4) "
                             "pairs")
    return t.to(device=V.device, dtype=torch.int32).contiguous()


def _interior_facets(V: FunctionSpace, facets):
    if facets is None:
        facets = V.mesh.interior_facets()
    t = torch.as_tensor(np.asarray(facets)) if not torch.is_tensor(facets) else facets
    t = t.reshape(-1, 4) if t.numel() else t.reshape(0, 4)
    if t.numel():
        # quads index the mesh in the kernels: checked here
        lo, hi = t.min(0).values.tolist(), t.max(0).values.tolist()
        if (min(lo[0], lo[2]) < 0 or max(hi[0], hi[2]) >= V.mesh.num_cells
                or min(lo[1], lo[3]) < 0 or max(hi[1], hi[3]) > 3):
            raise ValueError(f"interior facets must be (cell < {V.mesh.num_cells}, local facet "
                             "< 4, cell, local facet) quads")
    return t.to(device=V.device, dtype=torch.int32).contiguous()


def interior_facet_source_form(V: FunctionSpace, g=1.0, facets=None) -> Form:
    """L(v) = int_F avg(g) avg(v) dS over interior facets (all of them by
    default); g constant or P1 values on the geometry nodes."""
    _require_scalar(V)
    return Form(_capi.FORM_SOURCE, V, f=_dev(g, V, V.mesh.num_nodes, "g (per geometry node)"),
                f_const=(float(g) if np.isscalar(g) else 0.0, 0.0, 0.0),
                facets=_interior_facets(V, facets))


def interior_penalty_form(V: FunctionSpace, gamma=1.0, facets=None) -> Form:
    """a(u,v) = int_F gamma |F| [grad u . n][grad v . n] dS over interior
    facets: the continuous interior penalty (gradient-jump) term, with
    gamma constant or per cell (averaged over the facet's two cells) and
    |F| the facet's area. Its matrix needs the facet couplings in the
    pattern: create_matrix builds them for forms with such a term."""
    _require_scalar(V)
    return Form(_capi.FORM_FACET_JUMP, V, kappa=_dev(gamma, V, V.mesh.num_cells,
                                                     "gamma (per cell)"),
                kappa_const=float(gamma) if np.isscalar(gamma) else 1.0,
                facets=_interior_facets(V, facets))


def facet_source_form(V: FunctionSpace, g=1.0, facets=None) -> Form:
    """L(v) = int_F g v ds over exterior facets (all boundary facets by
    default); g constant or P1 values on the geometry nodes."""
    _require_scalar(V)
    return Form(_capi.FORM_SOURCE, V, f=_dev(g, V, V.mesh.num_nodes, "g (per geometry node)"),
                f_const=(float(g) if np.isscalar(g) else 0.0, 0.0, 0.0),
                facets=_facets(V, facets))


def facet_mass_form(V: FunctionSpace, alpha=1.0, facets=None) -> Form:
    """a(u,v) = int_F alpha u v ds over exterior facets (a Robin term);
    alpha constant or per cell (the cell of each facet)."""
    _require_scalar(V)
    return Form(_capi.FORM_FACET_MASS, V, kappa=_dev(alpha, V, V.mesh.num_cells, "alpha (per cell)"),
                kappa_const=float(alpha) if np.isscalar(alpha) else 1.0,
                facets=_facets(V, facets))


def body_force_form(V: FunctionSpace, f=(0.0, 0.0, -1.0)) -> Form:
    _require_vector_p2(V)
    return Form(_capi.FORM_BODYFORCE, V, f_const=tuple(float(v) for v in f))


def _mode(mode: str) -> int:
    return {"atomic": _capi.MODE_ATOMIC, "coloured": _capi.MODE_COLOURED,
            "colored": _capi.MODE_COLOURED}[mode]


def _colour_args(V: FunctionSpace, mode: int):
    if mode != _capi.MODE_COLOURED:
        return None, None, 0
    order, off = V.colouring()
    return C.c_void_p(order.data_ptr()), off.ctypes.data_as(C.c_void_p), int(off.size - 1)


def create_matrix(a) -> MatrixCSR:
    """Matrix with the form's sparsity pattern, values zero (create_matrix).
    The pattern is built on the device for spaces on a GPU; a space whose
    rows exceed the device builder's limit uses the host builder. A form
    with an interior-facet term adds its facets' macro-element couplings
    (host builder)."""
    dev = a.V.device
    bs = a.V.bs
    rp = cols = None
    quads = [t.facets for t in _terms(a) if t.interior]
    if quads:
        rph, colsh = a.V.sparsity_with_interior_facets(
            np.concatenate([q.cpu().numpy() for q in quads]))
        rp, cols = torch.from_numpy(rph).to(dev), torch.from_numpy(colsh).to(dev)
    elif torch.device(dev).type == "cuda":
        try:
            rp, cols = a.V.sparsity_device()
        except _capi.DfxError as e:
            if e.code != _capi.DFX_ERR_UNSUPPORTED:
                raise
    if rp is None:
        rph, colsh = a.V.sparsity()
        rp, cols = torch.from_numpy(rph).to(dev), torch.from_numpy(colsh).to(dev)
    vals = torch.zeros(cols.numel() * bs * bs, dtype=torch.float64, device=dev)
    return MatrixCSR(rp, cols, vals, bs)


def bc_markers(V: FunctionSpace, bcs) -> torch.Tensor | None:
    if not bcs:
        return None
    m = torch.zeros(V.num_dofs, dtype=torch.int8, device=V.device)
    for bc in bcs:
        bc.mark_dofs(m)
    return m


class MatrixAssembler:
    """Reusable matrix assembly for one form (or a sum of cell and
    exterior-facet terms): the cell->slot map, BC markers and colouring are
    computed once (serving-style reuse). Facet terms scatter with FP64
    atomics in either mode."""

    def __init__(self, a, bcs=(), diagonal: float = 1.0, mode: str = "atomic",
                 A: MatrixCSR | None = None, use_slot_map: bool = True):
        self.a, self.bcs, self.diagonal, self.mode = a, list(bcs), float(diagonal), _mode(mode)
        self.terms = _terms(a)
        V = self.terms[0].V
        if A is not None:
            if A.nrows != V.num_nodes or A.ncols != V.num_nodes or A.bs != V.bs:
                raise ValueError(f"A is {A.nrows}x{A.ncols} blocks of {A.bs}; the space needs "
                                 f"{V.num_nodes}x{V.num_nodes} blocks of {V.bs}")
            if A.vals.dtype != torch.float64 or A.vals.device.type != "cuda":
                raise ValueError("A must hold float64 values on a CUDA device")
        self.A = create_matrix(a) if A is None else A
        self.forms = [t.cstruct() for t in self.terms]
        cells = [cs for t, cs in zip(self.terms, self.forms) if t.facets is None]
        # The slot map depends only on the dofmap and the pattern: a facet-only
        # form builds it through a cell form of the same space.
        self.form = cells[0] if cells else Form(_capi.FORM_POISSON, V).cstruct()
        self.markers = bc_markers(V, self.bcs)
        self.map = None
        if use_slot_map:
            nb = int(_capi.lib().dfx_slot_map_bytes(C.byref(self.form)))
            self.map = torch.empty(nb, dtype=torch.uint8, device=V.device)
            _capi.check(_capi.lib().dfx_slot_map_create(C.byref(self.form), C.byref(self.A.csr()),
                                                        _ptr(self.map), _stream()))
        self.colour = _colour_args(V, self.mode)
        bc_dofs = [bc.dofs for bc in self.bcs if bc.V is V]
        self.diag_dofs = (torch.from_numpy(np.unique(np.concatenate(bc_dofs))).to(V.device)
                          if bc_dofs else None)

    def assemble(self, zero: bool = True) -> MatrixCSR:
        if zero:
            self.A.vals.zero_()
        order, off, ncol = self.colour
        L = _capi.lib()
        for t, cs in zip(self.terms, self.forms):
            if t.facets is None:
                _capi.check(L.dfx_assemble_matrix(C.byref(cs), C.byref(self.A.csr()),
                                                  _ptr(self.map), _ptr(self.markers), self.mode,
                                                  order, off, ncol, _stream()))
            elif t.interior:
                _capi.check(L.dfx_assemble_matrix_interior_facets(
                    C.byref(cs), _ptr(t.facets), int(t.facets.shape[0]), C.byref(self.A.csr()),
                    _ptr(self.markers), _stream()))
            else:
                _capi.check(L.dfx_assemble_matrix_facets(C.byref(cs), _ptr(t.facets),
                                                         int(t.facets.shape[0]),
                                                         C.byref(self.A.csr()), _ptr(self.map),
                                                         _ptr(self.markers), _stream()))
        if self.diag_dofs is not None:
            _capi.check(L.dfx_set_diagonal(C.byref(self.A.csr()), _ptr(self.diag_dofs),
                                           int(self.diag_dofs.numel()), self.diagonal,
                                           _stream()))
        return self.A


def assemble_matrix(a: Form, bcs=(), diagonal: float = 1.0, mode: str = "atomic",
                    use_slot_map: bool = True) -> MatrixCSR:
    """Assemble a bilinear form into a new MatrixCSR; constrained rows and
    columns are zeroed and `diagonal` placed on constrained diagonal entries
    (python/dolfinx/fem/assemble.py:282-372)."""
    return MatrixAssembler(a, bcs, diagonal, mode, use_slot_map=use_slot_map).assemble(zero=True)


def assemble_vector(L, b: torch.Tensor | None = None, mode: str = "atomic") -> torch.Tensor:
    """b += assembled linear form (a new zero vector when b is None); cell
    and exterior-facet terms. Facet terms scatter with FP64 atomics."""
    V = L.V
    if b is None:
        b = torch.zeros(V.num_dofs, dtype=torch.float64, device=V.device)
    _check_vec(b, V.num_dofs, torch.float64, V.dofmap_device().device, "b")
    m = _mode(mode)
    for t in _terms(L):
        cf = t.cstruct()
        if t.facets is None:
            order, off, ncol = _colour_args(V, m)
            _capi.check(_capi.lib().dfx_assemble_vector(C.byref(cf), _ptr(b), m, order, off, ncol,
                                                        _stream()))
        elif t.interior:
            _capi.check(_capi.lib().dfx_assemble_vector_interior_facets(
                C.byref(cf), _ptr(t.facets), int(t.facets.shape[0]), _ptr(b), _stream()))
        else:
            _capi.check(_capi.lib().dfx_assemble_vector_facets(C.byref(cf), _ptr(t.facets),
                                                               int(t.facets.shape[0]), _ptr(b),
                                                               _stream()))
    return b


@dataclass
class Functional:
    """M = a(u, u) for a Poisson/Helmholtz form, or M = L(u) for a source
    form: a rank-0 form for ``assemble_scalar``."""

    form: Form
    u: torch.Tensor


def functional(form: Form, u: torch.Tensor) -> Functional:
    return Functional(form, u)


def assemble_scalar(M: Functional) -> float:
    """fem::assemble_scalar over the cells (cpp/dolfinx/fem/assembler.h:173-215,
    cpp/dolfinx/fem/assemble_scalar_impl.h:32-61), summed in a fixed order."""
    f = M.form
    if f.facets is not None:
        raise ValueError("functionals are cell integrals")
    _check_vec(M.u, f.V.num_dofs, torch.float64, f.V.dofmap_device().device, "u")
    L = _capi.lib()
    nc = f.V.mesh.num_cells
    wb = int(L.dfx_assemble_scalar_workspace_bytes(nc))
    work = torch.empty(max(wb, 8), dtype=torch.uint8, device=f.V.device)
    v = C.c_double(0.0)
    cs = f.cstruct()
    _capi.check(L.dfx_assemble_scalar(C.byref(cs), _ptr(M.u), C.byref(v), _ptr(work), wb,
                                      _stream()))
    return v.value


def apply_lifting(b: torch.Tensor, a, bcs, x0=None, alpha: float = 1.0,
                  mode: str = "atomic") -> None:
    """b -= alpha * A (g - x0) restricted to constrained columns, for each
    form a[j] with boundary conditions bcs[j]."""
    m = _mode(mode)
    x0 = x0 or [None] * len(a)
    for aj, bcj, x0j in zip(a, bcs, x0):
        if aj is None or not bcj:
            continue
        V = aj.V
        dev = V.dofmap_device().device
        _check_vec(b, V.num_dofs, torch.float64, dev, "b")
        if x0j is not None:
            _check_vec(x0j, V.num_dofs, torch.float64, dev, "x0")
        markers = bc_markers(V, bcj)
        g = torch.zeros(V.num_dofs, dtype=torch.float64, device=V.device)
        for bc in bcj:
            bc.set(g)
        order, off, ncol = _colour_args(V, m)
        for t in _terms(aj):
            cf = t.cstruct()
            if t.facets is not None:
                # lift_bc over the facet domain (exterior mass or interior penalty)
                _capi.check(_capi.lib().dfx_apply_lifting_facets(
                    C.byref(cf), _ptr(t.facets), int(t.facets.shape[0]), int(t.interior),
                    _ptr(b), _ptr(markers), _ptr(g), _ptr(x0j), float(alpha), _stream()))
                continue
            _capi.check(_capi.lib().dfx_apply_lifting(C.byref(cf), _ptr(b), _ptr(markers),
                                                      _ptr(g), _ptr(x0j), float(alpha), m, order,
                                                      off, ncol, _stream()))


def set_bc(b: torch.Tensor, bcs, x0: torch.Tensor | None = None, alpha: float = 1.0) -> None:
    for bc in bcs:
        bc.set(b, x0, alpha)


class RhsAssembler:
    """Reusable right-hand side: b = assemble_vector(L); apply_lifting(b, [a],
    [bcs]); set_bc(b, bcs) -- the canonical sequence of
    python/test/unit/fem/test_fem_pipeline.py:91-98 -- with the BC markers,
    BC values and colouring prepared once."""

    def __init__(self, L: Form, a: Form | None, bcs=(), mode: str = "atomic"):
        self.L, self.a, self.bcs, self.mode = L, a, list(bcs), _mode(mode)
        V = L.V
        self.Lc = L.cstruct()
        self.ac = a.cstruct() if a is not None else None
        self.markers = bc_markers(V, self.bcs)
        self.g = torch.zeros(V.num_dofs, dtype=torch.float64, device=V.device)
        for bc in self.bcs:
            bc.set(self.g)
        self.colour = _colour_args(V, self.mode)

    def assemble(self, b: torch.Tensor | None = None) -> torch.Tensor:
        V = self.L.V
        if b is None:
            b = torch.zeros(V.num_dofs, dtype=torch.float64, device=V.device)
        else:
            _check_vec(b, V.num_dofs, torch.float64, V.dofmap_device().device, "b")
            b.zero_()
        order, off, ncol = self.colour
        L = _capi.lib()
        _capi.check(L.dfx_assemble_vector(C.byref(self.Lc), _ptr(b), self.mode, order, off, ncol,
                                          _stream()))
        if self.ac is not None and self.bcs:
            _capi.check(L.dfx_apply_lifting(C.byref(self.ac), _ptr(b), _ptr(self.markers),
                                            _ptr(self.g), None, 1.0, self.mode, order, off, ncol,
                                            _stream()))
        for bc in self.bcs:
            bc.set(b)
        return b
