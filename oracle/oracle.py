"""ctypes front end of the CPU oracle (test infrastructure only).

Loads ``oracle/_build/liboracle.so`` (the CPU restatement of the DOLFINx
hot path, ``oracle/dfx_oracle.cpp``) and, when it was built,
``oracle/_ref/libdfxref.so`` (the reference's own ordering / sort / CSR
code). Only the test-suite, ``__graft_entry__.smoke()`` and the CPU
baseline leg of ``bench.py`` use this module; the product package never
imports it.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
REFLIB = os.path.join(HERE, "_ref", "libdfxref.so")
# The DOLFINx source tree the reference pieces are compiled from; absent on
# hosts that only run the prebuilt oracle.
REF_SRC = os.environ.get("DOLFINX_SOURCE_DIR", "/root/reference")

_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_i8p = np.ctypeslib.ndpointer(np.int8, flags="C_CONTIGUOUS")


def build(with_ref: bool | None = None) -> None:
    """Compile the oracle (and the reference pieces when the tree exists)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    if with_ref is None:
        with_ref = os.path.isdir(os.path.join(REF_SRC, "cpp", "dolfinx"))
    if with_ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={REF_SRC}"], check=True)


class _Form(C.Structure):
    _fields_ = [
        ("kind", C.c_int),
        ("degree", C.c_int),
        ("kappa", C.c_void_p),
        ("k2", C.c_double),
        ("nu", C.c_double),
    ]


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build(with_ref=False)
        L = C.CDLL(LIB)
        L.orc_create_box_tet.argtypes = [C.c_int] * 3 + [_f64p, _f64p, C.c_int, _i32p, _f64p]
        L.orc_box_tet_raw.argtypes = [C.c_int] * 3 + [_f64p, _f64p, _i64p, _f64p]
        L.orc_dual_graph_tet.argtypes = [C.c_int, _i64p, _i32p, _i32p]
        L.orc_reorder_rcm.argtypes = [C.c_int, _i32p, _i32p, _i32p]
        L.orc_dofmap_tet.argtypes = [C.c_int, _i32p, C.c_int, _i32p]
        L.orc_sparsity.argtypes = [C.c_int, C.c_int, C.c_int, _i32p, C.c_void_p, C.c_void_p]
        L.orc_sparsity.restype = C.c_int64
        L.orc_kernel_poisson.argtypes = [C.c_int, _f64p, C.c_double, C.c_double, _f64p]
        L.orc_kernel_source.argtypes = [C.c_int, _f64p, _f64p, _f64p]
        L.orc_kernel_elasticity.argtypes = [_f64p, C.c_double, C.c_double, _f64p]
        L.orc_assemble_matrix.argtypes = [C.POINTER(_Form), C.c_int, _i32p, _f64p, _i32p,
                                          C.c_void_p, _i64p, _i32p, _f64p]
        L.orc_assemble_vector.argtypes = [C.c_int, C.c_int, C.c_int, _i32p, _f64p, _i32p,
                                          C.c_void_p, C.c_void_p, _f64p]
        L.orc_apply_lifting.argtypes = [C.POINTER(_Form), C.c_int, _i32p, _f64p, _i32p, _i8p,
                                        _f64p, C.c_void_p, C.c_double, _f64p]
        L.orc_set_bc.argtypes = [C.c_int, _f64p, C.c_int, _i32p, _f64p, C.c_void_p, C.c_double]
        L.orc_set_diagonal.argtypes = [C.c_int, _i64p, _i32p, _f64p, C.c_int, _i32p, C.c_double]
        L.orc_spmv.argtypes = [C.c_int, C.c_int, _i64p, _i32p, _f64p, _f64p, _f64p]
        L.orc_spmv_f32.argtypes = [C.c_int, C.c_int, _i64p, _i32p, _f32p, _f32p, _f32p]
        L.orc_q4_action.argtypes = [C.c_int] * 3 + [_f64p, C.c_double, _f64p, _f64p, C.c_int]
        L.orc_q4_tables.argtypes = [_f64p, _f64p, _f64p]
        L.orc_cg.argtypes = [C.c_int, C.c_int, _i64p, _i32p, _f64p, _f64p, _f64p, C.c_void_p,
                             C.c_double, C.c_int]
        L.orc_exterior_facets_tet.argtypes = [C.c_int, _i32p, _i32p]
        L.orc_interior_facets_tet.argtypes = [C.c_int, _i32p, _i32p]
        L.orc_assemble_vector_facets.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _f64p, _i32p,
                                                 C.c_void_p, C.c_double, _f64p]
        L.orc_assemble_matrix_facets.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _f64p, _i32p,
                                                 C.c_void_p, C.c_double, C.c_void_p, _i64p,
                                                 _i32p, _f64p]
        L.orc_assemble_scalar.argtypes = [C.c_int, C.c_int, C.c_int, _i32p, _f64p, _i32p,
                                          C.c_void_p, C.c_double, C.c_void_p, _f64p]
        L.orc_assemble_scalar.restype = C.c_double
        L.orc_assemble_matrix_interior_facets.argtypes = [
            C.c_int, C.c_int, _i32p, _i32p, _f64p, _i32p, C.c_void_p, C.c_double, C.c_void_p,
            _i64p, _i32p, _f64p]
        L.orc_colour_cells.argtypes = [C.c_int, C.c_int, _i32p, C.c_int, _i32p, _i32p, C.c_int]
        L.orc_poisson_step_threaded.argtypes = [
            C.POINTER(_Form), C.c_int, _i32p, _f64p, _i32p, C.c_int, _i8p, C.c_int, _i32p,
            C.c_void_p, C.c_void_p, _i64p, _i32p, _f64p, _f64p, _f64p, _i32p, _i32p, C.c_int,
            C.c_double, C.c_int, C.c_int, _f64p]
        _lib = L
    return _lib


def ref():
    """The reference's own compiled code, or None when it was not built."""
    global _ref
    if _ref is None and os.path.exists(REFLIB):
        R = C.CDLL(REFLIB)
        R.ref_reorder_rcm.argtypes = [C.c_int, _i32p, _i32p, _i32p]
        R.ref_sort_by_perm3.argtypes = [C.c_int64, _i64p, _i64p, _i64p, _i32p]
        R.ref_insert_csr_add.argtypes = [C.c_int, _f64p, C.c_int64, _i32p, _i64p, C.c_int64,
                                         _f64p, C.c_int, _i32p, C.c_int, _i32p]
        R.ref_spmv.argtypes = [C.c_int64, C.c_int, _i64p, _i32p, _f64p, C.c_int64, _f64p, _f64p]
        _ref = R
    return _ref


REFLIB_LA = os.path.join(HERE, "_ref", "libdfxref_la.so")
_ref_la = None


def ref_la():
    """The reference's own sparsity-pattern code, or None when not built."""
    global _ref_la
    if _ref_la is None and os.path.exists(REFLIB_LA):
        R = C.CDLL(REFLIB_LA)
        R.ref_sparsity.argtypes = [C.c_int32, C.c_int32, C.c_int32, _i32p, _i64p, C.c_void_p]
        R.ref_sparsity.restype = C.c_int64
        R.ref_timing_record.argtypes = [C.c_char_p, C.c_double]
        R.ref_timing_record.restype = None
        R.ref_timing_table.argtypes = [C.c_int, C.c_char_p, C.c_int64]
        R.ref_timing_table.restype = C.c_int64
        _ref_la = R
    return _ref_la


def ref_sparsity(n, dofmap):
    """(row_ptr, cols) from the reference's SparsityPattern on one rank."""
    R = ref_la()
    dm = np.ascontiguousarray(dofmap, np.int32)
    rp = np.empty(n + 1, np.int64)
    nnz = R.ref_sparsity(n, dm.shape[0], dm.shape[1], dm, rp, None)
    cols = np.empty(nnz, np.int32)
    R.ref_sparsity(n, dm.shape[0], dm.shape[1], dm, rp, cols.ctypes.data)
    return rp, cols


def ref_timing_record(task, seconds):
    """One more repetition of ``seconds`` for ``task`` in the reference's
    TimeLogger (this process's)."""
    ref_la().ref_timing_record(task.encode(), float(seconds))


def ref_timing_table(reduction):
    """The reference's summary table (TimeLogger::timing_table, reduced on
    one rank; reduction 0/1/2 = average/max/min) as a string."""
    R = ref_la()
    n = R.ref_timing_table(reduction, None, 0)
    buf = C.create_string_buffer(n + 1)
    R.ref_timing_table(reduction, buf, n + 1)
    return buf.raw[:n].decode()


def _ptr(a):
    return None if a is None else a.ctypes.data


# ---------------------------------------------------------------- mesh
def create_box_tet(nx, ny, nz, p0=(0.0, 0.0, 0.0), p1=(1.0, 1.0, 1.0), reorder=True):
    nc = 6 * nx * ny * nz
    nv = (nx + 1) * (ny + 1) * (nz + 1)
    cells = np.empty((nc, 4), np.int32)
    x = np.empty((nv, 3), np.float64)
    rc = lib().orc_create_box_tet(nx, ny, nz, np.asarray(p0, np.float64),
                                  np.asarray(p1, np.float64), int(reorder), cells, x)
    assert rc == 0
    return cells, x


def box_tet_raw(nx, ny, nz, p0=(0.0, 0.0, 0.0), p1=(1.0, 1.0, 1.0)):
    nc = 6 * nx * ny * nz
    nv = (nx + 1) * (ny + 1) * (nz + 1)
    cells = np.empty((nc, 4), np.int64)
    x = np.empty((nv, 3), np.float64)
    lib().orc_box_tet_raw(nx, ny, nz, np.asarray(p0, np.float64), np.asarray(p1, np.float64),
                          cells, x)
    return cells, x


def dual_graph_tet(cells64):
    nc = cells64.shape[0]
    off = np.empty(nc + 1, np.int32)
    adj = np.empty(4 * nc, np.int32)
    lib().orc_dual_graph_tet(nc, np.ascontiguousarray(cells64, np.int64), off, adj)
    return off, adj[: off[-1]].copy()


def reorder_rcm(off, adj):
    n = off.size - 1
    r = np.empty(n, np.int32)
    lib().orc_reorder_rcm(n, off, np.ascontiguousarray(adj, np.int32), r)
    return r


def dofmap_tet(cells, degree):
    nc = cells.shape[0]
    nd = 4 if degree == 1 else 10
    dm = np.empty((nc, nd), np.int32)
    n = lib().orc_dofmap_tet(nc, np.ascontiguousarray(cells, np.int32), degree, dm)
    return dm, int(n)


def sparsity(nrows, dofmap):
    nc, nd = dofmap.shape
    dm = np.ascontiguousarray(dofmap, np.int32)
    rp = np.empty(nrows + 1, np.int64)
    nnz = lib().orc_sparsity(nrows, nc, nd, dm, rp.ctypes.data, None)
    cols = np.empty(nnz, np.int32)
    lib().orc_sparsity(nrows, nc, nd, dm, rp.ctypes.data, cols.ctypes.data)
    return rp, cols


# ---------------------------------------------------------------- assembly
def _form(kind, degree, kappa, k2, nu):
    f = _Form(kind, degree, None, float(k2), float(nu))
    if kappa is not None:
        f.kappa = kappa.ctypes.data
    return f


def assemble_matrix(kind, degree, cells, x, dofmap, row_ptr, cols, kappa=None, k2=0.0, nu=0.3,
                    bc_markers=None, vals=None):
    bs = 3 if kind == 1 else 1
    if vals is None:
        vals = np.zeros(cols.size * bs * bs, np.float64)
    kap = None if kappa is None else np.ascontiguousarray(kappa, np.float64)
    f = _form(kind, degree, kap, k2, nu)
    bcm = None if bc_markers is None else np.ascontiguousarray(bc_markers, np.int8)
    rc = lib().orc_assemble_matrix(C.byref(f), cells.shape[0], np.ascontiguousarray(cells), x,
                                   np.ascontiguousarray(dofmap), _ptr(bcm), row_ptr, cols, vals)
    if rc == 3:
        raise RuntimeError("Entry not in sparsity")
    return vals


def assemble_vector(kind, degree, cells, x, dofmap, n, f=None, fvec=None, b=None):
    bs = 3 if kind == 1 else 1
    if b is None:
        b = np.zeros(n * bs, np.float64)
    fa = None if f is None else np.ascontiguousarray(f, np.float64)
    fv = None if fvec is None else np.ascontiguousarray(fvec, np.float64)
    lib().orc_assemble_vector(kind, degree, cells.shape[0], np.ascontiguousarray(cells), x,
                              np.ascontiguousarray(dofmap), _ptr(fa), _ptr(fv), b)
    return b


def apply_lifting(b, kind, degree, cells, x, dofmap, bc_markers, g, kappa=None, k2=0.0, nu=0.3,
                  x0=None, alpha=1.0):
    kap = None if kappa is None else np.ascontiguousarray(kappa, np.float64)
    f = _form(kind, degree, kap, k2, nu)
    x0a = None if x0 is None else np.ascontiguousarray(x0, np.float64)
    lib().orc_apply_lifting(C.byref(f), cells.shape[0], np.ascontiguousarray(cells), x,
                            np.ascontiguousarray(dofmap), np.ascontiguousarray(bc_markers, np.int8),
                            np.ascontiguousarray(g, np.float64), _ptr(x0a), float(alpha), b)
    return b


def set_bc(b, dofs, g, x0=None, alpha=1.0):
    x0a = None if x0 is None else np.ascontiguousarray(x0, np.float64)
    lib().orc_set_bc(b.size, b, dofs.size, np.ascontiguousarray(dofs, np.int32),
                     np.ascontiguousarray(g, np.float64), _ptr(x0a), float(alpha))
    return b


def set_diagonal(bs, row_ptr, cols, vals, dofs, diag=1.0):
    rc = lib().orc_set_diagonal(bs, row_ptr, cols, vals, dofs.size,
                                np.ascontiguousarray(dofs, np.int32), float(diag))
    if rc:
        raise RuntimeError("Entry not in sparsity")
    return vals


def spmv(row_ptr, cols, vals, x, bs=1, y=None):
    nrows = row_ptr.size - 1
    if y is None:
        y = np.zeros(nrows * bs, np.float64)
    lib().orc_spmv(nrows, bs, row_ptr, cols, vals, np.ascontiguousarray(x, np.float64), y)
    return y


def cg(row_ptr, cols, vals, b, bs=1, x=None, dinv=None, rtol=1e-10, kmax=100000):
    nrows = row_ptr.size - 1
    x = np.zeros(nrows * bs) if x is None else np.ascontiguousarray(x, np.float64).copy()
    d = None if dinv is None else np.ascontiguousarray(dinv, np.float64)
    it = lib().orc_cg(nrows, bs, row_ptr, cols, vals, np.ascontiguousarray(b, np.float64), x,
                      _ptr(d), float(rtol), int(kmax))
    return x, int(it)


def kernel_poisson(degree, coords, kappa=1.0, k2=0.0):
    nd = 4 if degree == 1 else 10
    Ae = np.zeros(nd * nd)
    lib().orc_kernel_poisson(degree, Ae, kappa, k2, np.ascontiguousarray(coords, np.float64).ravel())
    return Ae.reshape(nd, nd)


def kernel_elasticity(coords, E=1.0, nu=0.3):
    Ae = np.zeros(900)
    lib().orc_kernel_elasticity(Ae, E, nu, np.ascontiguousarray(coords, np.float64).ravel())
    return Ae.reshape(30, 30)


def q4_action(n, verts, u, kappa=1.0, apply_bc=True):
    """y = A u for the Q4 hex Laplacian on a structured mesh of n^3 cells
    (n an int) or nx x ny x nz cells (n a tuple); see orc_q4_action."""
    nx, ny, nz = (n, n, n) if np.isscalar(n) else n
    u = np.ascontiguousarray(u, np.float64)
    y = np.zeros_like(u)
    lib().orc_q4_action(nx, ny, nz, np.ascontiguousarray(verts, np.float64), float(kappa), u, y,
                        int(apply_bc))
    return y


# ---------------------------------------------------------------- facets, functionals
def exterior_facets(cells):
    """(num_facets, 2) int32 array of (cell, local facet), sorted."""
    cells = np.ascontiguousarray(cells, np.int32)
    out = np.empty((4 * cells.shape[0], 2), np.int32)
    nf = lib().orc_exterior_facets_tet(cells.shape[0], cells, out)
    return out[:nf].copy()


def interior_facets(cells):
    """(num_facets, 4) int32 array of (cell0, local facet0, cell1, local
    facet1), sorted."""
    cells = np.ascontiguousarray(cells, np.int32)
    out = np.empty((max(2 * cells.shape[0], 1), 4), np.int32)
    nf = lib().orc_interior_facets_tet(cells.shape[0], cells, out)
    return out[:nf].copy()


def assemble_vector_facets(degree, facets, cells, x, dofmap, n, g=None, g_const=1.0, b=None):
    r"""b += \int_F g v ds over the given exterior facets (scalar P1/P2)."""
    if b is None:
        b = np.zeros(n, np.float64)
    ga = None if g is None else np.ascontiguousarray(g, np.float64)
    fa = np.ascontiguousarray(facets, np.int32)
    lib().orc_assemble_vector_facets(degree, fa.shape[0], fa, np.ascontiguousarray(cells), x,
                                     np.ascontiguousarray(dofmap), _ptr(ga), float(g_const), b)
    return b


def assemble_matrix_facets(degree, facets, cells, x, dofmap, row_ptr, cols, alpha=None,
                           alpha_const=1.0, bc_markers=None, vals=None):
    r"""vals += \int_F alpha u v ds over the given exterior facets."""
    if vals is None:
        vals = np.zeros(cols.size, np.float64)
    al = None if alpha is None else np.ascontiguousarray(alpha, np.float64)
    bcm = None if bc_markers is None else np.ascontiguousarray(bc_markers, np.int8)
    fa = np.ascontiguousarray(facets, np.int32)
    rc = lib().orc_assemble_matrix_facets(degree, fa.shape[0], fa, np.ascontiguousarray(cells), x,
                                          np.ascontiguousarray(dofmap), _ptr(al),
                                          float(alpha_const), _ptr(bcm), row_ptr, cols, vals)
    if rc == 3:
        raise RuntimeError("Entry not in sparsity")
    return vals


def assemble_scalar(kind, degree, cells, x, dofmap, u, kappa=None, k2=0.0, f=None):
    r"""kind 0: a(u, u) = \int kappa |grad u|^2 + k2 u^2 dx; kind 1: \int f u dx."""
    kap = None if kappa is None else np.ascontiguousarray(kappa, np.float64)
    fa = None if f is None else np.ascontiguousarray(f, np.float64)
    return lib().orc_assemble_scalar(kind, degree, cells.shape[0], np.ascontiguousarray(cells), x,
                                     np.ascontiguousarray(dofmap), _ptr(kap), float(k2), _ptr(fa),
                                     np.ascontiguousarray(u, np.float64))


def colour_cells(dofmap, ndofs, max_colours=256):
    """Greedy first-fit cell colouring in cell order (no two cells of a
    colour share a dof): (order, offsets) of the colour classes."""
    dm = np.ascontiguousarray(dofmap, np.int32)
    order = np.empty(dm.shape[0], np.int32)
    off = np.zeros(max_colours + 1, np.int32)
    k = lib().orc_colour_cells(dm.shape[0], dm.shape[1], dm, int(ndofs), order, off, max_colours)
    if k < 0:
        raise RuntimeError("cell colouring needs more than %d colours" % max_colours)
    return order, off[:k + 1].copy()


def poisson_step_threaded(degree, cells, x, dofmap, ndofs, bc_dofs, row_ptr, cols, colours,
                          kappa=None, f=None, g=None, rtol=1e-10, kmax=100000, threads=1,
                          vals=None, b=None, u=None):
    """One full step of the scalar Poisson workload on host threads (matrix,
    right-hand side with lifting and set_bc, Jacobi-PCG from zero). Returns
    (iterations, seconds[matrix, rhs, solve], vals, b, u)."""
    nc = cells.shape[0]
    kap = None if kappa is None else np.ascontiguousarray(kappa, np.float64)
    form = _form(0, degree, kap, 0.0, 0.3)
    bcd = np.ascontiguousarray(bc_dofs, np.int32)
    mk = np.zeros(ndofs, np.int8)
    mk[bcd] = 1
    fa = None if f is None else np.ascontiguousarray(f, np.float64)
    ga = None if g is None else np.ascontiguousarray(g, np.float64)
    vals = np.empty(cols.size) if vals is None else vals
    b = np.empty(ndofs) if b is None else b
    u = np.empty(ndofs) if u is None else u
    order, off = colours
    sec = np.zeros(3)
    it = lib().orc_poisson_step_threaded(
        C.byref(form), nc, np.ascontiguousarray(cells), x, np.ascontiguousarray(dofmap),
        int(ndofs), mk, bcd.size, bcd, _ptr(ga), _ptr(fa), row_ptr, cols, vals, b, u, order,
        off, off.size - 1, float(rtol), int(kmax), int(threads), sec)
    if it == -1000001:
        raise ValueError("the colour classes do not cover the cells")
    if it <= -1000000:
        raise RuntimeError("Entry not in sparsity")
    return it, sec, vals, b, u


def assemble_matrix_interior_facets(degree, quads, cells, x, dofmap, row_ptr, cols, gamma=None,
                                    gamma_const=1.0, bc_markers=None, vals=None):
    """Continuous interior penalty over interior facets (quads), added into
    vals (a new zero array when None)."""
    q = np.ascontiguousarray(quads, np.int32).reshape(-1, 4)
    if vals is None:
        vals = np.zeros(cols.size, np.float64)
    ga = None if gamma is None else np.ascontiguousarray(gamma, np.float64)
    bcm = None if bc_markers is None else np.ascontiguousarray(bc_markers, np.int8)
    rc = lib().orc_assemble_matrix_interior_facets(int(degree), q.shape[0], q,
                                                   np.ascontiguousarray(cells), x,
                                                   np.ascontiguousarray(dofmap), _ptr(ga),
                                                   float(gamma_const), _ptr(bcm), row_ptr, cols,
                                                   vals)
    if rc == 3:
        raise RuntimeError("Entry not in sparsity")
    return vals


def assemble_vector_interior_facets(degree, quads, cells, x, dofmap, n, g=None, g_const=1.0,
                                    b=None):
    """int_F avg(g) avg(v) dS: each side's half of the facet integral, by
    the exterior-facet loop on the quads' two (cell, local facet) pairs."""
    q = np.ascontiguousarray(quads, np.int32).reshape(-1, 4)
    pairs = np.ascontiguousarray(np.concatenate([q[:, :2], q[:, 2:]]), np.int32)
    half_g = None if g is None else 0.5 * np.asarray(g, np.float64)
    return assemble_vector_facets(degree, pairs, cells, x, dofmap, n, g=half_g,
                                  g_const=0.5 * g_const, b=b)
