"""Device-resident linear algebra mirroring ``dolfinx.la`` (MatrixCSR, Vector,
inner_product, norm) plus the Jacobi-preconditioned CG of the matrix-free
demo. Storage is la::MatrixCSR's (int64 row pointers, int32 columns,
row-major bs x bs blocks) in device memory owned by torch tensors; every
operation runs in libdfxgpu.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from . import _capi


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _check_vec(t, n: int, dtype, device, name: str) -> None:
    """A vector that a kernel reads or writes through a raw pointer must be a
    contiguous CUDA tensor of `dtype` with n entries on `device`: checked on
    the host, so that a wrong argument raises instead of reaching the GPU."""
    if not torch.is_tensor(t):
        raise TypeError(f"{name} must be a torch tensor")
    if t.device.type != "cuda":
        raise ValueError(f"{name} must be on a CUDA device (got {t.device})")
    if t.device != device:
        raise ValueError(f"{name} must be on {device} (got {t.device})")
    if t.dtype != dtype:
        raise TypeError(f"{name} must be {dtype} (got {t.dtype})")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")
    if t.numel() != n:
        raise ValueError(f"{name} must have {n} entries (got {t.numel()})")


class MatrixCSR:
    """CSR matrix with square bs x bs blocks (cpp/dolfinx/la/MatrixCSR.h:67-1017)."""

    def __init__(self, row_ptr: torch.Tensor, cols: torch.Tensor, vals: torch.Tensor, bs: int = 1,
                 ncols: int | None = None):
        if row_ptr.dtype != torch.int64 or cols.dtype != torch.int32:
            raise TypeError("row_ptr must be int64 and cols int32")
        if vals.dtype not in (torch.float64, torch.float32):
            raise TypeError("values must be float64 or float32")
        if not (row_ptr.device == cols.device == vals.device):
            raise ValueError("row_ptr, cols and values must be on one device")
        if row_ptr.dim() != 1 or row_ptr.numel() < 1 or cols.dim() != 1:
            raise ValueError("row_ptr and cols must be 1-D, row_ptr non-empty")
        if vals.numel() != cols.numel() * int(bs) * int(bs):
            raise ValueError(f"{cols.numel()} entries of {bs}x{bs} blocks need "
                             f"{cols.numel() * int(bs) * int(bs)} values (got {vals.numel()})")
        self.row_ptr, self.cols, self.vals, self.bs = row_ptr, cols, vals, int(bs)
        self.nrows = int(row_ptr.numel() - 1)
        self.ncols = self.nrows if ncols is None else int(ncols)
        self.nnz = int(cols.numel())
        self._slot_map = None
        self._csr = None

    @property
    def dtype(self):
        return self.vals.dtype

    @property
    def block_size(self):
        return (self.bs, self.bs)

    def csr(self) -> _capi.Csr:
        c = self._csr
        if c is None or c.vals != self.vals.data_ptr():
            c = _capi.Csr(self.nrows, self.ncols, self.bs,
                          _capi.F64 if self.vals.dtype == torch.float64 else _capi.F32, self.nnz,
                          self.row_ptr.data_ptr(), self.cols.data_ptr(), self.vals.data_ptr())
            self._csr = c
        return c

    def set_value(self, v: float = 0.0) -> None:
        self.vals.fill_(v)

    def _check_xy(self, x, y) -> None:
        dev, dt = self.vals.device, self.vals.dtype
        _check_vec(x, self.ncols * self.bs, dt, dev, "x")
        _check_vec(y, self.nrows * self.bs, dt, dev, "y")

    def mult(self, x: torch.Tensor, y: torch.Tensor) -> None:
        """y += A x (MatrixCSR::mult)."""
        self._check_xy(x, y)
        _capi.check(_capi.lib().dfx_spmv(C.byref(self.csr()), _ptr(x), _ptr(y), 1.0, _stream()))

    def matvec(self, x: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        """Return A x (overwrites `out`)."""
        if out is None:
            out = torch.empty(self.nrows * self.bs, dtype=x.dtype, device=x.device)
        self._check_xy(x, out)
        _capi.check(_capi.lib().dfx_spmv(C.byref(self.csr()), _ptr(x), _ptr(out), 0.0, _stream()))
        return out

    def astype_float32(self) -> "MatrixCSR":
        """The float copy of the values (MatrixCSR converting constructor)."""
        v32 = torch.empty(self.vals.numel(), dtype=torch.float32, device=self.vals.device)
        _capi.check(_capi.lib().dfx_csr_values_to_f32(C.byref(self.csr()), _ptr(v32), _stream()))
        return MatrixCSR(self.row_ptr, self.cols, v32, self.bs, self.ncols)

    def expand_blocks(self, out: "MatrixCSR | None" = None) -> "MatrixCSR":
        """Scalar CSR of a block matrix (out: refresh its values only)."""
        if self.vals.dtype != torch.float64:
            raise TypeError("expand_blocks needs float64 values")
        if out is None:
            dev = self.vals.device
            rp = torch.empty(self.nrows * self.bs + 1, dtype=torch.int64, device=dev)
            cols = torch.empty(self.nnz * self.bs * self.bs, dtype=torch.int32, device=dev)
            vals = torch.empty(self.nnz * self.bs * self.bs, dtype=torch.float64, device=dev)
            _capi.check(_capi.lib().dfx_csr_expand_blocks(C.byref(self.csr()), _ptr(rp),
                                                          _ptr(cols), _ptr(vals), _stream()))
            return MatrixCSR(rp, cols, vals, 1, self.ncols * self.bs)
        _capi.check(_capi.lib().dfx_csr_expand_blocks(C.byref(self.csr()), _ptr(out.row_ptr),
                                                      None, _ptr(out.vals), _stream()))
        return out

    def inverse_diagonal(self) -> torch.Tensor:
        d = torch.empty(self.nrows * self.bs, dtype=torch.float64, device=self.vals.device)
        _capi.check(_capi.lib().dfx_jacobi_inverse_diagonal(C.byref(self.csr()), _ptr(d),
                                                            _stream()))
        return d

    def squared_norm(self) -> float:
        return float((self.vals.double() ** 2).sum())

    def to_scipy(self):
        import scipy.sparse as sp

        rp = self.row_ptr.cpu().numpy()
        cols = self.cols.cpu().numpy()
        vals = self.vals.cpu().numpy()
        if self.bs == 1:
            return sp.csr_matrix((vals, cols, rp), shape=(self.nrows, self.ncols))
        return sp.bsr_matrix((vals.reshape(-1, self.bs, self.bs), cols, rp),
                             shape=(self.nrows * self.bs, self.ncols * self.bs))


class Vector:
    """la::Vector on the device: ``array`` is a torch tensor."""

    def __init__(self, array: torch.Tensor, bs: int = 1):
        self.array = array
        self.bs = bs

    def scatter_forward(self):  # one rank: no ghosts
        pass

    def scatter_reverse(self, *args):  # one rank: no ghosts
        pass


def inner_product(a: torch.Tensor, b: torch.Tensor) -> float:
    """la::inner_product (deterministic two-stage device reduction)."""
    n = a.numel()
    _check_vec(a, n, torch.float64, a.device, "a")
    _check_vec(b, n, torch.float64, a.device, "b")
    wb = _capi.lib().dfx_inner_product_workspace_bytes(n)
    work = torch.empty(int(wb) // 8 + 1, dtype=torch.float64, device=a.device)
    out = C.c_double(0.0)
    _capi.check(_capi.lib().dfx_inner_product(_ptr(a), _ptr(b), n, _ptr(work), wb, C.byref(out),
                                              _stream()))
    return out.value


def squared_norm(a: torch.Tensor) -> float:
    return inner_product(a, a)


def norm(a: torch.Tensor) -> float:
    return float(np.sqrt(squared_norm(a)))


@dataclass
class CGResult:
    iterations: int
    status: int
    rnorm0_sq: float
    rnorm_sq: float
    kernel_launches: int = 0


class CGSolver:
    """Jacobi-preconditioned CG on a device CSR matrix, FP64 (graph-captured
    iterations; workspace allocated once and reused)."""

    def __init__(self, A: MatrixCSR, jacobi: bool = True, graph_iters: int = 20):
        if A.dtype != torch.float64:
            raise TypeError("CG needs a float64 matrix")
        self.A = A
        self.n = A.nrows * A.bs
        self.dinv = A.inverse_diagonal() if jacobi else None
        wb = int(_capi.lib().dfx_cg_workspace_bytes(self.n))
        self.work = torch.empty(wb, dtype=torch.uint8, device=A.vals.device)
        self.graph_iters = graph_iters

    def refresh_preconditioner(self):
        if self.dinv is not None:
            _capi.check(_capi.lib().dfx_jacobi_inverse_diagonal(C.byref(self.A.csr()),
                                                                _ptr(self.dinv), _stream()))

    def solve(self, b: torch.Tensor, x: torch.Tensor, rtol: float = 1e-10,
              max_iters: int = 100000, raise_on_fail: bool = True) -> CGResult:
        _check_vec(b, self.n, torch.float64, self.A.vals.device, "b")
        _check_vec(x, self.n, torch.float64, self.A.vals.device, "x")
        info = _capi.CgInfo()
        rc = _capi.lib().dfx_cg_solve(C.byref(self.A.csr()), _ptr(b), _ptr(x), _ptr(self.dinv),
                                      float(rtol), int(max_iters), int(self.graph_iters),
                                      _ptr(self.work), self.work.numel(), C.byref(info), _stream())
        if raise_on_fail:
            _capi.check(rc)
        return CGResult(info.iterations, info.status, info.rnorm0_sq, info.rnorm_sq,
                        info.kernel_launches)


class SellOperator:
    """Sliced-ELL (SELL-32-sigma) solver copy of a scalar MatrixCSR: FP64, or
    FP32 with 16-bit column deltas, or (split=True) each FP64 value as two
    FP32 words multiplied on the FP32 pipe with error-free transformations
    -- FP64-equivalent products on FP64 vectors. A 3x3-block MatrixCSR
    (bs 3) gives a block operator, FP64 or split: one column index per
    block, slices of 32 block rows, sigma counted in block rows. Values are
    refreshed from the CSR values with update_values() after re-assembly."""

    def __init__(self, A: MatrixCSR, dtype=torch.float64, sigma: int = 256,
                 compress_cols: bool | None = None, share_of: "SellOperator | None" = None,
                 build: int = 0, split: bool = False, pool_stream=None):
        """build: where the structure is built (0 device with host fallback,
        1 device only, 2 host); every place gives the same operator.
        pool_stream (shares only): take the values from the library's
        stream-ordered pool in the order of this torch stream, and return them
        there when the share is dropped -- for servers that make and drop a
        share per request, where cudaMalloc / cudaFree would wait for the
        whole device. Drop such a share only after its last use."""
        self.A, self.dtype, self.sigma = A, dtype, sigma
        self.csr_nnz = A.nnz if A is not None else share_of.csr_nnz
        self.split = bool(split)
        if self.split and dtype != torch.float64:
            raise ValueError("a split operator acts on FP64 vectors")
        h = C.c_void_p()
        if share_of is not None:
            # same structure as share_of, own values (one set per request)
            self.dtype, self.sigma, self.compressed = share_of.dtype, share_of.sigma, share_of.compressed
            self.split = share_of.split
            self.n, self.device = share_of.n, share_of.device
            if pool_stream is not None:
                self._pool_stream = pool_stream
                _capi.check(_capi.lib().dfx_operator_share_async(
                    share_of.handle, C.c_void_p(pool_stream.cuda_stream), C.byref(h)))
            else:
                _capi.check(_capi.lib().dfx_operator_share(share_of.handle, C.byref(h)))
            self.source = share_of
            self.handle = h
            if A is not None:
                self.update_values()
            return
        self.n, self.device = A.nrows * A.bs, A.vals.device
        if compress_cols is None:
            compress_cols = (dtype == torch.float32 or self.split) and A.bs == 1
        dt = _capi.F64 if dtype == torch.float64 else _capi.F32
        if self.split:
            dt = _capi.F32X2
        _capi.check(_capi.lib().dfx_operator_create_ex(C.byref(A.csr()), sigma, dt,
                                                       int(bool(compress_cols)), int(build),
                                                       C.byref(h), _stream()))
        self.handle = h
        self.compressed = bool(compress_cols)

    def share(self, A: MatrixCSR, pool_stream=None) -> "SellOperator":
        """An operator with this structure and the values of A (pool_stream:
        see __init__)."""
        return SellOperator(A, share_of=self, pool_stream=pool_stream)

    def to_operator(self, v: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        """v in the operator's (renumbered) numbering."""
        if out is None:
            out = torch.empty_like(v)
        _check_vec(v, self.n, torch.float64, self.device, "v")
        _check_vec(out, self.n, torch.float64, self.device, "out")
        _capi.check(_capi.lib().dfx_operator_permute(self.handle, _ptr(v), _ptr(out), 1, _stream()))
        return out

    def from_operator(self, v: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        """v back in the original numbering."""
        if out is None:
            out = torch.empty_like(v)
        _check_vec(v, self.n, torch.float64, self.device, "v")
        _check_vec(out, self.n, torch.float64, self.device, "out")
        _capi.check(_capi.lib().dfx_operator_permute(self.handle, _ptr(v), _ptr(out), 0, _stream()))
        return out

    def update_values(self):
        _capi.check(_capi.lib().dfx_operator_update_values(self.handle, C.byref(self.A.csr()),
                                                           _stream()))

    def apply(self, x: torch.Tensor, y: torch.Tensor | None = None) -> torch.Tensor:
        if y is None:
            y = torch.empty_like(x)
        _check_vec(x, self.n, self.dtype, self.device, "x")
        _check_vec(y, self.n, self.dtype, self.device, "y")
        _capi.check(_capi.lib().dfx_operator_apply(self.handle, _ptr(x), _ptr(y), _stream()))
        return y

    def apply_renumbered(self, xp: torch.Tensor, yp: torch.Tensor) -> torch.Tensor:
        """The bare SpMV in the operator's numbering."""
        _check_vec(xp, self.n, self.dtype, self.device, "xp")
        _check_vec(yp, self.n, self.dtype, self.device, "yp")
        _capi.check(_capi.lib().dfx_operator_apply_renumbered(self.handle, _ptr(xp), _ptr(yp),
                                                              _stream()))
        return yp

    def set_chunk(self, chunk: int) -> None:
        """Value pairs per load chunk of the FP32 SpMV (2, 4 or 8); for a
        3x3-block operator 2, 4 or 8 stand for 1, 2 or 4 block slots per
        round. The product is bitwise the same for each."""
        _capi.check(_capi.lib().dfx_operator_set_chunk(self.handle, int(chunk)))

    def info(self):
        ns = C.c_int64()
        nsl = C.c_int32()
        perm = C.c_void_p()
        _capi.check(_capi.lib().dfx_operator_info(self.handle, C.byref(ns), C.byref(nsl),
                                                   C.byref(perm)))
        pad = ns.value / self.csr_nnz - 1 if self.csr_nnz else 0.0
        return {"slots": ns.value, "slices": nsl.value, "padding": pad}

    def release_values(self) -> None:
        """Free the values and scratch of a structure-owning operator that is
        only shared from: its shares keep their own values, and applying or
        solving with this operator raises afterwards. The operator lets go
        of its matrix too."""
        _capi.check(_capi.lib().dfx_operator_release_values(self.handle))
        self.A = None

    def device_bytes(self) -> int:
        """Device memory the operator holds (values and scratch; the
        structure arrays too unless it is a share)."""
        b = C.c_size_t(0)
        _capi.check(_capi.lib().dfx_operator_device_bytes(self.handle, C.byref(b)))
        return int(b.value)

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value and _capi is not None:
            try:
                ps = getattr(self, "_pool_stream", None)
                if ps is not None:
                    _capi.lib().dfx_operator_destroy_async(h, C.c_void_p(ps.cuda_stream))
                else:
                    _capi.lib().dfx_operator_destroy(h)
            except Exception:
                pass
            self.handle = None


class OperatorCGSolver:
    """FP64 Jacobi-PCG on the sliced-ELL operator (same iteration and
    stopping test as CGSolver). split=True applies the matrix as two FP32
    words per value on the FP32 pipe (SellOperator(split=True)); vectors,
    dot products and updates stay FP64."""

    def __init__(self, A: MatrixCSR, jacobi: bool = True, graph_iters: int = 20,
                 sigma: int = 256, split: bool = False):
        self.A = A
        self.op = SellOperator(A, torch.float64, sigma, split=split)
        self.n = A.nrows * A.bs
        self.dinv = A.inverse_diagonal() if jacobi else None
        wb = int(_capi.lib().dfx_cg_op_workspace_bytes(self.n))
        self.work = torch.empty(wb, dtype=torch.uint8, device=A.vals.device)
        self.graph_iters = graph_iters

    def refresh(self):
        """Re-read the CSR values (after re-assembly)."""
        self.op.update_values()
        if self.dinv is not None:
            _capi.check(_capi.lib().dfx_jacobi_inverse_diagonal(C.byref(self.A.csr()),
                                                                _ptr(self.dinv), _stream()))

    def solve(self, b, x, rtol=1e-10, max_iters=100000, raise_on_fail=True) -> CGResult:
        _check_vec(b, self.n, torch.float64, self.op.device, "b")
        _check_vec(x, self.n, torch.float64, self.op.device, "x")
        info = _capi.CgInfo()
        rc = _capi.lib().dfx_cg_solve_op(self.op.handle, _ptr(b), _ptr(x), _ptr(self.dinv),
                                         float(rtol), int(max_iters), int(self.graph_iters),
                                         _ptr(self.work), self.work.numel(), C.byref(info),
                                         _stream())
        if raise_on_fail:
            _capi.check(rc)
        return CGResult(info.iterations, info.status, info.rnorm0_sq, info.rnorm_sq,
                        info.kernel_launches)


@dataclass
class IRResult:
    outer_iterations: int
    inner_iterations: int
    status: int
    rnorm0_sq: float
    rnorm_sq: float
    kernel_launches: int = 0

    @property
    def iterations(self):
        return self.inner_iterations


class IRSolver:
    """Mixed-precision iterative refinement: FP64 residual, norm and update
    with the FP64 operator; FP32 Jacobi-PCG corrections on the FP32
    16-bit-column operator."""

    def __init__(self, A: MatrixCSR, jacobi: bool = True, graph_iters: int = 20,
                 sigma: int = 256, inner_rtol: float | None = None, compress_cols: bool = True,
                 variant: str = "reliable"):
        self.variant = {"restart": _capi.IR_RESTART, "reliable": _capi.IR_RELIABLE,
                        "flexible": _capi.IR_FLEXIBLE}[variant]
        if inner_rtol is None:
            # Reliable updates: replace the residual each time |r| drops by this
            # factor. On the P2 Poisson problem of a 64^3 x 6 mesh the inner
            # iteration count does not depend on it (~1,360 from 0.3 down to 0.01),
            # and 0.03 needs the fewest FP64 replacements. Flexible CG: each
            # inner FP32 solve reduces its residual by this factor.
            inner_rtol = {_capi.IR_RELIABLE: 0.03, _capi.IR_FLEXIBLE: 0.1}.get(self.variant, 1e-4)
        self.A = A
        self.op64 = SellOperator(A, torch.float64, sigma)
        self.op32 = SellOperator(A, torch.float32, sigma, compress_cols=compress_cols)
        self.n = A.nrows
        self.dinv = A.inverse_diagonal() if jacobi else None
        wb = int(_capi.lib().dfx_ir_workspace_bytes(self.n))
        self.work = torch.empty(wb, dtype=torch.uint8, device=A.vals.device)
        self.graph_iters = graph_iters
        self.inner_rtol = inner_rtol

    def refresh(self):
        self.op64.update_values()
        self.op32.update_values()
        if self.dinv is not None:
            _capi.check(_capi.lib().dfx_jacobi_inverse_diagonal(C.byref(self.A.csr()),
                                                                _ptr(self.dinv), _stream()))

    def solve(self, b, x, rtol=1e-10, max_outer=200, max_inner=100000,
              raise_on_fail=True) -> IRResult:
        _check_vec(b, self.n, torch.float64, self.op64.device, "b")
        _check_vec(x, self.n, torch.float64, self.op64.device, "x")
        info = _capi.IrInfo()
        rc = _capi.lib().dfx_ir_solve(self.op64.handle, self.op32.handle, _ptr(b), _ptr(x),
                                      _ptr(self.dinv), float(rtol), float(self.inner_rtol),
                                      int(max_outer), int(max_inner), int(self.graph_iters),
                                      int(self.variant), _ptr(self.work), self.work.numel(),
                                      C.byref(info), _stream())
        if raise_on_fail:
            _capi.check(rc)
        return IRResult(info.outer_iterations, info.inner_iterations, info.status,
                        info.rnorm0_sq, info.rnorm_sq, info.kernel_launches)


def cg(A: MatrixCSR, b: torch.Tensor, x: torch.Tensor | None = None, rtol: float = 1e-10,
       max_iters: int = 100000, jacobi: bool = True):
    """Solve A x = b; returns (x, CGResult)."""
    if x is None:
        x = torch.zeros_like(b)
    res = CGSolver(A, jacobi=jacobi).solve(b, x, rtol, max_iters)
    return x, res
