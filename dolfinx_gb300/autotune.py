"""In-project autotuner: launch shapes picked by timing on this GPU.

- cells per block of the matrix assembly kernel (16, 32, 64; elasticity
  2, 4, 8), recorded in the library's table per form and mode, so every
  later ``assemble_matrix`` of that workload uses it;
- lanes per row of the scalar CSR SpMV (4, 8, 16, 32: the row split of
  ``MatrixCSR::mult`` and of the CSR CG), recorded per matrix shape;
- the window sigma of the sliced-ELL solver operator (rows are sorted by
  length inside windows of sigma rows: a wider window pads less, a narrower
  one keeps rows nearer their RCM neighbours), picked by timing the FP32 and
  FP64 operators built with each candidate.

Every candidate computes the same result; the tuner only measures.
"""

from __future__ import annotations

import ctypes as C

import torch

from . import _capi, la

SIGMA_CANDIDATES = (64, 256, 1024)


def tune_assembly(asm) -> dict:
    """Time the candidates of a ``fem.MatrixAssembler``'s matrix kernel (into
    scratch values) and record the fastest."""
    order, off, ncol = asm.colour
    scratch = torch.empty_like(asm.A.vals)
    best = C.c_int32(0)
    ms = (C.c_float * 3)()
    _capi.check(_capi.lib().dfx_tune_assembly(
        C.byref(asm.form), C.byref(asm.A.csr()), la._ptr(asm.map), la._ptr(asm.markers),
        asm.mode, order, off, ncol, la._ptr(scratch), C.byref(best), ms, la._stream()))
    cand = (2, 4, 8) if asm.A.bs == 3 else (16, 32, 64)
    return {"cells_per_block": best.value, "ms": {c: float(t) for c, t in zip(cand, ms)}}


def tune_spmv(A: la.MatrixCSR) -> dict:
    """Time 4/8/16/32 lanes per row on y = A x and record the fastest."""
    x = torch.rand(A.ncols * A.bs, dtype=A.vals.dtype, device=A.vals.device)
    y = torch.empty(A.nrows * A.bs, dtype=A.vals.dtype, device=A.vals.device)
    best = C.c_int32(0)
    ms = (C.c_float * 4)()
    _capi.check(_capi.lib().dfx_tune_spmv(C.byref(A.csr()), la._ptr(x), la._ptr(y),
                                          C.byref(best), ms, la._stream()))
    return {"lanes_per_row": best.value, "ms": {c: float(t) for c, t in zip((4, 8, 16, 32), ms)}}


def _op_ms(op: la.SellOperator, dtype, n: int, reps: int) -> float:
    x = torch.rand(n, dtype=dtype, device="cuda")
    y = torch.empty_like(x)
    for _ in range(2):
        op.apply_renumbered(x, y)
    s = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(reps):
        op.apply_renumbered(x, y)
    e1.record(s)
    e1.synchronize()
    return e0.elapsed_time(e1) / reps


def tune_sigma(A: la.MatrixCSR, candidates=SIGMA_CANDIDATES, reps: int = 10) -> dict:
    """Window sigma for the FP32 (16-bit columns) and FP64 operators of A:
    the candidate with the least FP32 + FP64 SpMV time. Both operators of a
    mixed-precision solve must share one sigma, so one value is picked."""
    n = A.nrows
    res = {}
    for sg in candidates:
        o32 = la.SellOperator(A, torch.float32, sg, compress_cols=True)
        o64 = la.SellOperator(A, torch.float64, sg)
        res[sg] = {"f32_ms": _op_ms(o32, torch.float32, n, reps),
                   "f64_ms": _op_ms(o64, torch.float64, n, reps),
                   "padding_f32": o32.info()["padding"]}
        del o32, o64
    best = min(res, key=lambda sg: res[sg]["f32_ms"] + res[sg]["f64_ms"])
    return {"sigma": best, "candidates": res}


def clear() -> None:
    """Forget every choice recorded in the library's table."""
    _capi.check(_capi.lib().dfx_tune_clear())
