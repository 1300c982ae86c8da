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

The choices can be written to a tuning cache file and read back by a later
process (``save`` / ``load``), so that a restarted server skips the timing:
``tune_assembly`` and ``tune_sigma`` with ``reuse=True`` return a recorded
choice without timing.
"""

from __future__ import annotations

import ctypes as C
import json
import os

import numpy as np
import torch

from . import _capi, la

SIGMA_CANDIDATES = (64, 256, 1024, 2048, 4096)
CACHE_FORMAT = "dfx-tuning"
CACHE_VERSION = 1

_WHAT_ASSEMBLY, _WHAT_SPMV = 1, 2

# Window sigma per (device, rows, entries), recorded by tune_sigma.
_sigma_choices: dict[tuple[int, int, int], int] = {}


def _device_index(t=None) -> int:
    if t is not None:
        return t.device.index if t.device.type == "cuda" else 0
    return torch.cuda.current_device() if torch.cuda.is_available() else 0


def assembly_key(form, mode: int) -> int:
    """The workload key of a matrix assembly in the library's table:
    16 kind + 4 degree + 2 mass + mode (mass: a Poisson form with k2 != 0)."""
    mass = int(form.kind == _capi.FORM_POISSON and form.k2 != 0.0)
    return ((form.kind * 4 + form.degree) * 2 + mass) * 2 + int(mode)


def _table() -> np.ndarray:
    L = _capi.lib()
    n = C.c_int64(0)
    _capi.check(L.dfx_tune_export(None, 0, C.byref(n)))
    rows = np.zeros((max(n.value, 1), 6), np.int64)
    _capi.check(L.dfx_tune_export(rows.ctypes.data, rows.shape[0], C.byref(n)))
    return rows[: n.value]


def recorded_cells_per_block(form, mode: int, device: int | None = None) -> int | None:
    """The cells per block recorded for this form and mode (tuned, pinned or
    loaded from a cache file), or None when the kernel would use its
    default."""
    dev = _device_index() if device is None else device
    key = (dev, _WHAT_ASSEMBLY, form.num_cells, assembly_key(form, mode), 0)
    for r in _table():
        if tuple(int(v) for v in r[:5]) == key:
            return int(r[5])
    return None


def recorded_sigma(A) -> int | None:
    """The window sigma recorded for matrices of A's shape, or None."""
    return _sigma_choices.get((_device_index(A.vals), int(A.nrows), int(A.nnz)))


def pin_sigma(A, sigma: int) -> None:
    """Record a window sigma for matrices of A's shape (a positive multiple
    of 32), or forget it (sigma = 0)."""
    key = (_device_index(A.vals), int(A.nrows), int(A.nnz))
    if sigma == 0:
        _sigma_choices.pop(key, None)
        return
    if sigma < 32 or sigma % 32:
        raise ValueError("sigma must be a positive multiple of 32")
    _sigma_choices[key] = int(sigma)


def tune_assembly(asm, reuse: bool = False) -> dict:
    """Time the candidates of a ``fem.MatrixAssembler``'s matrix kernel (into
    scratch values) and record the fastest. reuse: when a choice is already
    recorded for this workload, return it without timing."""
    if reuse:
        v = recorded_cells_per_block(asm.form, asm.mode)
        if v is not None:
            return {"cells_per_block": v, "ms": None, "recorded": True}
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


def tune_sigma(A: la.MatrixCSR, candidates=SIGMA_CANDIDATES, reps: int = 10,
               reuse: bool = False) -> dict:
    """Window sigma for the FP32 (16-bit columns) and FP64 operators of A:
    the candidate with the least FP32 + FP64 SpMV time. Both operators of a
    mixed-precision solve must share one sigma, so one value is picked. The
    choice is recorded for matrices of A's shape. reuse: when a sigma is
    already recorded for the shape, return it without timing. A 3x3-block
    matrix (bs 3) has no FP32 operator: its split and FP64 block operators
    are timed instead, sigma counted in block rows."""
    if reuse:
        v = recorded_sigma(A)
        if v is not None:
            return {"sigma": v, "candidates": None, "recorded": True}
    n = A.nrows * A.bs
    res = {}
    if A.bs == 3:
        for sg in candidates:
            osp = la.SellOperator(A, torch.float64, sg, split=True)
            o64 = la.SellOperator(A, torch.float64, sg)
            res[sg] = {"split_ms": _op_ms(osp, torch.float64, n, reps),
                       "f64_ms": _op_ms(o64, torch.float64, n, reps)}
            del osp, o64
        best = min(res, key=lambda sg: res[sg]["split_ms"] + res[sg]["f64_ms"])
        _sigma_choices[(_device_index(A.vals), int(A.nrows), int(A.nnz))] = best
        return {"sigma": best, "candidates": res}
    for sg in candidates:
        o32 = la.SellOperator(A, torch.float32, sg, compress_cols=True)
        o64 = la.SellOperator(A, torch.float64, sg)
        res[sg] = {"f32_ms": _op_ms(o32, torch.float32, n, reps),
                   "f64_ms": _op_ms(o64, torch.float64, n, reps),
                   "padding_f32": o32.info()["padding"]}
        del o32, o64
    best = min(res, key=lambda sg: res[sg]["f32_ms"] + res[sg]["f64_ms"])
    _sigma_choices[(_device_index(A.vals), int(A.nrows), int(A.nnz))] = best
    return {"sigma": best, "candidates": res}


CHUNK_CANDIDATES = (2, 4, 8)


def tune_chunk(op: la.SellOperator, candidates=CHUNK_CANDIDATES, reps: int = 20) -> dict:
    """Value pairs per load chunk of an FP32 operator's SpMV: each candidate
    timed on the operator itself (the product is bitwise the same for all),
    the fastest kept on the operator."""
    if op.dtype != torch.float32:
        raise ValueError("the chunk is a launch shape of FP32 operators")
    res = {}
    for ch in candidates:
        op.set_chunk(ch)
        res[ch] = _op_ms(op, torch.float32, op.n, reps)
    best = min(res, key=res.get)
    op.set_chunk(best)
    return {"chunk": best, "candidates": res}


def clear() -> None:
    """Forget every recorded choice (the library's table and the sigmas)."""
    _capi.check(_capi.lib().dfx_tune_clear())
    _sigma_choices.clear()


def _device_names() -> dict[int, str]:
    if not torch.cuda.is_available():
        return {}
    return {d: torch.cuda.get_device_name(d) for d in range(torch.cuda.device_count())}


def save(path: str) -> int:
    """Write every recorded choice to a tuning cache file (JSON, replaced
    atomically) with the names of the devices they were measured on.
    Returns the number of choices written."""
    rows = _table()
    names = _device_names()
    sig = sorted(_sigma_choices.items())
    devs = sorted({int(r[0]) for r in rows} | {k[0] for k, _ in sig})
    doc = {"format": CACHE_FORMAT, "version": CACHE_VERSION,
           "abi": int(_capi.lib().dfx_abi_version()),
           "devices": {str(d): names.get(d) for d in devs},
           "choices": [[int(v) for v in r] for r in rows],
           "sigma": [[d, n, nnz, s] for (d, n, nnz), s in sig]}
    tmp = f"{path}.tmp{os.getpid()}"
    with open(tmp, "w") as f:
        json.dump(doc, f, indent=1)
    os.replace(tmp, path)
    return len(doc["choices"]) + len(doc["sigma"])


def load(path: str, check_devices: bool = True) -> int:
    """Read a tuning cache file into this process's choices (replacing
    entries of the same workload). With check_devices, choices measured on
    a device whose name differs from this process's device of that index
    (or that this process does not have) are skipped; without a GPU in this
    process nothing is skipped. The whole file is checked before anything is
    recorded: a file of another format or version, or a bad choice, raises
    ValueError / DfxError and records nothing. Returns the number of choices
    recorded."""
    with open(path) as f:
        doc = json.load(f)
    if not isinstance(doc, dict) or doc.get("format") != CACHE_FORMAT:
        raise ValueError(f"{path} is not a tuning cache file")
    if doc.get("version") != CACHE_VERSION:
        raise ValueError(f"{path}: tuning cache version {doc.get('version')} is not "
                         f"{CACHE_VERSION}")
    names = _device_names()
    saved = {int(k): v for k, v in doc.get("devices", {}).items()}

    def usable(d: int) -> bool:
        if not (check_devices and names):
            return True
        return d in names and saved.get(d) == names[d]

    choices = doc.get("choices", [])
    if any(len(r) != 6 for r in choices):
        raise ValueError(f"{path}: a choice is not 6 integers")
    sig = [tuple(int(v) for v in e) for e in doc.get("sigma", [])]
    for e in sig:
        if len(e) != 4 or e[0] < 0 or e[1] < 0 or e[2] < 0 or e[3] <= 0 or e[3] % 32:
            raise ValueError(f"{path}: bad sigma entry {list(e)}")
    rows = np.array([r for r in choices if usable(int(r[0]))], np.int64).reshape(-1, 6)
    _capi.check(_capi.lib().dfx_tune_import(rows.ctypes.data if len(rows) else None, len(rows)))
    sig = [e for e in sig if usable(e[0])]
    for d, n, nnz, s in sig:
        _sigma_choices[(d, n, nnz)] = s
    return len(rows) + len(sig)
