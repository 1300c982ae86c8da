"""Device-resident serving loop for assemble-and-solve requests.

Each request is a Poisson/Helmholtz problem
``a(u, v) = int kappa grad u.grad v + k2 u v``, ``L(v) = int f v`` on a unit
cube of n^3 x 6 tetrahedra, Lagrange P1 or P2, with u = 0 on the whole
boundary. kappa is lognormal(0, 1) per cell and f ~ U[-1, 1] per P1 node, both
from the request's seed. The ``+ k2`` sign keeps the operator SPD for every
kappa field, so CG applies. The reference defines this Helmholtz problem in
python/demo/demo_helmholtz.py; the sign is this loop's stated choice.

Design (GB300, one GPU):

- **Resident structure.** Meshes, dofmaps, CSR structure, the cell->slot
  maps and the sliced-ELL operator structures are built once per
  (n, degree) and kept on the device in an LRU cache. A request only adds
  its own values: the CSR values, operator values and vectors.
- **Admission by HBM budget.** A request enters when its bytes fit under
  the budget, next to the cached structures and the requests in flight.
- **Small systems** (at most ``batch_max_dofs`` dofs) share one persistent
  batched CG launch (``dfx_batch_step``), one CTA per system. The launch
  advances every active system by ``quantum`` iterations; between launches
  finished systems retire and new requests join. This is continuous
  batching: requests that arrive while others run are admitted as slots and
  memory free up, and their work overlaps on the device.
- **Larger systems** go to a whole-GPU solver on worker threads, each with
  its own CUDA stream, so they overlap with the batch.

``mode = "mixed"``: FP32 operator and inner PCG with FP64 reliable updates.
``mode = "fp64"``: plain FP64 PCG. Both stop at ``|b - A x| / |b| < rtol``,
evaluated in FP64.
"""

from __future__ import annotations

import collections
import ctypes as C
import gc
import math
import queue
import threading
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _capi, autotune, fem, la, mesh
from . import log as _log


@dataclass
class Request:
    rid: int
    n: int
    degree: int
    k2: float
    seed: int
    arrival: float = 0.0  # seconds from the start of the stream


# Largest n whose 6 n^3 tetrahedra keep every cell-vertex index in int32.
MAX_N = 447


def request_error(req: Request) -> str | None:
    """Why a request cannot be served, or None: checked on the host before
    any device work, so that a malformed request is refused alone instead of
    stopping the loop."""
    if isinstance(req.n, bool) or not isinstance(req.n, (int, np.integer)) or req.n < 1:
        return f"n must be a positive integer (got {req.n!r})"
    if req.n > MAX_N:
        return f"n = {req.n}: mesh too large for int32 cell indices (n <= {MAX_N})"
    if req.degree not in (1, 2):
        return f"Lagrange degree {req.degree!r} not supported (1 or 2)"
    try:
        k2 = float(req.k2)
    except (TypeError, ValueError):
        return f"k2 must be a number (got {req.k2!r})"
    if not math.isfinite(k2) or k2 < 0.0:
        return f"k2 must be finite and >= 0 so that the operator is SPD (got {req.k2!r})"
    if isinstance(req.seed, bool) or not isinstance(req.seed, (int, np.integer)) or \
            not 0 <= req.seed < 2 ** 64:
        return f"seed must be an integer in [0, 2^64) (got {req.seed!r})"
    return None


@dataclass
class Rejected:
    """A request refused without a solve: malformed, larger than the whole
    HBM budget, or its set-up failed. status is a DFX_ERR_* code."""

    req: Request
    status: int
    error: str
    t_done: float
    st: None = None
    x: None = None
    iterations: int = 0


def make_requests(count: int, rate: float, seed: int = 0, n_range=(8, 96)) -> list[Request]:
    """Synthetic request stream: Poisson arrivals at `rate`/s, n log-uniform
    in n_range, P1/P2 with equal probability, k2 ~ U[0, 10]."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, count))
    lo, hi = math.log(n_range[0]), math.log(n_range[1])
    out = []
    for i in range(count):
        n = int(round(math.exp(rng.uniform(lo, hi))))
        deg = 1 if rng.uniform() < 0.5 else 2
        out.append(Request(i, n, deg, float(rng.uniform(0.0, 10.0)), int(rng.integers(2 ** 31)),
                           float(t[i])))
    return out


def request_inputs(msh: mesh.Mesh, seed: int, device="cuda"):
    """kappa ~ lognormal(0, 1) per cell and f ~ U[-1, 1] per P1 node, drawn on
    the device from the request's seed (on the current stream), so that a
    request costs the host no sampling and no host->device copy of its
    fields. The same seed gives the same fields, alone or in any mix."""
    g = torch.Generator(device=device)
    g.manual_seed(int(seed))
    kappa = torch.randn(msh.num_cells, dtype=torch.float64, device=device, generator=g).exp_()
    f = torch.rand(msh.num_nodes, dtype=torch.float64, device=device, generator=g)
    return kappa, f.mul_(2.0).sub_(1.0)


def _stream_ptr(s):
    return C.c_void_p(s.cuda_stream)


def unit_cube_boundary_nodes(X: np.ndarray) -> np.ndarray:
    """Nodes of a unit-cube space whose point (a row of X, every coordinate
    in [0, 1] up to rounding) has a coordinate that np.isclose (default
    tolerances) finds equal to 0 or to 1. On [0, 1] the coordinate closest
    to 0 is the smallest and the one closest to 1 the largest, so isclose's
    own test on those two gives the same answer as on all three, at a
    fraction of the work."""
    lo = np.minimum(np.minimum(X[:, 0], X[:, 1]), X[:, 2])
    hi = np.maximum(np.maximum(X[:, 0], X[:, 1]), X[:, 2])
    near0 = np.abs(lo) <= 1e-8 + 1e-5 * 0.0
    near1 = np.abs(hi - 1.0) <= 1e-8 + 1e-5 * 1.0
    return np.flatnonzero(near0 | near1).astype(np.int32)


def device_bytes(*roots) -> int:
    """Device memory held by the CUDA tensors and sliced-ELL operators
    reachable from `roots` through this package's objects, dicts, lists and
    tuples; each tensor storage and each operator is counted once."""
    seen: set[int] = set()
    storages: dict[int, int] = {}
    ops: dict[int, int] = {}
    stack = list(roots)
    while stack:
        o = stack.pop()
        if id(o) in seen or o is None:
            continue
        seen.add(id(o))
        if isinstance(o, torch.Tensor):
            if o.is_cuda:
                st = o.untyped_storage()
                storages[st.data_ptr()] = st.nbytes()
            continue
        if isinstance(o, dict):
            stack.extend(o.values())
            continue
        if isinstance(o, (list, tuple)):
            stack.extend(o)
            continue
        if not type(o).__module__.startswith(__package__ or "dolfinx_gb300"):
            continue
        if isinstance(o, la.SellOperator) and getattr(o, "handle", None) is not None:
            ops[o.handle.value] = o.device_bytes()
        stack.extend(getattr(o, "__dict__", {}).values())
    return sum(storages.values()) + sum(ops.values())


class Structure:
    """Everything of one (n, degree) that requests share."""

    def __init__(self, n: int, degree: int, device="cuda", tune: bool = True):
        """tune: time the launch-shape candidates on this structure (cells per
        block of the assembly, sliced-ELL window sigma) and use the fastest;
        a choice already recorded for the workload (an earlier structure of
        this size, or a loaded tuning cache file) is used without timing."""
        self.n, self.degree = n, degree
        self.mesh = mesh.create_unit_cube(n, n, n, device=device)
        self.V = fem.functionspace(self.mesh, ("Lagrange", degree), device=device)
        bnd = unit_cube_boundary_nodes(self.V.tabulate_dof_coordinates())
        self.bc = fem.dirichletbc(0.0, bnd, self.V)
        a = fem.poisson_form(self.V, 1.0, k2=1.0)
        self.asm = fem.MatrixAssembler(a, [self.bc])  # slot map, markers, structure
        self.A0 = self.asm.A
        self.A0.vals.fill_(1.0)  # any values: tuning times the kernels on them
        sigma = 256
        self.tuning = {}
        if tune:
            self.tuning["assembly"] = autotune.tune_assembly(self.asm, reuse=True)
            self.tuning["sigma"] = autotune.tune_sigma(self.A0, reuse=True)
            sigma = self.tuning["sigma"]["sigma"]
        self.op64 = la.SellOperator(self.A0, torch.float64, sigma)
        self.op32 = la.SellOperator(self.A0, torch.float32, sigma, compress_cols=True)
        self.ndofs = self.V.num_dofs
        self.nnz = self.A0.nnz
        # Every request holds its own matrix and operator values: the
        # structure keeps the pattern only (CSR row pointers and columns, the
        # operators' structure arrays), about half of what it would hold with
        # values.
        self.op64.release_values()
        self.op32.release_values()
        self.row_ptr, self.cols = self.A0.row_ptr, self.A0.cols
        self.asm.A = None
        self.A0 = None
        self.mesh.device(device)
        # Everything above that lives on the device: tensors and operators.
        self.bytes = device_bytes(self)
        self.users = 0

    def ops_slots(self):
        return self.op64.info()["slots"]

    def request_bytes(self) -> int:
        n = self.ndofs
        slots = self.ops_slots()
        return (self.nnz * 8 + slots * 12 + n * 8 * 8 + self.mesh.num_cells * 8
                + self.mesh.num_nodes * 8 + int(_capi.lib().dfx_ir_workspace_bytes(n)))


# Structures built in this process, shared by every server: a server counts
# the ones it uses against its own HBM budget, and an eviction drops the
# structure from this cache too, so that its memory is returned.
_structure_cache: collections.OrderedDict = collections.OrderedDict()
_structure_lock = threading.Lock()


def cached_structure(n: int, degree: int) -> Structure:
    key = (n, degree)
    with _structure_lock:
        st = _structure_cache.get(key)
    if st is None:
        t0 = time.perf_counter()
        built = Structure(n, degree)
        _log.logger.info("structure n=%s P%s built in %.3f s (%s dofs)", n, degree,
                         time.perf_counter() - t0, built.ndofs)
        with _structure_lock:
            st = _structure_cache.setdefault(key, built)
    return st


def drop_structure(n: int, degree: int) -> None:
    with _structure_lock:
        _structure_cache.pop((n, degree), None)


def clear_structure_cache() -> None:
    with _structure_lock:
        _structure_cache.clear()


class Job:
    """One admitted request: its values and vectors on the device."""

    def __init__(self, req: Request, st: Structure, mode: str, stream, assembly: str = "atomic"):
        self.req, self.st, self.mode = req, st, mode
        V = st.V
        with torch.cuda.stream(stream):
            self.kappa, self.f = request_inputs(st.mesh, req.seed)
            a = fem.poisson_form(V, self.kappa, k2=req.k2)
            L = fem.source_form(V, self.f)
            self.A = la.MatrixCSR(st.row_ptr, st.cols,
                                  torch.zeros(st.nnz, dtype=torch.float64,
                                              device=st.cols.device), 1)
            asm = st.asm
            amode = fem._mode(assembly)
            order, off, ncol = fem._colour_args(V, amode)
            _capi.check(_capi.lib().dfx_assemble_matrix(
                C.byref(a.cstruct()), C.byref(self.A.csr()), la._ptr(asm.map),
                la._ptr(asm.markers), amode, order, off, ncol, _stream_ptr(stream)))
            _capi.check(_capi.lib().dfx_set_diagonal(
                C.byref(self.A.csr()), la._ptr(asm.diag_dofs), int(asm.diag_dofs.numel()), 1.0,
                _stream_ptr(stream)))
            self.b = fem.RhsAssembler(L, a, [st.bc], mode=assembly).assemble()
            self.dinv = self.A.inverse_diagonal()
            # Shares from the library's stream-ordered pool: dropping one at
            # the end of the request does not wait for the whole device.
            self.op64 = st.op64.share(self.A, pool_stream=stream)
            self.op32 = st.op32.share(self.A, pool_stream=stream) if mode == "mixed" else None
            self.bp = self.op64.to_operator(self.b)
            self.dp = self.op64.to_operator(self.dinv)
            self.xp = torch.zeros_like(self.bp)
        self.slot = None
        self.info = None
        self.t_done = None

    def solution(self) -> torch.Tensor:
        return self.op64.from_operator(self.xp)

    def release_device(self) -> None:
        """Drop the request's device buffers (matrix values, operator values,
        vectors, coefficients) once its solution is on the host: a finished
        request keeps only x, its status and its timings."""
        for name in ("A", "op64", "op32", "b", "dinv", "bp", "dp", "xp", "kappa", "f", "work"):
            setattr(self, name, None)


class Server:
    """Continuous-batching server (one GPU)."""

    def __init__(self, mode: str = "mixed", hbm_budget: float = 64e9, capacity: int = 512,
                 quantum: int = 25, batch_max_dofs: int = 65536, rtol: float = 1e-10,
                 workers: int = 4, delta: float = 0.01, assembly: str = "atomic",
                 retain_systems: bool = False):
        """assembly: "atomic" (FP64 atomics) or "coloured" (deterministic
        summation order, so a request's matrix is bitwise reproducible).
        retain_systems: finished requests keep their device matrix and
        vectors (for checks); by default they are released when the
        solution reaches the host, so a long stream holds only the requests
        in flight.
        workers: threads (each with its own stream) solving the requests
        above batch_max_dofs. Four concurrent whole-GPU solves served 7 %
        more requests per second than two, in both modes, on a 64-request
        draw at 5000/s (the solves are bound by memory latency, and their
        launches and reductions interleave)."""
        self.retain_systems = bool(retain_systems)
        if mode not in ("mixed", "fp64"):
            raise ValueError(f'mode must be "mixed" or "fp64" (got {mode!r})')
        if assembly not in ("atomic", "coloured", "colored"):
            raise ValueError(f'assembly must be "atomic" or "coloured" (got {assembly!r})')
        self.assembly = assembly
        self.mode, self.budget, self.capacity = mode, hbm_budget, capacity
        self.quantum, self.batch_max_dofs, self.rtol = quantum, batch_max_dofs, rtol
        self.delta = delta
        self.structures: collections.OrderedDict = collections.OrderedDict()
        self.used = 0
        h = C.c_void_p()
        _capi.check(_capi.lib().dfx_batch_create(capacity, C.byref(h)))
        self.batch = h
        self.free_slots = list(range(capacity))
        self.active: dict[int, Job] = {}
        self.stream_setup = torch.cuda.Stream()
        self.stream_batch = torch.cuda.Stream()
        self.lock = threading.Lock()
        self.large_q: queue.Queue = queue.Queue()
        self.workers = [threading.Thread(target=self._worker, daemon=True) for _ in range(workers)]
        self.finished: list[Job] = []
        self._stop = False
        for w in self.workers:
            w.start()

    # ------------------------------------------------------------ structures
    def structure(self, n: int, degree: int) -> Structure:
        key = (n, degree)
        st = self.structures.get(key)
        if st is None:
            st = cached_structure(n, degree)
            self.structures[key] = st
            self.used += st.bytes
            self._evict(keep=key)
        self.structures.move_to_end(key)
        return st

    def _evict(self, keep=None, need: int = 0):
        """Drop least recently used idle structures (other than `keep`) until
        they and `need` more bytes fit under the budget."""
        for key in list(self.structures):
            if self.used + need <= self.budget:
                break
            st = self.structures[key]
            if st.users == 0 and key != keep:
                self.used -= st.bytes
                del self.structures[key]
                drop_structure(*key)
                del st
                # Collect cycles so the structure's operators and tensors are
                # freed now, and return torch's cached blocks to the device so
                # the library's own allocations can use them.
                gc.collect()
                torch.cuda.empty_cache()
                _capi.check(_capi.lib().dfx_operator_pool_trim())
                _log.logger.info("structure n=%s P%s evicted", key[0], key[1])

    def prewarm(self, requests):
        for key in sorted({(r.n, r.degree) for r in requests}):
            self.structure(*key)
        torch.cuda.synchronize()

    # ------------------------------------------------------------ admission
    def _reject(self, req: Request, status: int, error: str) -> Rejected:
        _log.logger.warning("request %s refused (status %s): %s", req.rid, status, error)
        rej = Rejected(req, int(status), error, time.perf_counter())
        with self.lock:
            self.finished.append(rej)
        return rej

    def admit(self, req: Request) -> Job | Rejected | None:
        """A Job when the request is admitted; None when it must wait for
        memory or a batch slot; a Rejected record when it can never run (its
        structure and values exceed the whole budget) or its set-up failed."""
        key = (req.n, req.degree)
        try:
            st = self.structure(*key)
        except Exception as exc:
            return self._reject(req, getattr(exc, "code", -1), f"structure set-up failed: {exc}")
        need = st.request_bytes()
        small = st.ndofs <= self.batch_max_dofs
        if st.bytes + need > self.budget:
            rej = self._reject(req, _capi.DFX_ERR_NO_MEMORY,
                               f"needs {st.bytes + need} bytes with its structure; the HBM "
                               f"budget is {self.budget:.0f}")
            with self.lock:
                self._evict()
            return rej
        with self.lock:
            if self.used + need > self.budget:
                self._evict(keep=key, need=need)
            if self.used + need > self.budget:
                return None
            if small and not self.free_slots:
                return None
            self.used += need
            st.users += 1
        t_setup = time.perf_counter()
        try:
            job = Job(req, st, self.mode, self.stream_setup, self.assembly)
        except Exception as exc:
            with self.lock:
                self.used -= need
                st.users -= 1
            return self._reject(req, getattr(exc, "code", -1), f"request set-up failed: {exc}")
        job.bytes = need
        job.t_setup = t_setup
        if small:
            self.stream_setup.synchronize()
            slot = self.free_slots.pop()
            wb = int(_capi.lib().dfx_batch_workspace_bytes(st.ndofs, 1 if self.mode == "mixed" else 0))
            job.work = torch.empty(wb, dtype=torch.uint8, device="cuda")
            sysd = _capi.BatchSystem(
                None if job.op32 is None else job.op32.handle.value, job.op64.handle.value,
                job.bp.data_ptr(), job.xp.data_ptr(), job.dp.data_ptr(), job.work.data_ptr(),
                self.rtol, self.delta, 100000, 1 if self.mode == "mixed" else 0)
            _capi.check(_capi.lib().dfx_batch_set(self.batch, slot, C.byref(sysd),
                                                  _stream_ptr(self.stream_setup)))
            job.slot = slot
            self.active[slot] = job
        else:
            self.stream_setup.synchronize()
            job.t_ready = time.perf_counter()
            self.large_q.put(job)
        return job

    def _release(self, job: Job):
        if not self.retain_systems:
            job.release_device()
        with self.lock:
            self.used -= job.bytes
            job.st.users -= 1
            if job.slot is not None:
                self.free_slots.append(job.slot)
            self.finished.append(job)

    # ------------------------------------------------------------ solving
    def _worker(self):
        stream = torch.cuda.Stream()
        # Whole-GPU solves run concurrently from several workers: the
        # four-kernel FP32 iteration, not the fused cooperative one, which
        # holds every SM while it runs (measured: 38.3 solves/s against
        # 33.1 on the 64-request sample).
        _capi.check(_capi.lib().dfx_set_cg_fused_update(0))
        while True:
            job = self.large_q.get()
            if job is None:
                return
            try:
                self._solve_large(job, stream)
            except Exception as exc:  # a failed request must still leave the loop
                job.t_done = time.perf_counter()
                job.status = getattr(exc, "code", -1)
                job.error = str(exc)
                self._release(job)

    def _solve_large(self, job, stream):
        n = job.st.ndofs
        job.t_solve = time.perf_counter()
        with torch.cuda.stream(stream):
            if self.mode == "mixed":
                wb = int(_capi.lib().dfx_ir_workspace_bytes(n))
                work = torch.empty(wb, dtype=torch.uint8, device="cuda")
                info = _capi.IrInfo()
                x = torch.zeros_like(job.b)
                _capi.check(_capi.lib().dfx_ir_solve(
                    job.op64.handle, job.op32.handle, la._ptr(job.b), la._ptr(x),
                    la._ptr(job.dinv), self.rtol, self.delta, 200, 100000, 20,
                    _capi.IR_RELIABLE, la._ptr(work), wb, C.byref(info), _stream_ptr(stream)))
                job.iterations = info.inner_iterations
            else:
                wb = int(_capi.lib().dfx_cg_op_workspace_bytes(n))
                work = torch.empty(wb, dtype=torch.uint8, device="cuda")
                info = _capi.CgInfo()
                x = torch.zeros_like(job.b)
                _capi.check(_capi.lib().dfx_cg_solve_op(
                    job.op64.handle, la._ptr(job.b), la._ptr(x), la._ptr(job.dinv),
                    self.rtol, 100000, 20, la._ptr(work), wb, C.byref(info),
                    _stream_ptr(stream)))
                job.iterations = info.iterations
            job.x = x.cpu()
            stream.synchronize()
        job.t_done = time.perf_counter()
        job.status = info.status
        self._release(job)

    def step(self) -> int:
        """One batched launch; retires finished systems. Returns #active."""
        if not self.active:
            return 0
        cnt = C.c_int32(0)
        _capi.check(_capi.lib().dfx_batch_step(self.batch, self.quantum, C.byref(cnt),
                                               _stream_ptr(self.stream_batch)))
        now = time.perf_counter()
        for slot in list(self.active):
            done = C.c_int32(0)
            rep = C.c_int32(0)
            info = _capi.CgInfo()
            _capi.lib().dfx_batch_info(self.batch, slot, C.byref(info), C.byref(done),
                                       C.byref(rep))
            if done.value:
                job = self.active.pop(slot)
                _capi.lib().dfx_batch_clear(self.batch, slot)
                with torch.cuda.stream(self.stream_batch):
                    job.x = job.solution().cpu()
                job.t_done = now
                job.status = info.status
                job.iterations = info.iterations
                self._release(job)
        return len(self.active)

    def run(self, requests: list[Request], max_wall_s: float = 600.0) -> dict:
        """Serve a timed stream (arrival times relative to the start). Stops
        with an error after max_wall_s seconds."""
        pending = collections.deque(sorted(requests, key=lambda r: r.arrival))
        total = len(pending)
        self.finished = []
        t0 = time.perf_counter()
        waiting: collections.deque = collections.deque()
        arrivals = {}
        while len(self.finished) < total:
            now = time.perf_counter() - t0
            if now > max_wall_s:
                raise RuntimeError(f"serving stream not finished after {max_wall_s} s "
                                   f"({len(self.finished)} of {total} done)")
            while pending and pending[0].arrival <= now:
                r = pending.popleft()
                arrivals[r.rid] = t0 + r.arrival
                err = request_error(r)
                if err is None:
                    waiting.append(r)
                else:
                    self._reject(r, _capi.DFX_ERR_INVALID, err)
            while waiting:
                job = self.admit(waiting[0])
                if job is None:
                    break
                waiting.popleft()
            if self.active:
                self.step()
            elif pending and not waiting:
                time.sleep(max(0.0, min(0.002, pending[0].arrival - (time.perf_counter() - t0))))
            else:
                time.sleep(0.0005)
        wall = time.perf_counter() - t0
        served = [j for j in self.finished if not isinstance(j, Rejected)]
        lat = np.array([j.t_done - arrivals[j.req.rid] for j in served])

        def ms(v):
            return float(v * 1e3) if len(lat) else None

        return {"mode": self.mode, "requests": total, "wall_s": wall,
                "solves_per_s": len(served) / wall,
                "p50_ms": ms(np.percentile(lat, 50) if len(lat) else 0.0),
                "p99_ms": ms(np.percentile(lat, 99) if len(lat) else 0.0),
                "mean_ms": ms(lat.mean() if len(lat) else 0.0),
                "dofs_per_s": float(sum(j.st.ndofs for j in served) / wall),
                "failed": [j.req.rid for j in self.finished if j.status != 0],
                "rejected": {j.req.rid: j.error for j in self.finished
                             if isinstance(j, Rejected)}}

    def close(self):
        for _ in self.workers:
            self.large_q.put(None)
        for w in self.workers:
            w.join(timeout=30)
        _capi.lib().dfx_batch_destroy(self.batch)
        self.batch = None
        # Drop this server's hold on its structures and finished requests,
        # so that a cache clear returns their memory.
        self.structures.clear()
        self.active.clear()
        self.finished = []
        self.used = 0
        gc.collect()
        torch.cuda.empty_cache()
        _capi.check(_capi.lib().dfx_operator_pool_trim())


def serve(requests, mode="mixed", max_wall_s: float = 600.0, **kw) -> tuple[dict, list[Job]]:
    srv = Server(mode=mode, **kw)
    try:
        srv.prewarm(requests)
        stats = srv.run(requests, max_wall_s=max_wall_s)
        return stats, list(srv.finished)
    finally:
        srv.close()


if __name__ == "__main__":
    import argparse
    import json

    p = argparse.ArgumentParser(description="serving-loop measurement (one GPU)")
    p.add_argument("--requests", type=int, default=200)
    p.add_argument("--rates", type=float, nargs="+", default=[100.0, 1000.0])
    p.add_argument("--nmin", type=int, default=8)
    p.add_argument("--nmax", type=int, default=96)
    p.add_argument("--budget-gb", type=float, default=64.0)
    args = p.parse_args()
    for rate in args.rates:
        reqs = make_requests(args.requests, rate, seed=1, n_range=(args.nmin, args.nmax))
        for mode in ("fp64", "mixed"):
            stats, _ = serve(reqs, mode=mode, hbm_budget=args.budget_gb * 1e9)
            stats["rate"] = rate
            print(json.dumps(stats), flush=True)
