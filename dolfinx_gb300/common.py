"""Timing tools: the ``dolfinx.common`` timing API (python/dolfinx/common.py:
58-187) over the library's process-wide table of named timings.

- ``Timer``: a wall-clock timer that registers its time under a task name
  when flushed, stopped by a ``with`` block, or collected while running
  (common/Timer.h:38-141);
- ``timing(task)``: (repetitions, total wall time) of a task;
- ``timings()``: every task, in byte-wise name order;
- ``list_timings(comm, reduction)``: print the summary table of
  TimeLogger::list_timings (common/TimeLogger.cpp:42-53), reduced over
  ranks when ``comm`` is a ``torch.distributed`` process group;
- ``timed(task)``: a decorator that times each call.

The library's host set-up registers here under the reference's task names
("Build BoxMesh (tetrahedra)", "Reverse Cuthill-McKee ordering",
"Dofmap builder: build dofmap data", "Build sparsity", ...). Kernels run
asynchronously: a ``Timer`` around a device call measures the host call
only, unless the block synchronises the stream.
"""

from __future__ import annotations

import ctypes as C
import datetime
import enum
import functools
import time
import typing
from collections.abc import Callable

from . import _capi
from . import log as _log

__all__ = ["Reduction", "Timer", "list_timings", "timed", "timing", "timing_table", "timings"]

_TITLE = "Summary of timings (s)"


class Reduction(enum.IntEnum):
    """Reduction of a timing table over ranks (Table::Reduction,
    common/Table.h:33-38)."""

    average = 0
    max = 1
    min = 2


def _record(task: str, seconds: float) -> None:
    _capi.check(_capi.lib().dfx_timing_record(task.encode(), float(seconds)))
    _log.logger.debug("Elapsed time: %s (%s)", float(seconds), task)


def timing(task: str) -> tuple[int, datetime.timedelta]:
    """(number of times logged, total wall time) of ``task`` in this process.
    Raises ``DfxError`` ('No timings registered for task "<task>".') when the
    task has none."""
    n, t = C.c_int32(0), C.c_double(0.0)
    _capi.check(_capi.lib().dfx_timing(task.encode(), C.byref(n), C.byref(t)))
    return n.value, datetime.timedelta(seconds=t.value)


def _raw_timings() -> list[tuple[str, int, float]]:
    L = _capi.lib()
    num = C.c_int32(0)
    _capi.check(L.dfx_timing_num_tasks(C.byref(num)))
    out = []
    cap = 256
    for i in range(num.value):
        while True:
            buf = C.create_string_buffer(cap)
            ln, n, t = C.c_int32(0), C.c_int32(0), C.c_double(0.0)
            _capi.check(L.dfx_timing_task(i, buf, cap, C.byref(ln), C.byref(n), C.byref(t)))
            if ln.value < cap:
                break
            cap = ln.value + 1
        out.append((buf.raw[: ln.value].decode(), n.value, t.value))
    return out


def timings() -> dict[str, tuple[int, datetime.timedelta]]:
    """Every task: name -> (repetitions, total wall time), in byte-wise name
    order (dolfinx::timings, common/timing.h:42-46)."""
    return {k: (n, datetime.timedelta(seconds=t)) for k, n, t in _raw_timings()}


def clear_timings() -> None:
    """Forget every timing of this process."""
    _capi.check(_capi.lib().dfx_timing_clear())


# ---------------------------------------------------------------- the table
# A table of rows x columns whose cells are int or float (the reference's
# Table, common/Table.cpp), enough of it for the timing summary: rows and
# columns in first-set order, ints printed as "%d", floats as "%f".


class _Table:
    def __init__(self, title: str):
        self.title = title
        self.rows: list[str] = []
        self.cols: list[str] = []
        self.values: dict[tuple[str, str], int | float] = {}

    def set(self, row: str, col: str, value) -> None:
        if row not in self.rows:
            self.rows.append(row)
        if col not in self.cols:
            self.cols.append(col)
        self.values[(row, col)] = value

    def _cell(self, row: str, col: str) -> str:
        try:
            v = self.values[(row, col)]
        except KeyError:
            raise RuntimeError(f'Missing table value for entry ("{row}", "{col}")') from None
        return str(v) if isinstance(v, int) else "%f" % v

    def str(self) -> str:
        """The title and row names left-justified, the columns right-justified
        in the width of their longest entry, separated by two spaces; a
        dashed rule under the header. Empty when there are no rows."""
        cells = [[self._cell(r, c) for c in self.cols] for r in self.rows]
        if not cells:
            return ""
        w0 = max([len(self.title)] + [len(r) for r in self.rows])
        w = [max([len(c)] + [len(cells[i][j]) for i in range(len(self.rows))])
             for j, c in enumerate(self.cols)]
        width = 2 * (len(w) + 1) + 1 + w0 + sum(w)
        lines = [f"{self.title:<{w0}}  |" + "".join(f"  {c:>{wj}}" for c, wj in zip(self.cols, w)),
                 "-" * width]
        for r, row in zip(self.rows, cells):
            lines.append(f"{r:<{w0}}  |" + "".join(f"  {v:>{wj}}" for v, wj in zip(row, w)))
        return "\n".join(lines)


def _local_table() -> _Table:
    """TimeLogger::timing_table (common/TimeLogger.cpp:55-69)."""
    t = _Table(_TITLE)
    for task, n, total in _raw_timings():
        t.set(task, "reps", n)
        t.set(task, "avg", total / n)
        t.set(task, "tot", total)
    return t


_PREFIX = {Reduction.average: "[MPI_AVG] ", Reduction.max: "[MPI_MAX] ",
           Reduction.min: "[MPI_MIN] "}


def _reduce(t: _Table, comm, reduction: Reduction) -> _Table:
    """Table::reduce (common/Table.cpp:71-199): the float cells reduced over
    the ranks of ``comm`` onto rank 0; the int cells (repetitions) are rank
    0's own; other ranks get an empty table."""
    reduction = Reduction(reduction)
    title = _PREFIX[reduction] + t.title
    import torch.distributed as dist

    size = 1 if comm is None else dist.get_world_size(comm)
    if size == 1:
        out = _Table(title)
        out.rows, out.cols, out.values = list(t.rows), list(t.cols), dict(t.values)
        return out
    mine = [(k, v) for k, v in t.values.items() if isinstance(v, float)]
    every = [None] * size
    dist.all_gather_object(every, mine, group=comm)
    if dist.get_rank(comm) > 0:
        return _Table(title)
    op = {Reduction.average: lambda y, x: y + x, Reduction.max: max, Reduction.min: min}[reduction]
    acc: dict[tuple[str, str], float] = {}
    for part in every:
        for k, v in part:
            acc[k] = op(acc[k], v) if k in acc else v
    if reduction == Reduction.average:
        acc = {k: v * (1.0 / size) for k, v in acc.items()}
    out = _Table(title)
    for k in sorted(t.values):
        if isinstance(t.values[k], int):
            out.set(k[0], k[1], t.values[k])
    for k in sorted(acc):
        out.set(k[0], k[1], acc[k])
    return out


def timing_table(comm=None, reduction: Reduction = Reduction.max) -> str:
    """The summary that ``list_timings`` prints, as a string (without the
    leading and trailing newline)."""
    return _reduce(_local_table(), comm, reduction).str()


def list_timings(comm=None, reduction: Reduction = Reduction.max) -> None:
    """Print a summary of all Timer measurements (on rank 0 of ``comm``; the
    maximum over ranks by default). ``comm``: None for this process alone,
    or a ``torch.distributed`` process group."""
    s = timing_table(comm, reduction)
    import torch.distributed as dist

    if comm is None or dist.get_rank(comm) == 0:
        print("\n" + s)


class Timer:
    """A timer for timing sections of code (python/dolfinx/common.py:84-172).

    With a ``with`` block the timer is (re)started on entry, and stopped and
    flushed on exit::

        with Timer("Some costly operation"):
            costly_call()
        count, total = timing("Some costly operation")

    It can also be driven explicitly: ``start`` resets and starts, ``stop``
    returns the elapsed time, ``resume`` continues a stopped timer, and
    ``flush`` registers a stopped, named timer's time once. A named timer
    that is still running when it is collected registers its time then.
    A new timer is already running.
    """

    def __init__(self, name: str | None = None):
        self._task = name
        self._acc = 0.0
        self._t0: float | None = time.perf_counter()

    def __enter__(self) -> typing.Self:
        self.start()
        return self

    def __exit__(self, *args: object) -> None:
        self.stop()
        self.flush()

    def __del__(self):
        if getattr(self, "_t0", None) is not None and self._task is not None:
            try:
                _record(self._task, self._acc + time.perf_counter() - self._t0)
            except Exception:
                pass

    def start(self) -> None:
        """Reset elapsed time and (re-)start timer."""
        self._acc = 0.0
        self._t0 = time.perf_counter()

    def stop(self) -> datetime.timedelta:
        """Stop timer and return elapsed time."""
        if self._t0 is not None:
            self._acc += time.perf_counter() - self._t0
            self._t0 = None
        return datetime.timedelta(seconds=self._acc)

    def resume(self) -> None:
        """Resume a stopped timer (no effect on a running one)."""
        if self._t0 is None:
            self._t0 = time.perf_counter()

    def elapsed(self) -> datetime.timedelta:
        """Elapsed time: the accumulated time, plus the current run if the
        timer is running."""
        t = self._acc
        if self._t0 is not None:
            t += time.perf_counter() - self._t0
        return datetime.timedelta(seconds=t)

    def flush(self) -> None:
        """Register the time under the timer's name. The timer must be
        stopped; a timer is flushed once, later calls do nothing."""
        if self._t0 is not None:
            raise RuntimeError("Timer must be stopped before flushing.")
        if self._task is not None:
            _record(self._task, self._acc)
            self._task = None


def timed(task: str) -> Callable:
    """Decorator that times each call of a function under ``task``."""

    def decorator(func: Callable) -> Callable:
        @functools.wraps(func)
        def wrapper(*args: typing.Any, **kwargs: typing.Any) -> typing.Any:
            with Timer(task):
                return func(*args, **kwargs)

        return wrapper

    return decorator
