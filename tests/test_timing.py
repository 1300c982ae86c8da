"""Timing tools (the dolfinx.common timing API): Timer semantics, the host
set-up's task names, the summary table against the reference's own
TimeLogger and Table (compiled from its sources), and the reduction of the
table over two gloo ranks."""

import datetime
import multiprocessing as mp
import os
import socket
import subprocess
import sys
import time

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture
def common(capi):
    from dolfinx_gb300 import common as cm

    cm.clear_timings()
    yield cm
    cm.clear_timings()


def test_timer_start_stop_resume_flush(common):
    t = common.Timer("task A")
    time.sleep(0.01)
    e1 = t.stop()
    assert isinstance(e1, datetime.timedelta) and e1.total_seconds() >= 0.01
    assert t.elapsed() == e1  # stopped: elapsed does not grow
    time.sleep(0.005)
    assert t.stop() == e1  # stopping twice changes nothing
    t.resume()
    time.sleep(0.01)
    with pytest.raises(RuntimeError, match="Timer must be stopped before flushing."):
        t.flush()
    e2 = t.stop()
    assert e2.total_seconds() >= e1.total_seconds() + 0.01
    t.flush()
    t.flush()  # a timer flushes once
    n, tot = common.timing("task A")
    assert n == 1 and tot == e2
    t.start()  # reset: accumulated time starts again from zero
    assert t.elapsed() < e2


def test_with_block_and_decorator_accumulate(common):
    for _ in range(3):
        with common.Timer("block") as t:
            time.sleep(0.002)
        assert t.elapsed().total_seconds() >= 0.002

    @common.timed("decorated")
    def f(a, b=1):
        """doc"""
        return a + b

    assert f(2, b=3) == 5 and f.__name__ == "f" and f.__doc__ == "doc"
    assert common.timing("block")[0] == 3
    assert common.timing("block")[1].total_seconds() >= 0.006
    assert common.timing("decorated")[0] == 1
    with common.Timer() as anon:  # unnamed: nothing registered
        pass
    assert anon.elapsed().total_seconds() >= 0
    assert list(common.timings()) == ["block", "decorated"]


def test_running_named_timer_registers_when_collected(common):
    t = common.Timer("collected")
    del t
    assert common.timing("collected")[0] == 1
    t = common.Timer("stopped, not flushed")
    t.stop()
    del t
    assert "stopped, not flushed" not in common.timings()


def test_unknown_task_raises(common, capi):
    with pytest.raises(capi.DfxError, match='No timings registered for task "nothing".'):
        common.timing("nothing")


def test_host_setup_registers_reference_task_names(common):
    from dolfinx_gb300 import fem, mesh

    m = mesh.create_unit_cube(4, 3, 2)
    V = fem.functionspace(m, ("Lagrange", 2), device="cpu")
    V.sparsity()
    got = {k: n for k, (n, t) in common.timings().items()}
    # the pseudo-peripheral root search runs two or more level structures
    assert got.pop("Graph: create_level_structure") >= 2
    dual = "Compute local part of mesh dual graph"
    stages = {f"{dual}: {s}": 1 for s in ("sort", "adjacency")}
    assert got == {"Build BoxMesh (tetrahedra)": 1, dual: 1, **stages,
                   "Reverse Cuthill-McKee ordering": 1, "Dofmap builder: build dofmap data": 1,
                   "Dofmap builder: compute dof reordering map": 1, "Build sparsity": 2}
    assert all(t.total_seconds() >= 0 for n, t in common.timings().values())
    mesh.create_box(((0, 0, 0), (1, 1, 1)), (2, 2, 2), reorder=False)
    got = {k: n for k, (n, t) in common.timings().items()}
    assert got["Build BoxMesh (tetrahedra)"] == 2 and got["Reverse Cuthill-McKee ordering"] == 1


def test_long_task_names_round_trip(common):
    name = "x" * 700 + " (long)"
    common.Timer(name).stop()
    t = common.Timer(name)
    t.stop()
    t.flush()
    assert list(common.timings()) == [name]


def test_empty_table_prints_blank_lines(common, capsys):
    assert common.timing_table() == ""
    common.list_timings()
    assert capsys.readouterr().out == "\n\n"


_PIN_SCRIPT = r"""
import sys
sys.path.insert(0, sys.argv[1])
from dolfinx_gb300 import common
from oracle import oracle as O

out = {}
for r in (0, 1, 2):
    out[("empty", r)] = (common.timing_table(None, r), O.ref_timing_table(r))
# The same repetitions into both tables: equal sums in the same order.
seq = [("Build sparsity", 0.1), ("Build sparsity", 0.2), ("Build sparsity", 0.3),
       ("[Assemble Matrix]", 1e-7), ("a", 12345.678901234), ("Zebra task", 2.5),
       ("Zebra task", 1e-9), ("A much longer task name than the table title", 0.0),
       ("[Apply lifting]", 0.04999999999), ("SparsityPattern::finalize", 3.0)]
for task, s in seq:
    common._record(task, s)
    O.ref_timing_record(task, s)
for r in (0, 1, 2):
    out[("full", r)] = (common.timing_table(None, r), O.ref_timing_table(r))
bad = [k for k, (a, b) in out.items() if a != b]
for k in bad:
    print(k, repr(out[k][0]), repr(out[k][1]), sep="\n")
print("rows", len(out[("full", 1)][0].splitlines()))
sys.exit(1 if bad else 0)
"""


def test_summary_table_matches_reference(capi, oracle, tmp_path):
    """Against the reference's TimeLogger::timing_table and Table::reduce /
    Table::str (common/TimeLogger.cpp, common/Table.cpp compiled from its
    sources, one rank), in a fresh process so both tables start empty."""
    if oracle.ref_la() is None:
        pytest.skip("the reference's la/common sources were not built here")
    script = tmp_path / "pin.py"
    script.write_text(_PIN_SCRIPT)
    p = subprocess.run([sys.executable, str(script), ROOT], capture_output=True, text=True,
                       timeout=120)
    assert p.returncode == 0, p.stdout + p.stderr
    assert "rows 9" in p.stdout  # header, rule, 7 tasks


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist

    from dolfinx_gb300 import common

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        common.clear_timings()
        # rank 0: 2 x 1 s; rank 1: 3 x 2 s (reps differ: rank 0's are shown)
        for _ in range(2 + rank):
            common._record("solve", 1.0 + rank)
        common._record("setup", 4.0 - 3.0 * rank)
        res = {r: common.timing_table(dist.group.WORLD, r) for r in common.Reduction}
        if rank == 1:
            common._record("only on rank 1", 1.0)
        try:
            common.timing_table(dist.group.WORLD, common.Reduction.max)
            res["missing"] = None
        except RuntimeError as e:
            res["missing"] = str(e)
        q.put((rank, {str(k): v for k, v in res.items()}))
    finally:
        dist.destroy_process_group()


def test_table_reduced_over_two_gloo_ranks():
    """Table::reduce over two ranks: float cells (avg, tot) reduced onto rank
    0, repetitions are rank 0's, other ranks get an empty table; a task that
    rank 0 never timed has no repetitions and the table cannot be printed
    (the reference's 'Missing table value' error)."""
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=180) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert all(v in ("", None) for k, v in out[1].items())
    r0 = out[0]

    def row(table, task):
        line = next(s for s in table.splitlines() if s.startswith(task + " "))
        return line.split("|")[1].split()

    mx, mn, av = r0[str(1)], r0[str(2)], r0[str(0)]
    assert mx.startswith("[MPI_MAX] Summary of timings (s)")
    assert mn.startswith("[MPI_MIN] ") and av.startswith("[MPI_AVG] ")
    # solve: rank 0 avg 1, tot 2; rank 1 avg 2, tot 6
    assert row(mx, "solve") == ["2", "2.000000", "6.000000"]
    assert row(mn, "solve") == ["2", "1.000000", "2.000000"]
    assert row(av, "solve") == ["2", "1.500000", "4.000000"]
    # setup: rank 0 4 s, rank 1 1 s
    assert row(mx, "setup") == ["1", "4.000000", "4.000000"]
    assert row(av, "setup") == ["1", "2.500000", "2.500000"]
    assert [s.split("|")[0].strip() for s in mx.splitlines()[2:]] == ["setup", "solve"]
    assert r0["missing"] == 'Missing table value for entry ("only on rank 1", "reps")'
