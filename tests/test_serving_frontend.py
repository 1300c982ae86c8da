"""Failure handling of the serving front-end, on the host (no GPU): a
malformed request is refused alone, a request larger than the whole HBM
budget is refused instead of waiting forever, idle structures are evicted
to make room, and a request whose set-up fails is refused with its error
code and its memory returned. The server's device parts (structures, jobs,
streams) are stand-ins that record what the front-end does with them."""

import collections
import queue
import threading

import pytest


class _Structure:
    def __init__(self, n, degree, sizes):
        self.n, self.degree = n, degree
        self.bytes, need = sizes[(n, degree)]
        self._need = need
        self.ndofs = 10 ** 9  # above batch_max_dofs: the whole-GPU path (a queue here)
        self.users = 0

    def request_bytes(self):
        return self._need


class _Stream:
    def synchronize(self):
        pass


@pytest.fixture
def front(capi, monkeypatch):
    """A Server whose structures and jobs are stand-ins; sizes[(n, degree)]
    = (structure bytes, request bytes)."""
    from dolfinx_gb300 import serving

    sizes, dropped, built = {}, [], []

    def cached_structure(n, degree):
        if (n, degree) not in sizes:
            raise capi.DfxError(capi.DFX_ERR_UNSUPPORTED, "no such structure")
        built.append((n, degree))
        return _Structure(n, degree, sizes)

    class _Job:
        def __init__(self, req, st, mode, stream, assembly):
            if req.seed == 13:
                raise capi.DfxError(capi.DFX_ERR_CUDA, "CUDA error cudaErrorMemoryAllocation")
            self.req, self.st, self.slot = req, st, None

    monkeypatch.setattr(serving, "cached_structure", cached_structure)
    monkeypatch.setattr(serving, "drop_structure", lambda n, d: dropped.append((n, d)))
    monkeypatch.setattr(serving, "Job", _Job)
    srv = serving.Server.__new__(serving.Server)
    srv.mode, srv.assembly, srv.budget, srv.capacity = "mixed", "atomic", 1000, 4
    srv.quantum, srv.batch_max_dofs, srv.rtol, srv.delta = 25, 65536, 1e-10, 0.03
    srv.structures = collections.OrderedDict()
    srv.used = 0
    srv.free_slots = list(range(4))
    srv.active = {}
    srv.lock = threading.Lock()
    srv.large_q = queue.Queue()
    srv.finished = []
    srv.stream_setup = _Stream()
    return serving, srv, sizes, dropped, built


@pytest.mark.parametrize("field,value,msg", [
    ("n", 0, "positive integer"), ("n", 2.5, "positive integer"), ("n", True, "positive"),
    ("n", 448, "too large for int32"), ("degree", 3, "degree 3 not supported"),
    ("k2", -1.0, ">= 0"), ("k2", float("nan"), "finite"), ("k2", "x", "a number"),
    ("seed", -1, "seed"), ("seed", 2 ** 64, "seed"), ("seed", 1.5, "seed"),
])
def test_malformed_requests_are_named(capi, field, value, msg):
    from dolfinx_gb300 import serving

    ok = serving.Request(0, 8, 2, 1.0, 7)
    assert serving.request_error(ok) is None
    assert serving.request_error(serving.Request(0, serving.MAX_N, 1, 0.0, 2 ** 64 - 1)) is None
    bad = serving.Request(**dict(ok.__dict__, **{field: value}))
    assert msg in serving.request_error(bad)


def test_run_refuses_malformed_requests_alone(front, capi):
    serving, srv, sizes, dropped, built = front
    reqs = [serving.Request(0, 0, 1, 0.0, 1), serving.Request(1, 8, 5, 0.0, 2, 0.001),
            serving.Request(2, 8, 1, -3.0, 3, 0.002)]
    stats = srv.run(reqs, max_wall_s=30.0)
    assert stats["failed"] == [0, 1, 2]
    assert sorted(stats["rejected"]) == [0, 1, 2]
    assert "degree 5" in stats["rejected"][1]
    assert all(j.status == capi.DFX_ERR_INVALID for j in srv.finished)
    assert stats["solves_per_s"] == 0 and stats["p50_ms"] is None and stats["dofs_per_s"] == 0
    assert built == []  # nothing was set up for them


def test_a_request_larger_than_the_budget_is_refused(front, capi):
    serving, srv, sizes, dropped, built = front
    sizes[(50, 2)] = (900, 200)  # 1,100 bytes > 1,000 even alone
    stats = srv.run([serving.Request(0, 50, 2, 1.0, 1)], max_wall_s=30.0)
    assert stats["failed"] == [0]
    assert "HBM budget" in stats["rejected"][0]
    assert srv.finished[0].status == capi.DFX_ERR_NO_MEMORY
    assert srv.used == 900 and dropped == []  # the structure fits, so it stays resident
    sizes[(60, 2)] = (1200, 10)  # the structure alone is over budget
    rej = srv.admit(serving.Request(1, 60, 2, 1.0, 1))
    assert isinstance(rej, serving.Rejected) and (60, 2) in dropped
    assert (60, 2) not in srv.structures and srv.used <= srv.budget


def test_idle_structures_are_evicted_to_make_room(front):
    serving, srv, sizes, dropped, built = front
    sizes[(8, 1)] = (300, 50)
    sizes[(9, 1)] = (300, 50)
    sizes[(10, 1)] = (300, 250)
    srv.structure(8, 1)
    srv.structure(9, 1)
    assert srv.used == 600
    job = srv.admit(serving.Request(0, 10, 1, 0.0, 1))  # 900 resident + 250 > 1,000
    assert isinstance(job, serving.Job)
    assert dropped == [(8, 1)]  # least recently used first, only as many as needed
    assert srv.used == 300 + 300 + 250 and job.st.users == 1
    assert srv.large_q.get_nowait() is job
    # a second request: 850 + 250 > 1,000, so the idle (9, 1) goes too
    assert isinstance(srv.admit(serving.Request(1, 10, 1, 0.0, 2)), serving.Job)
    assert dropped == [(8, 1), (9, 1)] and srv.used == 300 + 2 * 250
    # a third: 800 + 250 > 1,000 with nothing idle left, so it waits
    assert srv.admit(serving.Request(2, 10, 1, 0.0, 3)) is None
    assert srv.used == 800 and list(srv.structures) == [(10, 1)]


def test_a_failed_set_up_is_refused_and_returns_its_memory(front, capi):
    serving, srv, sizes, dropped, built = front
    sizes[(8, 1)] = (300, 50)
    rej = srv.admit(serving.Request(0, 8, 1, 0.0, 13))  # the stand-in job fails on seed 13
    assert isinstance(rej, serving.Rejected) and rej.status == capi.DFX_ERR_CUDA
    assert "cudaErrorMemoryAllocation" in rej.error
    assert srv.used == 300 and srv.structures[(8, 1)].users == 0
    rej = srv.admit(serving.Request(1, 7, 1, 0.0, 1))  # its structure cannot be built
    assert rej.status == capi.DFX_ERR_UNSUPPORTED and "structure set-up failed" in rej.error
    assert [j.req.rid for j in srv.finished] == [0, 1]


@pytest.mark.parametrize("kw,msg", [({"mode": "fp16"}, "mode"), ({"assembly": "serial"}, "assembly")])
def test_server_rejects_unknown_modes_before_device_work(capi, kw, msg):
    from dolfinx_gb300 import serving

    with pytest.raises(ValueError, match=msg):
        serving.Server(**kw)


def test_refusals_are_logged_as_warnings(front, capi, tmp_path):
    import logging
    import sys

    from dolfinx_gb300 import log as lg

    serving, srv, sizes, dropped, built = front
    path = tmp_path / "serving.log"
    lg.set_output_file(str(path))
    try:
        srv.run([serving.Request(5, 8, 7, 0.0, 1)], max_wall_s=30.0)
    finally:
        lg._install(logging.StreamHandler(sys.stderr))
    text = path.read_text()
    assert "[WARNING] request 5 refused (status 1): Lagrange degree 7 not supported" in text
