"""Serving path: batched persistent CG, continuous batching, admission.

The batched kernel solves each system in its own CTA, so a request's result
must not depend on which other requests share the launch (checked
bitwise). Its solutions must meet the FP64 stopping test like the
whole-GPU solvers."""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _residual(oracle, job):
    A = job.A
    rp = A.row_ptr.cpu().numpy()
    cols = A.cols.cpu().numpy()
    vals = A.vals.cpu().numpy()
    b = job.b.cpu().numpy()
    x = job.x.numpy()
    r = b - oracle.spmv(rp, cols, vals, x)
    return np.linalg.norm(r) / np.linalg.norm(b)


@pytest.mark.parametrize("mode", ["mixed", "fp64"])
def test_batched_cg_meets_fp64_stopping_test(cuda, oracle, capi, mode):
    from dolfinx_gb300 import serving

    reqs = [serving.Request(i, n, d, k2, 100 + i) for i, (n, d, k2) in
            enumerate([(6, 1, 0.0), (5, 2, 3.0), (9, 1, 7.5), (4, 2, 0.5)])]
    stats, jobs = serving.serve(reqs, mode=mode, hbm_budget=8e9, quantum=10,
                                retain_systems=True)
    assert stats["failed"] == []
    for job in jobs:
        assert job.slot is not None  # all went through the batched kernel
        assert _residual(oracle, job) < 1e-10 * 1.001


@pytest.mark.parametrize("assembly", ["coloured", "atomic"])
def test_result_is_the_same_alone_and_in_the_mix(cuda, capi, assembly):
    """Deterministic (coloured) assembly: bitwise identical. FP64-atomic
    assembly sums in a run-dependent order, so the matrices differ in the
    last bits; the solutions then agree to the solver tolerance."""
    from dolfinx_gb300 import serving

    target = serving.Request(0, 7, 2, 2.5, 777)
    others = [serving.Request(i, n, d, k2, 900 + i, 0.0) for i, (n, d, k2) in
              enumerate([(5, 1, 1.0), (8, 2, 0.0), (6, 2, 9.0), (10, 1, 4.0)], start=1)]
    _, alone = serving.serve([target], mode="mixed", hbm_budget=8e9, quantum=7,
                             assembly=assembly)
    _, mixed = serving.serve([target] + others, mode="mixed", hbm_budget=8e9, quantum=3,
                             assembly=assembly)
    x_alone = alone[0].x.numpy()
    x_mixed = [j for j in mixed if j.req.rid == 0][0].x.numpy()
    if assembly == "coloured":
        np.testing.assert_array_equal(x_alone, x_mixed)
    else:
        rel = np.linalg.norm(x_alone - x_mixed) / np.linalg.norm(x_alone)
        assert rel < 1e-9, rel


def test_whole_gpu_path_for_large_requests(cuda, oracle, capi):
    from dolfinx_gb300 import serving

    reqs = [serving.Request(0, 12, 2, 1.0, 5), serving.Request(1, 5, 1, 2.0, 6)]
    stats, jobs = serving.serve(reqs, mode="mixed", hbm_budget=8e9, batch_max_dofs=2000,
                                retain_systems=True)
    assert stats["failed"] == []
    big = [j for j in jobs if j.req.rid == 0][0]
    assert big.slot is None  # above batch_max_dofs: whole-GPU solver
    for job in jobs:
        assert _residual(oracle, job) < 1e-10 * 1.001


def test_admission_respects_the_hbm_budget(cuda, capi):
    from dolfinx_gb300 import serving

    srv = serving.Server(mode="mixed", hbm_budget=1e9)
    try:
        st = srv.structure(6, 1)
        need = st.request_bytes()
        srv.budget = srv.used + need - 1  # one byte short even alone: refused
        rej = srv.admit(serving.Request(0, 6, 1, 0.0, 1))
        assert isinstance(rej, serving.Rejected) and rej.status == capi.DFX_ERR_NO_MEMORY
        srv.budget = srv.used + need  # exactly enough for one
        job = srv.admit(serving.Request(1, 6, 1, 0.0, 1))
        assert isinstance(job, serving.Job)
        assert srv.admit(serving.Request(2, 6, 1, 0.0, 1)) is None  # waits for the first
    finally:
        srv.close()


def test_concurrent_whole_gpu_workers(cuda, oracle, capi):
    """Several large requests on two worker threads at once (each thread
    captures and replays its own CG graphs)."""
    from dolfinx_gb300 import serving

    reqs = [serving.Request(i, 9 + i % 3, 1 + i % 2, 0.5 * i, 40 + i, 0.0) for i in range(6)]
    for mode in ("mixed", "fp64"):
        stats, jobs = serving.serve(reqs, mode=mode, hbm_budget=8e9, batch_max_dofs=100,
                                    workers=2, retain_systems=True)
        assert stats["failed"] == []
        assert all(j.slot is None for j in jobs)
        for job in jobs:
            assert _residual(oracle, job) < 1e-10 * 1.001


def test_structure_counts_what_it_holds(cuda, capi):
    """A serving structure keeps the pattern only (its operators' values
    released, no CSR values) and its byte count is what its tensors and
    operators hold on the device."""
    from dolfinx_gb300 import serving

    st = serving.Structure(7, 2)
    assert st.A0 is None and st.asm.A is None
    ops = st.op64.device_bytes() + st.op32.device_bytes()
    slots = st.ops_slots()
    # structure arrays only: FP64 map + columns (8 B/slot), FP32 map + deltas (6 B/slot)
    assert ops >= 14 * slots and ops < 14 * slots + 64 * st.ndofs + (1 << 20)
    assert st.bytes == serving.device_bytes(st)
    assert st.bytes > ops + st.nnz * 4  # and the CSR pattern, slot map, dofmap, mesh
