"""The autotuner: every candidate launch shape computes the same result as
the oracle, the tuner picks one of the candidates, and the library's table
applies and forgets choices as documented."""

import ctypes as C

import numpy as np
import pytest
import torch

from gpu_util import assert_close, problem

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _fresh_table(capi):
    capi.check(capi.lib().dfx_tune_clear())
    yield
    capi.check(capi.lib().dfx_tune_clear())


def _cpb(capi, a, mode):
    v = C.c_int32(0)
    capi.check(capi.lib().dfx_get_cells_per_block(C.byref(a.cstruct()), mode, C.byref(v)))
    return v.value


@pytest.mark.parametrize("mode", ["atomic", "coloured"])
@pytest.mark.parametrize("kind,deg,k2", [("poisson", 1, 0.0), ("poisson", 2, 2.5),
                                         ("elasticity", 2, 0.0)])
def test_every_cells_per_block_matches_the_oracle(cuda, oracle, capi, kind, deg, k2, mode):
    from dolfinx_gb300 import fem

    bs = 3 if kind == "elasticity" else 1
    m, V, kappa, f, rp, cols = problem(oracle, (5, 4, 3), deg, seed=21, bs=bs)
    a = fem.poisson_form(V, kappa, k2=k2) if bs == 1 else fem.elasticity_form(V, kappa, 0.3)
    ref = oracle.assemble_matrix(0 if bs == 1 else 1, deg, m.cells, m.x, V.dofmap, rp, cols,
                                 kappa=kappa, k2=k2, nu=0.3)
    m_id = fem._mode(mode)
    assert _cpb(capi, a, m_id) == (4 if bs == 3 else 32)  # default
    for cpb in ((2, 4, 8) if bs == 3 else (16, 32, 64)):
        capi.check(capi.lib().dfx_set_cells_per_block(C.byref(a.cstruct()), m_id, cpb))
        assert _cpb(capi, a, m_id) == cpb
        A = fem.assemble_matrix(a, mode=mode)
        assert_close(A.vals.cpu().numpy(), ref)


def test_tuned_assembly_is_recorded_and_used(cuda, oracle, capi):
    from dolfinx_gb300 import autotune, fem

    m, V, kappa, f, rp, cols = problem(oracle, (8, 8, 8), 2, seed=22)
    a = fem.poisson_form(V, kappa)
    asm = fem.MatrixAssembler(a)
    asm.assemble()
    before = asm.A.vals.clone()
    res = autotune.tune_assembly(asm)
    assert res["cells_per_block"] in (16, 32, 64)
    assert all(t > 0 for t in res["ms"].values())
    assert torch.equal(asm.A.vals, before)  # the tuner wrote only its scratch
    assert _cpb(capi, a, 0) == res["cells_per_block"]
    A = fem.assemble_matrix(a)
    ref = oracle.assemble_matrix(0, 2, m.cells, m.x, V.dofmap, rp, cols, kappa=kappa)
    assert_close(A.vals.cpu().numpy(), ref)
    autotune.clear()
    assert _cpb(capi, a, 0) == 32


def test_invalid_choices_are_refused(cuda, oracle, capi):
    from dolfinx_gb300 import fem

    m, V, kappa, f, rp, cols = problem(oracle, (2, 2, 2), 1, seed=23)
    a = fem.poisson_form(V, kappa)
    assert capi.lib().dfx_set_cells_per_block(C.byref(a.cstruct()), 0, 48) == capi.DFX_ERR_INVALID
    A = fem.assemble_matrix(a)
    assert capi.lib().dfx_set_spmv_lanes(C.byref(A.csr()), 3) == capi.DFX_ERR_INVALID


def test_every_row_split_matches_the_oracle(cuda, oracle, capi):
    from dolfinx_gb300 import autotune, fem, la

    m, V, kappa, f, rp, cols = problem(oracle, (6, 5, 4), 2, seed=24)
    A = fem.assemble_matrix(fem.poisson_form(V, kappa, k2=1.0))  # SPD without BCs
    vals = A.vals.cpu().numpy()
    x = np.random.default_rng(25).standard_normal(A.nrows)
    ref = oracle.spmv(rp, cols, vals, x)
    xd = torch.from_numpy(x).cuda()
    for lanes in (4, 8, 16, 32):
        capi.check(capi.lib().dfx_set_spmv_lanes(C.byref(A.csr()), lanes))
        got = C.c_int32(0)
        capi.check(capi.lib().dfx_get_spmv_lanes(C.byref(A.csr()), C.byref(got)))
        assert got.value == lanes
        y = A.matvec(xd)
        assert_close(y.cpu().numpy(), ref, rtol=1e-13)
    res = autotune.tune_spmv(A)
    assert res["lanes_per_row"] in (4, 8, 16, 32)
    got = C.c_int32(0)
    capi.check(capi.lib().dfx_get_spmv_lanes(C.byref(A.csr()), C.byref(got)))
    assert got.value == res["lanes_per_row"]
    # the CSR CG uses the tuned split and still meets its stopping test
    b = torch.from_numpy(np.abs(x)).cuda()
    xs, r = la.cg(A, b, rtol=1e-10)
    res_vec = b.cpu().numpy() - oracle.spmv(rp, cols, vals, xs.cpu().numpy())
    assert np.linalg.norm(res_vec) / np.linalg.norm(b.cpu().numpy()) < 1e-10 * 1.0001


def test_tuned_sigma_gives_a_correct_operator(cuda, oracle, capi):
    from dolfinx_gb300 import autotune, fem, la

    m, V, kappa, f, rp, cols = problem(oracle, (9, 8, 7), 2, seed=26)
    A = fem.assemble_matrix(fem.poisson_form(V, kappa))
    res = autotune.tune_sigma(A, candidates=(32, 256, 1024), reps=3)
    assert res["sigma"] in (32, 256, 1024)
    op = la.SellOperator(A, torch.float64, res["sigma"])
    x = np.random.default_rng(27).standard_normal(A.nrows)
    ref = oracle.spmv(rp, cols, A.vals.cpu().numpy(), x)
    assert_close(op.apply(torch.from_numpy(x).cuda()).cpu().numpy(), ref, rtol=1e-13)


def test_fp32_spmv_chunks_are_bitwise_equal(cuda, oracle, capi):
    """The load chunk of the FP32 sliced-ELL SpMV changes only how many
    loads are in flight: the products of chunks 2, 4 and 8 are bitwise
    equal, and tune_chunk keeps one of them on the operator."""
    from dolfinx_gb300 import autotune, fem, la

    from gpu_util import problem

    m, V, kappa, f, rp, cols = problem(oracle, (7, 6, 5), 2, seed=24)
    A = fem.assemble_matrix(fem.poisson_form(V, kappa))
    op = la.SellOperator(A, torch.float32, 256, compress_cols=True)
    x = torch.rand(V.num_dofs, dtype=torch.float32, device="cuda")
    outs = []
    for ch in (2, 4, 8):
        op.set_chunk(ch)
        outs.append(op.apply(x).clone())
    assert torch.equal(outs[0], outs[1]) and torch.equal(outs[1], outs[2])
    r = autotune.tune_chunk(op, reps=3)
    assert r["chunk"] in (2, 4, 8) and set(r["candidates"]) == {2, 4, 8}
    assert torch.equal(op.apply(x), outs[1])
    with pytest.raises(capi.DfxError):
        op.set_chunk(3)
