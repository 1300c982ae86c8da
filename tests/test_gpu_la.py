"""GPU parity: SpMV (FP64, FP32 values, 3x3 blocks), Jacobi diagonal,
inner product and CG against the oracle."""

import ctypes as C

import numpy as np
import pytest
import torch

from gpu_util import assert_close, problem

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("deg,bs", [(1, 1), (2, 1), (2, 3)])
@pytest.mark.parametrize("beta", [0.0, 1.0])
def test_spmv_f64(cuda, oracle, capi, deg, bs, beta):
    from dolfinx_gb300 import fem

    m, V, kappa, f, rp, cols = problem(oracle, (5, 6, 4), deg, bs=bs)
    a = fem.poisson_form(V, kappa) if bs == 1 else fem.elasticity_form(V, kappa)
    A = fem.assemble_matrix(a)
    vals = A.vals.cpu().numpy()
    rng = np.random.default_rng(11)
    x = rng.standard_normal(V.num_dofs)
    y0 = rng.standard_normal(V.num_dofs)
    xd = torch.from_numpy(x).cuda()
    yd = torch.from_numpy(y0.copy()).cuda()
    if beta == 1.0:
        A.mult(xd, yd)
        ref = oracle.spmv(rp, cols, vals, x, bs=bs, y=y0.copy())
    else:
        A.matvec(xd, yd)
        ref = oracle.spmv(rp, cols, vals, x, bs=bs)
    assert_close(yd.cpu().numpy(), ref, rtol=1e-13)


@pytest.mark.parametrize("bs", [1, 3])
def test_spmv_f32(cuda, oracle, capi, bs):
    from dolfinx_gb300 import fem

    m, V, kappa, f, rp, cols = problem(oracle, (4, 4, 4), 2, bs=bs)
    a = fem.poisson_form(V, kappa) if bs == 1 else fem.elasticity_form(V, kappa)
    A32 = fem.assemble_matrix(a).astype_float32()
    x = np.random.default_rng(3).standard_normal(V.num_dofs).astype(np.float32)
    y = A32.matvec(torch.from_numpy(x).cuda()).cpu().numpy()
    ref = oracle.spmv(rp, cols, A32.vals.cpu().numpy().astype(np.float64), x.astype(np.float64),
                      bs=bs)
    assert_close(y, ref, rtol=2e-6)


def test_inner_product(cuda, capi):
    from dolfinx_gb300 import la

    rng = np.random.default_rng(5)
    for n in [1, 1000, 1234567]:
        a = rng.standard_normal(n)
        b = rng.standard_normal(n)
        v = la.inner_product(torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda())
        assert abs(v - np.dot(a, b)) <= 1e-12 * np.abs(a * b).sum()


@pytest.mark.parametrize("deg", [1, 2])
def test_cg_poisson_pipeline(cuda, oracle, capi, deg):
    """The demo's full Poisson pipeline: assemble, lift, set_bc, Jacobi-CG; solution
    vs the oracle's CG on the oracle's system (rtol 1e-10)."""
    from dolfinx_gb300 import fem, la

    n = (8, 8, 8) if deg == 2 else (16, 16, 16)
    m, V, kappa, f, rp, cols = problem(oracle, n, deg, seed=12)
    X = V.tabulate_dof_coordinates()
    bnd = np.flatnonzero(np.isclose(X, 0).any(1) | np.isclose(X, 1).any(1)).astype(np.int32)
    bc = fem.dirichletbc(0.0, bnd, V)
    a = fem.poisson_form(V, kappa)
    A = fem.assemble_matrix(a, bcs=[bc])
    b = fem.assemble_vector(fem.source_form(V, f))
    fem.apply_lifting(b, [a], [[bc]])
    fem.set_bc(b, [bc])
    x, res = la.cg(A, b, rtol=1e-10)
    assert res.status == 0 and res.iterations > 0
    mk = np.zeros(V.num_nodes, np.int8)
    mk[bnd] = 1
    Ar = oracle.assemble_matrix(0, deg, m.cells, m.x, V.dofmap, rp, cols, kappa=kappa,
                                bc_markers=mk)
    oracle.set_diagonal(1, rp, cols, Ar, bnd)
    br = oracle.assemble_vector(0, deg, m.cells, m.x, V.dofmap, V.num_nodes, f=f)
    oracle.set_bc(br, bnd, np.zeros(V.num_nodes))
    assert_close(b.cpu().numpy(), br)
    diag = np.array([Ar[rp[i] + np.searchsorted(cols[rp[i]:rp[i + 1]], i)]
                     for i in range(V.num_nodes)])
    xr, it = oracle.cg(rp, cols, Ar, br, dinv=1.0 / diag, rtol=1e-10)
    assert it > 0
    assert abs(res.iterations - it) <= 2
    xs = x.cpu().numpy()
    rel = np.linalg.norm(xs - xr) / np.linalg.norm(xr)
    assert rel < 1e-8, rel
    # residual of the GPU solution in the oracle's system
    r = br - oracle.spmv(rp, cols, Ar, xs)
    assert np.linalg.norm(r) / np.linalg.norm(br) < 1e-9


def test_cg_elasticity_small(cuda, oracle, capi):
    from dolfinx_gb300 import fem, la

    m, V, E, f, rp, cols = problem(oracle, (4, 2, 2), 2, bs=3, seed=2)
    X = V.tabulate_dof_coordinates()
    clamp = np.flatnonzero(np.isclose(X[:, 0], 0)).astype(np.int32)
    bc = fem.dirichletbc(np.zeros(3), clamp, V)
    a = fem.elasticity_form(V, 1e3 * E, 0.3)
    A = fem.assemble_matrix(a, bcs=[bc])
    b = fem.assemble_vector(fem.body_force_form(V, (0, 0, -1)))
    fem.apply_lifting(b, [a], [[bc]])
    fem.set_bc(b, [bc])
    x, res = la.cg(A, b, rtol=1e-10)
    vals = A.vals.cpu().numpy()
    bh = b.cpu().numpy()
    r = bh - oracle.spmv(rp, cols, vals, x.cpu().numpy(), bs=3)
    assert np.linalg.norm(r) / np.linalg.norm(bh) < 1e-9


def test_cg_not_converged_reports(cuda, oracle, capi):
    from dolfinx_gb300 import fem, la

    m, V, kappa, f, rp, cols = problem(oracle, (6, 6, 6), 1)
    X = V.tabulate_dof_coordinates()
    bnd = np.flatnonzero(np.isclose(X, 0).any(1)).astype(np.int32)
    bc = fem.dirichletbc(0.0, bnd, V)
    A = fem.assemble_matrix(fem.poisson_form(V, kappa), bcs=[bc])
    b = fem.assemble_vector(fem.source_form(V, f))
    with pytest.raises(capi.DfxError, match="exceeded max iterations"):
        la.cg(A, b, rtol=1e-14, max_iters=3)


def test_nan_coefficient_reports_breakdown(cuda, oracle, capi):
    """An injected fault: one cell's kappa is NaN. The solves end with an
    error status (p.Ap or the residual is not finite) instead of returning
    a NaN solution; the iteration caps bound every loop."""
    from dolfinx_gb300 import fem, la

    m, V, kappa, f, rp, cols = problem(oracle, (6, 6, 6), 1, seed=31)
    kappa[m.num_cells // 2] = np.nan
    X = V.tabulate_dof_coordinates()
    bnd = np.flatnonzero(np.isclose(X, 0).any(1)).astype(np.int32)
    bc = fem.dirichletbc(0.0, bnd, V)
    A = fem.assemble_matrix(fem.poisson_form(V, kappa), bcs=[bc])
    b = fem.assemble_vector(fem.source_form(V, f))
    assert torch.isnan(A.vals).any() and torch.isfinite(b).all()
    with pytest.raises(capi.DfxError) as e:
        la.cg(A, b, rtol=1e-10, max_iters=500)
    assert e.value.code == capi.DFX_ERR_BREAKDOWN
    ir = la.IRSolver(A)
    res = ir.solve(b, torch.zeros_like(b), rtol=1e-10, max_outer=3, max_inner=200,
                   raise_on_fail=False)
    assert res.status in (capi.DFX_ERR_BREAKDOWN, capi.DFX_ERR_NOT_CONVERGED)


@pytest.mark.parametrize("sigma", [32, 256])
def test_sell_operator_f64(cuda, oracle, capi, sigma):
    from dolfinx_gb300 import fem, la

    m, V, kappa, f, rp, cols = problem(oracle, (6, 5, 7), 2, seed=21)
    A = fem.assemble_matrix(fem.poisson_form(V, kappa))
    op = la.SellOperator(A, torch.float64, sigma)
    inf = op.info()
    assert inf["slots"] % 32 == 0 and inf["padding"] >= 0
    x = np.random.default_rng(1).standard_normal(V.num_dofs)
    y = op.apply(torch.from_numpy(x).cuda()).cpu().numpy()
    ref = oracle.spmv(rp, cols, A.vals.cpu().numpy(), x)
    assert_close(y, ref, rtol=1e-13)
    # values refresh after re-assembly
    A.vals.mul_(2.0)
    op.update_values()
    y = op.apply(torch.from_numpy(x).cuda()).cpu().numpy()
    assert_close(y, 2 * ref, rtol=1e-13)


@pytest.mark.parametrize("compress", [False, True])
def test_sell_operator_f32(cuda, oracle, capi, compress):
    from dolfinx_gb300 import fem, la

    m, V, kappa, f, rp, cols = problem(oracle, (6, 5, 7), 2, seed=22)
    A = fem.assemble_matrix(fem.poisson_form(V, kappa))
    op = la.SellOperator(A, torch.float32, 256, compress_cols=compress)
    x = np.random.default_rng(2).standard_normal(V.num_dofs).astype(np.float32)
    y = op.apply(torch.from_numpy(x).cuda()).cpu().numpy()
    v32 = A.vals.cpu().numpy().astype(np.float32).astype(np.float64)
    ref = oracle.spmv(rp, cols, v32, x.astype(np.float64))
    assert_close(y, ref, rtol=2e-6)


@pytest.mark.parametrize("compress", [False, True])
def test_sell_operator_split_is_fp64_accurate(cuda, oracle, capi, compress):
    """The split operator (each value as two FP32 words, FP32-pipe products
    with error-free transformations) gives the FP64 product to ~1e-13 --
    FP64 accuracy, far from FP32's 1e-7 -- in both numberings, for n even
    and odd, and after a value refresh."""
    from dolfinx_gb300 import fem, la

    for shape in ((6, 5, 7), (5, 5, 4)):
        m, V, kappa, f, rp, cols = problem(oracle, shape, 2, seed=23)
        A = fem.assemble_matrix(fem.poisson_form(V, kappa))
        op = la.SellOperator(A, torch.float64, 256, compress_cols=compress, split=True)
        x = np.random.default_rng(3).standard_normal(V.num_dofs)
        y = op.apply(torch.from_numpy(x).cuda()).cpu().numpy()
        ref = oracle.spmv(rp, cols, A.vals.cpu().numpy(), x)
        assert_close(y, ref, rtol=1e-13)
        xp = op.to_operator(torch.from_numpy(x).cuda())
        yp = op.apply_renumbered(xp, torch.empty_like(xp))
        assert_close(op.from_operator(yp).cpu().numpy(), ref, rtol=1e-13)
        A.vals.mul_(3.0)
        op.update_values()
        y = op.apply(torch.from_numpy(x).cuda()).cpu().numpy()
        assert_close(y, 3 * ref, rtol=1e-13)


def test_split_operator_cg_matches_fp64(cuda, oracle, capi):
    """FP64 Jacobi-PCG on the split operator takes the FP64 operator's
    iteration count (within 1 %) and meets the stopping test in the oracle's
    FP64 SpMV, on a Poisson system and a clamped elasticity system."""
    from dolfinx_gb300 import fem, la

    A, b, rp, cols = _poisson_system(oracle, (10, 9, 8), 2, 31)
    systems = [(A, b, rp, cols, 1)]
    m, V, E, f, rpe, colse = problem(oracle, (8, 3, 3), 2, bs=3, seed=13)
    X = V.tabulate_dof_coordinates()
    clamp = np.flatnonzero(np.isclose(X[:, 0], 0)).astype(np.int32)
    bc = fem.dirichletbc(np.zeros(3), clamp, V)
    a = fem.elasticity_form(V, 1e3 * E, 0.3)
    Ae = fem.assemble_matrix(a, bcs=[bc])
    be = fem.RhsAssembler(fem.body_force_form(V, (0, 0, -1)), a, [bc]).assemble()
    S = Ae.expand_blocks()
    systems.append((S, be, S.row_ptr.cpu().numpy(), S.cols.cpu().numpy(), 1))
    for M, rhs, r_p, c_s, bs in systems:
        x64 = torch.zeros_like(rhs)
        r64 = la.OperatorCGSolver(M).solve(rhs, x64, rtol=1e-11)
        xs = torch.zeros_like(rhs)
        rs = la.OperatorCGSolver(M, split=True).solve(rhs, xs, rtol=1e-11)
        # CG's iteration count in finite precision moves by a few iterations
        # with the last bits of its products (the split rows round at
        # ~2^-44, FP64 rows at 2^-53): within 1 % (and at least 2).
        tol = max(2, int(0.01 * r64.iterations))
        assert rs.status == 0 and abs(rs.iterations - r64.iterations) <= tol, (rs, r64)
        bh = rhs.cpu().numpy()
        res = bh - oracle.spmv(r_p, c_s, M.vals.cpu().numpy(), xs.cpu().numpy(), bs=bs)
        # The stopping test reads the recursive residual. It drifts from the
        # true residual as the products' rounding (~2^-44 per row for the
        # split operator) accumulates over the iterations: on the clamped
        # elasticity system (~450 iterations) the true residual measured
        # 1.06e-11 at rtol 1e-11.
        assert np.linalg.norm(res) / np.linalg.norm(bh) < 1e-11 * 1.25
        assert (xs - x64).norm().item() / x64.norm().item() < 1e-9


@pytest.mark.parametrize("split", [False, True])
@pytest.mark.parametrize("sigma", [32, 4096])
def test_block_operator_matches_oracle(cuda, oracle, capi, split, sigma):
    """The 3x3-block operator of an elasticity matrix (one column per block,
    FP64 or split values) against the oracle's block SpMV, in both
    numberings, for block-row counts that are not multiples of 32, after a
    value refresh and through a share with other values."""
    from dolfinx_gb300 import fem, la

    for shape in ((5, 3, 4), (6, 4, 3)):
        m, V, E, f, rp, cols = problem(oracle, shape, 2, bs=3, seed=29)
        A = fem.assemble_matrix(fem.elasticity_form(V, 1e3 * E, 0.3))
        op = la.SellOperator(A, torch.float64, sigma, split=split)
        assert op.n == V.num_dofs and not op.compressed
        x = np.random.default_rng(5).standard_normal(V.num_dofs)
        # Row-wise against (|A| |x|)_i: elasticity rows cancel, so a bound
        # relative to the largest entry of y would not hold. FP64 rows of
        # ~81 entries are within (81 + 81) u of the oracle's; split rows
        # round at ~2^-44 of |A| |x|.
        tol = 2e-13 if split else 2e-14

        def check(y, M):
            v = M.vals.cpu().numpy()
            ref = oracle.spmv(rp, cols, v, x, bs=3)
            mag = oracle.spmv(rp, cols, np.abs(v), np.abs(x), bs=3)
            err = (np.abs(np.asarray(y) - ref) / np.maximum(mag, 1e-300)).max()
            assert err <= tol, f"row error {err:.3e} of |A||x| > {tol:.1e}"

        y0 = op.apply(torch.from_numpy(x).cuda())
        check(y0.cpu().numpy(), A)
        # 1, 2 and 4 block slots per round give the same bits
        for ch in (2, 4, 8):
            op.set_chunk(ch)
            assert torch.equal(op.apply(torch.from_numpy(x).cuda()), y0)
        xp = op.to_operator(torch.from_numpy(x).cuda())
        yp = op.apply_renumbered(xp, torch.empty_like(xp))
        check(op.from_operator(yp).cpu().numpy(), A)
        A2 = fem.assemble_matrix(fem.elasticity_form(V, 2e3 * E, 0.25))
        sh = op.share(A2)
        check(sh.apply(torch.from_numpy(x).cuda()).cpu().numpy(), A2)
        del sh
        A.vals.mul_(3.0)
        op.update_values()
        check(op.apply(torch.from_numpy(x).cuda()).cpu().numpy(), A)


@pytest.mark.parametrize("nb", [1, 31, 32, 33, 97])
def test_block_operator_edge_sizes(cuda, capi, nb):
    """3x3-block operators of random block CSR matrices (ragged rows of 1
    to 9 blocks, block-row counts around the 32-row slice) against a dense
    product in numpy, FP64 and split, for every slots-per-round choice;
    an empty bs 3 matrix gives an empty operator."""
    from dolfinx_gb300 import la

    rng = np.random.default_rng(nb)
    rows = []
    for i in range(nb):
        k = int(rng.integers(1, min(nb, 9) + 1))
        rows.append(np.unique(np.concatenate([[i], rng.choice(nb, k - 1, replace=True)]))
                    .astype(np.int64))
    rp = np.zeros(nb + 1, np.int64)
    rp[1:] = np.cumsum([r.size for r in rows])
    cols = np.concatenate(rows).astype(np.int32)
    vals = rng.standard_normal(9 * cols.size)
    dense = np.zeros((3 * nb, 3 * nb))
    for i, r in enumerate(rows):
        for j, c in enumerate(r):
            blk = vals[9 * (rp[i] + j): 9 * (rp[i] + j + 1)].reshape(3, 3)
            dense[3 * i:3 * i + 3, 3 * c:3 * c + 3] = blk
    A = la.MatrixCSR(torch.from_numpy(rp).cuda(), torch.from_numpy(cols).cuda(),
                     torch.from_numpy(vals).cuda(), 3)
    x = rng.standard_normal(3 * nb)
    ref = dense @ x
    mag = np.abs(dense) @ np.abs(x)
    for split in (False, True):
        op = la.SellOperator(A, torch.float64, 32, split=split)
        assert op.n == 3 * nb
        tol = 2e-13 if split else 2e-15 * 27
        for ch in (2, 4, 8):
            op.set_chunk(ch)
            y = op.apply(torch.from_numpy(x).cuda()).cpu().numpy()
            assert (np.abs(y - ref) / mag).max() <= tol

    E = la.MatrixCSR(torch.zeros(1, dtype=torch.int64, device="cuda"),
                     torch.zeros(0, dtype=torch.int32, device="cuda"),
                     torch.zeros(0, dtype=torch.float64, device="cuda"), 3)
    for split in (False, True):
        op = la.SellOperator(E, torch.float64, split=split)
        assert op.info()["slots"] == 0 and op.n == 0
        assert op.apply(torch.zeros(0, dtype=torch.float64, device="cuda")).numel() == 0


def test_block_operator_refuses_what_it_does_not_hold(cuda, capi):
    """3x3-block operators hold FP64 or split values with 32-bit columns,
    built on the host; refinement takes scalar operators."""
    from dolfinx_gb300 import la
    from dolfinx_gb300._capi import DfxError

    rp = torch.tensor([0, 1], dtype=torch.int64, device="cuda")
    A = la.MatrixCSR(rp, torch.zeros(1, dtype=torch.int32, device="cuda"),
                     torch.eye(3, dtype=torch.float64, device="cuda").flatten(), 3)
    with pytest.raises(DfxError, match="FP64 or split"):
        la.SellOperator(A, torch.float32)
    with pytest.raises(DfxError, match="32-bit block columns"):
        la.SellOperator(A, torch.float64, split=True, compress_cols=True)
    with pytest.raises(DfxError, match="built on the host"):
        la.SellOperator(A, torch.float64, build=1)


def test_block_operator_cg_matches_scalar(cuda, oracle, capi):
    """Jacobi-PCG on the 3x3-block operators (FP64 and split) of a clamped
    elasticity system takes the scalar FP64 operator's iteration count
    (within 1 %), meets the stopping test in the oracle's FP64 SpMV and
    reaches the same solution."""
    from dolfinx_gb300 import fem, la

    m, V, E, f, rpe, colse = problem(oracle, (8, 3, 3), 2, bs=3, seed=13)
    X = V.tabulate_dof_coordinates()
    clamp = np.flatnonzero(np.isclose(X[:, 0], 0)).astype(np.int32)
    bc = fem.dirichletbc(np.zeros(3), clamp, V)
    a = fem.elasticity_form(V, 1e3 * E, 0.3)
    Ae = fem.assemble_matrix(a, bcs=[bc])
    be = fem.RhsAssembler(fem.body_force_form(V, (0, 0, -1)), a, [bc]).assemble()
    S = Ae.expand_blocks()
    x64 = torch.zeros_like(be)
    r64 = la.OperatorCGSolver(S).solve(be, x64, rtol=1e-11)
    bh = be.cpu().numpy()
    for split in (False, True):
        solver = la.OperatorCGSolver(Ae, split=split)
        xb = torch.zeros_like(be)
        rb = solver.solve(be, xb, rtol=1e-11)
        tol = max(2, int(0.01 * r64.iterations))
        assert rb.status == 0 and abs(rb.iterations - r64.iterations) <= tol, (split, rb, r64)
        res = bh - oracle.spmv(rpe, colse, Ae.vals.cpu().numpy(), xb.cpu().numpy(), bs=3)
        assert np.linalg.norm(res) / np.linalg.norm(bh) < 1e-11 * 1.25
        assert (xb - x64).norm().item() / x64.norm().item() < 1e-9
        # a re-assembly with other coefficients, through refresh()
        Ae2 = fem.assemble_matrix(fem.elasticity_form(V, 2e3 * E, 0.3), bcs=[bc])
        Ae.vals.copy_(Ae2.vals)
        solver.refresh()
        xr = torch.zeros_like(be)
        assert solver.solve(be, xr, rtol=1e-11).status == 0
        res = bh - oracle.spmv(rpe, colse, Ae.vals.cpu().numpy(), xr.cpu().numpy(), bs=3)
        assert np.linalg.norm(res) / np.linalg.norm(bh) < 1e-11 * 1.25
        Ae = fem.assemble_matrix(a, bcs=[bc])


def _poisson_system(oracle, n, deg, seed):
    from dolfinx_gb300 import fem

    m, V, kappa, f, rp, cols = problem(oracle, n, deg, seed=seed)
    X = V.tabulate_dof_coordinates()
    bnd = np.flatnonzero(np.isclose(X[:, 0], 0) | np.isclose(X[:, 0], 1)).astype(np.int32)
    bc = fem.dirichletbc(0.0, bnd, V)
    a = fem.poisson_form(V, kappa)
    A = fem.assemble_matrix(a, bcs=[bc])
    b = fem.RhsAssembler(fem.source_form(V, f), a, [bc]).assemble()
    return A, b, rp, cols


def test_operator_cg_matches_csr_cg(cuda, oracle, capi):
    from dolfinx_gb300 import la

    A, b, rp, cols = _poisson_system(oracle, (10, 9, 8), 2, 31)
    x1, r1 = la.cg(A, b, rtol=1e-10)
    s = la.OperatorCGSolver(A)
    x2 = torch.zeros_like(b)
    r2 = s.solve(b, x2, rtol=1e-10)
    assert r2.status == 0 and abs(r2.iterations - r1.iterations) <= 3
    bh = b.cpu().numpy()
    res = bh - oracle.spmv(rp, cols, A.vals.cpu().numpy(), x2.cpu().numpy())
    assert np.linalg.norm(res) / np.linalg.norm(bh) < 1e-10 * 1.0001
    rel = (x1 - x2).norm() / x1.norm()
    assert rel < 1e-7


def test_cg_vector_and_scalar_elementwise_paths(cuda, oracle, capi):
    """The CG update kernels move 16-byte vectors when every array is 16-byte
    aligned (with a scalar tail: n = 6,783 is odd) and fall back to scalar
    loads otherwise; an x that starts 8 bytes into its allocation takes the
    fallback. Both paths meet the stopping test in the oracle's SpMV."""
    from dolfinx_gb300 import la

    A, b, rp, cols = _poisson_system(oracle, (10, 9, 8), 2, 31)
    assert A.nrows % 2 == 1
    x1, r1 = la.cg(A, b, rtol=1e-10)
    buf = torch.zeros(A.nrows + 1, dtype=torch.float64, device="cuda")
    x2 = buf[1:]
    assert x2.data_ptr() % 16 == 8
    x2, r2 = la.cg(A, b, x=x2, rtol=1e-10)
    assert r1.status == 0 and r2.status == 0 and abs(r1.iterations - r2.iterations) <= 2
    bh = b.cpu().numpy()
    vals = A.vals.cpu().numpy()
    for x in (x1, x2):
        res = bh - oracle.spmv(rp, cols, vals, x.cpu().numpy())
        assert np.linalg.norm(res) / np.linalg.norm(bh) < 1e-10 * 1.0001
    assert (x1 - x2).norm() / x1.norm() < 1e-7


@pytest.mark.parametrize("variant,inner_rtol", [("restart", 1e-3), ("restart", 1e-5),
                                                 ("reliable", 0.1), ("reliable", 0.01),
                                                 ("flexible", 0.1), ("flexible", 0.3)])
def test_iterative_refinement_reaches_fp64(cuda, oracle, capi, variant, inner_rtol):
    """FP32-inner refinement meets the FP64 stopping test (|r|/|r0| < 1e-10
    in FP64) and agrees with the plain FP64 CG solution to the accuracy
    both solves carry."""
    from dolfinx_gb300 import la

    A, b, rp, cols = _poisson_system(oracle, (12, 12, 12), 2, 32)
    s64 = la.OperatorCGSolver(A)
    x64 = torch.zeros_like(b)
    s64.solve(b, x64, rtol=1e-12)
    ir = la.IRSolver(A, inner_rtol=inner_rtol, variant=variant)
    x = torch.zeros_like(b)
    r = ir.solve(b, x, rtol=1e-12)
    assert r.status == 0 and r.outer_iterations >= 2
    bh = b.cpu().numpy()
    xs = x.cpu().numpy()
    res = bh - oracle.spmv(rp, cols, A.vals.cpu().numpy(), xs)
    assert np.linalg.norm(res) / np.linalg.norm(bh) < 1e-12 * 1.0001
    rel = (x - x64).norm().item() / x64.norm().item()
    assert rel < 1e-10, rel


def _fused_vs_unfused(capi, A, b, residual, jacobi=True, variant="reliable"):
    """IR solves of A x = b with the fused FP32 update on and off."""
    from dolfinx_gb300 import la

    L = capi.lib()
    out = {}
    try:
        for fused in (1, 0):
            capi.check(L.dfx_set_cg_fused_update(fused))
            on = C.c_int32(-1)
            capi.check(L.dfx_get_cg_fused_update(C.byref(on)))
            assert on.value == fused
            ir = la.IRSolver(A, jacobi=jacobi, variant=variant)
            x = torch.zeros_like(b)
            r = ir.solve(b, x, rtol=1e-11)
            assert r.status == 0
            assert residual(x) < 1e-11 * 1.0001
            out[fused] = (r, x)
    finally:
        capi.check(L.dfx_set_cg_fused_update(1))
    (r1, x1), (r0, x0) = out[1], out[0]
    assert abs(r1.inner_iterations - r0.inner_iterations) <= max(2, r0.inner_iterations // 100)
    assert (x1 - x0).norm().item() / x0.norm().item() < 1e-9
    # two kernels per inner iteration against four
    assert r1.kernel_launches < r0.kernel_launches


@pytest.mark.parametrize("n,jacobi,variant", [((12, 12, 12), True, "reliable"),
                                               ((23, 21, 19), True, "reliable"),
                                               ((12, 12, 12), False, "reliable"),
                                               ((12, 12, 12), True, "restart")])
def test_fused_update_matches_four_kernel_iteration(cuda, oracle, capi, n, jacobi, variant):
    """The two-kernel FP32 inner iteration (SpMV + one cooperative kernel
    with grid-wide barriers) and the four-kernel one run the same
    recurrence: both meet the FP64 stopping test in the oracle's SpMV, with
    inner iteration counts within 1 % and solutions within the accuracy the
    solves carry. (23, 21, 19) P2 has a ragged tail (n % 4 = 3); the cases
    without Jacobi and with restarted refinement take the kernel's other
    instantiations."""
    A, b, rp, cols = _poisson_system(oracle, n, 2, 33)
    bh = b.cpu().numpy()

    def residual(x):
        res = bh - oracle.spmv(rp, cols, A.vals.cpu().numpy(), x.cpu().numpy())
        return np.linalg.norm(res) / np.linalg.norm(bh)

    _fused_vs_unfused(capi, A, b, residual, jacobi=jacobi, variant=variant)


def test_pooled_operator_shares(cuda, oracle, capi):
    """Shares whose values come from the library's stream-ordered pool give
    the same products as plain shares; dropping them (in stream order) and
    making new ones reuses the pool, and trimming returns its memory."""
    from dolfinx_gb300 import la

    A, b, rp, cols = _poisson_system(oracle, (6, 5, 4), 2, 41)
    for dtype in (torch.float64, torch.float32):
        op = la.SellOperator(A, dtype, 256)
        x = torch.from_numpy(np.random.default_rng(2).standard_normal(A.nrows)).to(
            device="cuda", dtype=dtype)
        ref = op.share(A).apply(x)
        s = torch.cuda.Stream()
        for _ in range(3):
            with torch.cuda.stream(s):
                sh = op.share(A, pool_stream=s)
                y = sh.apply(x)
            s.synchronize()
            assert torch.equal(y, ref)
            del sh
        capi.check(capi.lib().dfx_operator_pool_trim())


def test_grid_barrier_wait_is_bounded(cuda, capi):
    """The grid barrier of the fused update gives up instead of hanging: with
    an arrival missing, both blocks of the self-test report DFX_ERR_TIMEOUT
    within the wait limit, and the context still runs work afterwards."""
    import time

    from dolfinx_gb300 import la

    gave_up = C.c_int32(-1)
    t0 = time.perf_counter()
    capi.check(capi.lib().dfx_selftest_grid_barrier(C.byref(gave_up)))
    assert gave_up.value == 2
    assert time.perf_counter() - t0 < 30.0
    x = torch.arange(1000, dtype=torch.float64, device="cuda")
    assert abs(la.inner_product(x, x) - float((x * x).sum())) < 1e-6


def test_fused_update_large_system(cuda, capi):
    """A P2 system of 1.77M unknowns: more float4 per thread than the fused
    kernel keeps in registers between its phases, so part of p, r and D^-1
    is read again for the p update. Residuals in the library's FP64 CSR
    SpMV (itself checked against the oracle)."""
    from dolfinx_gb300 import fem, la, mesh

    m = mesh.create_unit_cube(60, 60, 60)
    V = fem.functionspace(m, ("Lagrange", 2))
    rng = np.random.default_rng(5)
    kappa = torch.from_numpy(np.exp(rng.normal(0.0, 1.0, m.num_cells))).cuda()
    f = torch.from_numpy(rng.uniform(-1, 1, m.num_nodes)).cuda()
    X = V.tabulate_dof_coordinates()
    bnd = np.flatnonzero(np.isclose(X[:, 0], 0) | np.isclose(X[:, 0], 1)).astype(np.int32)
    bc = fem.dirichletbc(0.0, bnd, V)
    a = fem.poisson_form(V, kappa)
    A = fem.assemble_matrix(a, bcs=[bc])
    b = fem.RhsAssembler(fem.source_form(V, f), a, [bc]).assemble()
    assert V.num_dofs // 4 > 152 * 512 * 4

    def residual(x):
        return (b - A.matvec(x)).norm().item() / b.norm().item()

    _fused_vs_unfused(capi, A, b, residual)


def test_block_expansion_and_elasticity_refinement(cuda, oracle, capi):
    """bs-3 CSR -> scalar CSR: same product; FP64 PCG and mixed refinement
    on the expanded elasticity system meet the FP64 stopping test."""
    from dolfinx_gb300 import fem, la

    m, V, E, f, rp, cols = problem(oracle, (6, 3, 3), 2, bs=3, seed=13)
    X = V.tabulate_dof_coordinates()
    clamp = np.flatnonzero(np.isclose(X[:, 0], 0)).astype(np.int32)
    bc = fem.dirichletbc(np.zeros(3), clamp, V)
    a = fem.elasticity_form(V, 1e3 * E, 0.3)
    A = fem.assemble_matrix(a, bcs=[bc])
    b = fem.RhsAssembler(fem.body_force_form(V, (0, 0, -1)), a, [bc]).assemble()
    S = A.expand_blocks()
    x = torch.from_numpy(np.random.default_rng(0).standard_normal(V.num_dofs)).cuda()
    assert_close(S.matvec(x).cpu().numpy(), A.matvec(x).cpu().numpy(), rtol=1e-14)
    vals = A.vals.cpu().numpy()
    for solver in (la.OperatorCGSolver(S), la.IRSolver(S), la.IRSolver(S, variant="flexible")):
        xs = torch.zeros_like(b)
        solver.solve(b, xs, rtol=1e-10)
        bh = b.cpu().numpy()
        r = bh - oracle.spmv(rp, cols, vals, xs.cpu().numpy(), bs=3)
        assert np.linalg.norm(r) / np.linalg.norm(bh) < 1e-10 * 1.001


def test_refinement_on_a_system_above_four_million_rows(cuda, capi):
    """The p.Ap reduction of the FP32 sliced-ELL iteration takes more than
    16 partial slots per thread above ~4.2M rows (at most 32 blocks): P2 on
    82^3 x 6 tetrahedra has 4,492,125 rows. The mixed solve meets the FP64
    stopping test and lands within 1e-10 of the plain FP64 solution."""
    from dolfinx_gb300 import fem, la, mesh

    m = mesh.create_unit_cube(82, 82, 82, device="cuda")
    V = fem.functionspace(m, ("Lagrange", 2))
    assert V.num_dofs == 165 ** 3
    X = V.tabulate_dof_coordinates()
    bnd = np.flatnonzero(np.isclose(X[:, 0], 0.0) | np.isclose(X[:, 0], 1.0)).astype(np.int32)
    bc = fem.dirichletbc(0.0, bnd, V)
    rng = np.random.default_rng(5)
    kappa = torch.from_numpy(np.exp(rng.normal(0.0, 1.0, m.num_cells))).cuda()
    f = torch.from_numpy(rng.uniform(-1.0, 1.0, m.num_nodes)).cuda()
    a = fem.poisson_form(V, kappa)
    A = fem.assemble_matrix(a, [bc])
    b = fem.RhsAssembler(fem.source_form(V, f), a, [bc]).assemble()
    s64 = la.OperatorCGSolver(A, jacobi=True, sigma=1024)
    x64 = torch.zeros_like(b)
    r64 = s64.solve(b, x64, rtol=5e-12)
    ir = la.IRSolver(A, jacobi=True, sigma=1024)
    x = torch.zeros_like(b)
    r = ir.solve(b, x, rtol=5e-12)
    assert r64.status == 0 and r.status == 0
    y = A.matvec(x)
    assert ((b - y).norm() / b.norm()).item() < 5e-12 * 1.0001
    rel = ((x - x64).norm() / x64.norm()).item()
    assert rel < 1e-10, rel


def test_released_operator_is_shared_but_not_applied(cuda, oracle, capi):
    """dfx_operator_release_values: the source keeps its structure (shares
    work and permute), its own values and scratch are freed
    (dfx_operator_device_bytes drops by them), and applying or solving with
    it is refused with DFX_ERR_INVALID, not run on freed memory."""
    from dolfinx_gb300 import la

    A, b, rp, cols = _poisson_system(oracle, (6, 5, 4), 2, 17)
    src = la.SellOperator(A, torch.float32, 64, compress_cols=True)
    before = src.device_bytes()
    slots = src.info()["slots"]
    src.release_values()
    after = src.device_bytes()
    # values (4 B per slot) and scratch (2 n floats) are gone
    assert before - after == 4 * slots + 8 * A.nrows
    x = torch.rand(A.nrows, dtype=torch.float32, device="cuda")
    with pytest.raises(capi.DfxError) as e:
        src.apply(x)
    assert e.value.code == capi.DFX_ERR_INVALID
    share = src.share(A)
    assert share.device_bytes() == 4 * slots + 8 * A.nrows
    y = share.apply(x)
    ref = A.matvec(x.double()).float()
    assert torch.allclose(y, ref, rtol=1e-5, atol=1e-6 * ref.abs().max().item())
    assert torch.equal(share.to_operator(b), src.to_operator(b))
