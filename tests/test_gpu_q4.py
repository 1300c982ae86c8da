"""GPU parity of the matrix-free Q4 hexahedral Laplacian action (sum
factorisation, FP64 and FP32) against the oracle's full-quadrature element
loop, and of the matrix-free CG (FP64 and mixed precision)."""

import numpy as np
import pytest
import torch

from gpu_util import assert_close

pytestmark = pytest.mark.gpu


def _setup(dims, seed=0, kappa=1.0):
    from dolfinx_gb300 import matrix_free as mf

    v = mf.hex_box_vertices(*dims, perturb=0.05, seed=seed)
    op = mf.Q4Laplacian(v, *dims, kappa=kappa)
    return mf, v, op


@pytest.mark.parametrize("dims", [(1, 1, 1), (3, 3, 3), (2, 3, 4)])
def test_q4_action_f64(cuda, oracle, dims):
    mf, v, op = _setup(dims, seed=1, kappa=2.5)
    u = np.random.default_rng(2).standard_normal(op.n)
    y = op(torch.from_numpy(u).cuda()).cpu().numpy()
    ref = oracle.q4_action(dims, v, u, kappa=2.5)
    # The sum-factorised and full-matrix evaluations differ only in rounding.
    assert_close(y, ref, rtol=1e-12)


def test_q4_action_f32(cuda, oracle):
    dims = (3, 3, 3)
    mf, v, op = _setup(dims, seed=3)
    u = np.random.default_rng(4).standard_normal(op.n)
    y = op(torch.from_numpy(u).float().cuda()).double().cpu().numpy()
    ref = oracle.q4_action(dims, v, u)
    # FP32 contractions and geometry: a few units of FP32 rounding.
    assert_close(y, ref, rtol=2e-5)


@pytest.mark.parametrize("dims,cache", [((3, 3, 3), True), ((2, 3, 4), False),
                                        ((5, 4, 3), True)])
def test_q4_action_tensor_cores(cuda, oracle, dims, cache):
    """The tcgen05 action (TF32 words split hi + lo, three products per MMA)
    matches the oracle's full-quadrature FP64 element loop to FP32 accuracy,
    and the CUDA-core FP32 action to a few FP32 ulps, on odd and even
    meshes, with and without the edge cache."""
    from dolfinx_gb300 import matrix_free as mf

    v = mf.hex_box_vertices(*dims, perturb=0.05, seed=7)
    op = mf.Q4Laplacian(v, *dims, kappa=1.5, cache_edges=cache)
    u = np.random.default_rng(8).standard_normal(op.n)
    u32 = torch.from_numpy(u).float().cuda()
    y = torch.empty_like(u32)
    op.apply_tc(u32, y)
    op.check_tc()
    ref = oracle.q4_action(dims, v, u, kappa=1.5)
    assert_close(y.double().cpu().numpy(), ref, rtol=2e-5)
    assert_close(y.double().cpu().numpy(), op(u32).double().cpu().numpy(), rtol=5e-6)


def test_q4_tensor_core_cg(cuda):
    """Mixed CG on the tensor-core action meets the FP64 stopping test and
    agrees with the CUDA-core mixed CG and the FP64 CG."""
    from dolfinx_gb300 import matrix_free as mf

    dims = (8, 8, 8)
    v = mf.hex_box_vertices(*dims, perturb=0.05, seed=9)
    op = mf.Q4Laplacian(v, *dims)
    bnd = torch.from_numpy(mf.boundary_mask(*dims)).cuda()
    b = torch.from_numpy(np.random.default_rng(10).uniform(-1, 1, op.n)).cuda().masked_fill(bnd, 0)
    xs = {}
    for mode in ("fp64", "mixed", "mixed_tc"):
        x = torch.zeros_like(b)
        r = mf.MatrixFreeCG(op, mode=mode).solve(b, x, rtol=1e-10)
        assert r.status == 0
        assert ((b - op(x)).norm() / b.norm()).item() < 1e-10 * 1.001
        xs[mode] = x
    for mode in ("mixed", "mixed_tc"):
        assert ((xs[mode] - xs["fp64"]).norm() / xs["fp64"].norm()).item() < 1e-8


@pytest.mark.parametrize("dims", [(3, 3, 3), (1, 1, 1), (2, 3, 4), (5, 4, 3)])
def test_q4_geometry_cache_matches_oracle(cuda, oracle, dims):
    """Actions on the cached geometric factors (dfx_q4_geometry) against the
    oracle's full-quadrature element loop (FP64 to 1e-12, FP32 to 2e-5) and
    against the actions that form the geometry on the fly; the mixed CG on
    them meets the FP64 stopping test."""
    from dolfinx_gb300 import matrix_free as mf

    v = mf.hex_box_vertices(*dims, perturb=0.05, seed=21)
    op = mf.Q4Laplacian(v, *dims, kappa=1.7, cache_geometry=True)
    plain = mf.Q4Laplacian(v, *dims, kappa=1.7, cache_geometry=False)
    assert set(op.geom) == {torch.float32, torch.float64}
    assert op.geom[torch.float32].numel() == 750 * int(np.prod(dims))
    # G = w kappa adj adj^T / |det J| is positive definite: its diagonal
    # (entries 00, 11, 22 of each point) is positive everywhere.
    for g in op.geom.values():
        diag = g.view(-1, 6, 125)[:, [0, 3, 5], :]
        assert bool((diag > 0).all())
    u = np.random.default_rng(22).standard_normal(op.n)
    ref = oracle.q4_action(dims, v, u, kappa=1.7)
    u64 = torch.from_numpy(u).cuda()
    y64 = op(u64)
    assert_close(y64.cpu().numpy(), ref, rtol=1e-12)
    assert_close(y64.cpu().numpy(), plain(u64).cpu().numpy(), rtol=1e-13)
    y32 = op(u64.float()).double().cpu().numpy()
    assert_close(y32, ref, rtol=2e-5)
    assert_close(y32, plain(u64.float()).double().cpu().numpy(), rtol=5e-6)
    if min(dims) >= 3:
        bnd = torch.from_numpy(mf.boundary_mask(*dims)).cuda()
        b = u64.masked_fill(bnd, 0)
        x = torch.zeros_like(b)
        r = mf.MatrixFreeCG(op, mode="mixed").solve(b, x, rtol=1e-10)
        assert r.status == 0
        assert ((b - plain(x)).norm() / b.norm()).item() < 1e-10 * 1.001


def test_q4_edge_cache_is_bitwise_neutral(cuda):
    from dolfinx_gb300 import matrix_free as mf

    dims = (6, 5, 4)
    v = mf.hex_box_vertices(*dims, perturb=0.05, seed=12)
    cached = mf.Q4Laplacian(v, *dims, cache_edges=True)
    plain = mf.Q4Laplacian(v, *dims, cache_edges=False)
    u = torch.from_numpy(np.random.default_rng(13).standard_normal(cached.n)).float().cuda()
    assert torch.equal(cached(u), plain(u))


def test_q4_action_symmetric_and_deterministic(cuda):
    dims = (8, 8, 8)
    mf, v, op = _setup(dims, seed=5)
    rng = np.random.default_rng(6)
    bnd = torch.from_numpy(mf.boundary_mask(*dims)).cuda()
    u = torch.from_numpy(rng.standard_normal(op.n)).cuda().masked_fill(bnd, 0.0)
    w = torch.from_numpy(rng.standard_normal(op.n)).cuda().masked_fill(bnd, 0.0)
    Au, Aw = op(u), op(w)
    a, b = float(torch.dot(w, Au)), float(torch.dot(u, Aw))
    assert abs(a - b) <= 1e-11 * max(abs(a), abs(b))
    assert float(torch.dot(u, Au)) > 0.0
    # Colour order fixes the summation order: repeat applications agree bitwise.
    assert torch.equal(op(u), Au)


@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_q4_cg_oracle_residual(cuda, oracle, mode):
    dims = (4, 4, 4)
    mf, v, op = _setup(dims, seed=7)
    rng = np.random.default_rng(8)
    b = rng.standard_normal(op.n)
    b[mf.boundary_mask(*dims)] = 0.0
    x = torch.zeros(op.n, dtype=torch.float64, device="cuda")
    res = mf.MatrixFreeCG(op, mode=mode).solve(torch.from_numpy(b).cuda(), x, rtol=1e-10)
    assert res.status == 0 and res.iterations > 0
    xs = x.cpu().numpy()
    r = b - oracle.q4_action(dims, v, xs)
    assert np.linalg.norm(r) <= 1e-9 * np.linalg.norm(b)
    assert np.all(xs[mf.boundary_mask(*dims)] == 0.0)


def test_q4_cg_modes_agree(cuda):
    dims = (12, 10, 8)
    mf, v, op = _setup(dims, seed=9)
    rng = np.random.default_rng(10)
    bnd = torch.from_numpy(mf.boundary_mask(*dims)).cuda()
    b = torch.from_numpy(rng.uniform(-1, 1, op.n)).cuda().masked_fill(bnd, 0.0)
    xs = {}
    for mode in ("fp64", "mixed"):
        x = torch.zeros_like(b)
        res = mf.MatrixFreeCG(op, mode=mode).solve(b, x, rtol=1e-10)
        assert res.status == 0
        r = b - op(x)
        assert float(torch.linalg.norm(r)) <= 1.5e-10 * float(torch.linalg.norm(b))
        xs[mode] = x
    err = float(torch.linalg.norm(xs["fp64"] - xs["mixed"]) / torch.linalg.norm(xs["fp64"]))
    assert err < 1e-7


def test_q4_cg_nonzero_guess_and_errors(cuda):
    from dolfinx_gb300 import _capi

    dims = (3, 3, 3)
    mf, v, op = _setup(dims, seed=11)
    bnd = torch.from_numpy(mf.boundary_mask(*dims)).cuda()
    b = torch.ones(op.n, dtype=torch.float64, device="cuda").masked_fill(bnd, 0.0)
    x = torch.rand(op.n, dtype=torch.float64, device="cuda").masked_fill(bnd, 0.0)
    res = mf.MatrixFreeCG(op, mode="fp64").solve(b, x, rtol=1e-10)
    assert res.status == 0
    assert float(torch.linalg.norm(b - op(x))) <= 1e-9 * float(torch.linalg.norm(b))
    # An iteration cap reports non-convergence without touching the GPU state.
    x.zero_()
    with pytest.raises(_capi.DfxError):
        mf.MatrixFreeCG(op, mode="fp64").solve(b, x, rtol=1e-14, max_iters=3)
    # Host-side argument checks.
    with pytest.raises(_capi.DfxError):
        mf.MatrixFreeCG(op, mode="mixed", delta=1.5).solve(b, x)
