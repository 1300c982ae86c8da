"""Device-side set-up against the host builders and the oracle: the
sparsity pattern built on the GPU must equal the host one bit for bit."""

import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _device_sparsity(capi, nrows, dofmap):
    from dolfinx_gb300 import la

    L = capi.lib()
    nc, nd = dofmap.shape
    dm = torch.from_numpy(np.ascontiguousarray(dofmap, np.int32)).cuda()
    wb = int(L.dfx_sparsity_device_workspace_bytes(nrows, nc, nd))
    work = torch.empty(max(wb, 1), dtype=torch.uint8, device="cuda")
    rp = torch.empty(nrows + 1, dtype=torch.int64, device="cuda")
    nnz = C.c_int64(0)
    capi.check(L.dfx_sparsity_create_device(nrows, nc, nd, la._ptr(dm), la._ptr(rp), None,
                                            C.byref(nnz), la._ptr(work), wb, None))
    cols = torch.empty(max(nnz.value, 1), dtype=torch.int32, device="cuda")
    capi.check(L.dfx_sparsity_create_device(nrows, nc, nd, la._ptr(dm), la._ptr(rp),
                                            la._ptr(cols), C.byref(nnz), la._ptr(work), wb, None))
    return rp.cpu().numpy(), cols[: nnz.value].cpu().numpy()


@pytest.mark.parametrize("deg", [1, 2])
@pytest.mark.parametrize("n", [(1, 1, 1), (2, 3, 4), (9, 8, 7), (16, 16, 16)])
def test_device_sparsity_equals_host_and_oracle(cuda, capi, oracle, n, deg):
    from dolfinx_gb300 import fem, mesh

    m = mesh.create_unit_cube(*n)
    V = fem.functionspace(m, ("Lagrange", deg))
    rp_d, cols_d = V.sparsity_device()
    rp_h, cols_h = V.sparsity()
    rp_o, cols_o = oracle.sparsity(V.num_nodes, V.dofmap)
    np.testing.assert_array_equal(rp_d.cpu().numpy(), rp_h)
    np.testing.assert_array_equal(cols_d.cpu().numpy(), cols_h)
    np.testing.assert_array_equal(rp_h, rp_o)
    np.testing.assert_array_equal(cols_h, cols_o)


def test_device_sparsity_known_sizes(cuda, capi):
    """Known answers: 16^3 x 6 P1 has 66,961 entries (4,913 dofs)."""
    from dolfinx_gb300 import fem, mesh

    V = fem.functionspace(mesh.create_unit_cube(16, 16, 16), ("Lagrange", 1))
    rp, cols = V.sparsity_device()
    assert V.num_nodes == 4913 and int(rp[-1]) == 66961 and cols.numel() == 66961


def test_device_sparsity_arbitrary_dofmap(cuda, capi):
    """A random dofmap (not a mesh): unsorted cells, repeated dofs within a
    cell, dofs that no cell uses (empty rows)."""
    rng = np.random.default_rng(3)
    nrows, nc, nd = 500, 300, 7
    dofmap = rng.integers(0, nrows - 50, (nc, nd)).astype(np.int32)
    rp, cols = _device_sparsity(capi, nrows, dofmap)
    ref = [set() for _ in range(nrows)]
    for c in dofmap:
        for i in c:
            ref[i].update(int(j) for j in c)
    rp_ref = np.zeros(nrows + 1, np.int64)
    rp_ref[1:] = np.cumsum([len(r) for r in ref])
    np.testing.assert_array_equal(rp, rp_ref)
    np.testing.assert_array_equal(cols, np.concatenate([sorted(r) for r in ref]).astype(np.int32))
    assert (np.diff(rp)[-50:] == 0).all()


def test_device_sparsity_limits_and_fallback(cuda, capi):
    """A row whose cells hold more than 1024 dofs is refused with
    DFX_ERR_UNSUPPORTED; an out-of-range dofmap entry with DFX_ERR_INVALID."""
    nc, nd = 110, 10
    dofmap = np.arange(nc * nd, dtype=np.int32).reshape(nc, nd) + 1
    dofmap[:, 0] = 0  # dof 0 in every cell: 1,100 candidates in row 0
    with pytest.raises(capi.DfxError) as e:
        _device_sparsity(capi, nc * nd + 1, dofmap)
    assert e.value.code == capi.DFX_ERR_UNSUPPORTED
    bad = np.array([[0, 1, 2, 9]], np.int32)
    with pytest.raises(capi.DfxError) as e:
        _device_sparsity(capi, 5, bad)
    assert e.value.code == capi.DFX_ERR_INVALID


class _DevPtr:
    """A device int32 array given by pointer, for torch.as_tensor."""

    def __init__(self, ptr, n):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": "<i4", "data": (ptr, False),
                                         "version": 3}


def _perm(capi, op, n):
    ns, nsl, perm = C.c_int64(), C.c_int32(), C.c_void_p()
    capi.check(capi.lib().dfx_operator_info(op.handle, C.byref(ns), C.byref(nsl), C.byref(perm)))
    return torch.as_tensor(_DevPtr(perm.value, n), device="cuda").clone()


@pytest.mark.parametrize("dtype,compress", [(torch.float64, False), (torch.float32, True),
                                            (torch.float32, False)])
@pytest.mark.parametrize("sigma", [32, 256, 1024])
def test_device_operator_build_equals_host(cuda, capi, oracle, dtype, compress, sigma):
    """The sliced-ELL structure built on the device equals the host build:
    same permutation, slot count, and bitwise-equal products (the slot order
    fixes the summation order)."""
    from dolfinx_gb300 import fem, la
    from gpu_util import problem

    m, V, kappa, f, rp, cols = problem(oracle, (7, 6, 5), 2, seed=5)
    A = fem.assemble_matrix(fem.poisson_form(V, kappa))
    dev = la.SellOperator(A, dtype, sigma, compress, build=1)
    host = la.SellOperator(A, dtype, sigma, compress, build=2)
    assert dev.info() == host.info()
    n = A.nrows
    assert torch.equal(_perm(capi, dev, n), _perm(capi, host, n))
    x = torch.rand(n, dtype=dtype, device="cuda")
    y1, y2 = torch.empty_like(x), torch.empty_like(x)
    assert torch.equal(dev.apply_renumbered(x, y1), host.apply_renumbered(x, y2))
    assert torch.equal(dev.apply(x), host.apply(x))


def test_device_operator_long_row_falls_back_to_host(cuda, capi):
    """A row of 301 entries: the device-only build refuses it, the default
    build takes the host path, and the result equals the host build."""
    from dolfinx_gb300 import la

    nc, nd = 50, 7
    dofmap = (np.arange(nc * nd, dtype=np.int32).reshape(nc, nd) + 1)
    dofmap[:, 0] = 0
    nrows = nc * nd + 1
    rp, cols = _device_sparsity(capi, nrows, dofmap)
    assert rp[1] - rp[0] == 1 + nc * (nd - 1)
    rng = np.random.default_rng(1)
    vals = torch.from_numpy(rng.standard_normal(cols.size)).cuda()
    A = la.MatrixCSR(torch.from_numpy(rp).cuda(), torch.from_numpy(cols).cuda(), vals, 1)
    with pytest.raises(capi.DfxError) as e:
        la.SellOperator(A, torch.float64, build=1)
    assert e.value.code == capi.DFX_ERR_UNSUPPORTED
    auto = la.SellOperator(A, torch.float64, build=0)
    host = la.SellOperator(A, torch.float64, build=2)
    assert auto.info() == host.info()
    x = torch.rand(nrows, dtype=torch.float64, device="cuda")
    assert torch.equal(auto.apply(x), host.apply(x))


@pytest.mark.parametrize("nrows", [0, 5])
def test_device_sparsity_without_cells(cuda, capi, nrows):
    rp, cols = _device_sparsity(capi, nrows, np.zeros((0, 4), np.int32))
    np.testing.assert_array_equal(rp, np.zeros(nrows + 1, np.int64))
    assert cols.size == 0


@pytest.mark.parametrize("build", [1, 2])
def test_empty_operator(cuda, capi, build):
    from dolfinx_gb300 import la

    A = la.MatrixCSR(torch.zeros(1, dtype=torch.int64, device="cuda"),
                     torch.zeros(0, dtype=torch.int32, device="cuda"),
                     torch.zeros(0, dtype=torch.float64, device="cuda"), 1)
    op = la.SellOperator(A, torch.float64, build=build)
    assert op.info()["slots"] == 0
    x = torch.zeros(0, dtype=torch.float64, device="cuda")
    assert op.apply(x).numel() == 0


@pytest.mark.parametrize("tag", ["p1", "p2"])
def test_device_sparsity_matches_reference(cuda, capi, tag):
    """The device builder against the reference's own SparsityPattern
    (golden vectors written from la/SparsityPattern.cpp)."""
    import os

    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_golden.npz"))
    dm, rp_ref, cols_ref = g[f"sp_dofmap_{tag}"], g[f"sp_rowptr_{tag}"], g[f"sp_cols_{tag}"]
    rp, cols = _device_sparsity(capi, rp_ref.size - 1, dm)
    np.testing.assert_array_equal(rp, rp_ref)
    np.testing.assert_array_equal(cols, cols_ref)


@pytest.mark.parametrize("deg", [1, 2])
@pytest.mark.parametrize("n,reorder", [((1, 1, 1), True), ((5, 3, 4), True), ((24, 24, 24), True),
                                       ((30, 20, 26), False)])
def test_device_dofmap_matches_host(cuda, capi, oracle, n, reorder, deg):
    """The device dofmap builder (first positions by atomic minimum, an edge
    hash table, a scan) gives the host builder's and the oracle's numbering
    bit for bit, in RCM and in build order."""
    from dolfinx_gb300 import fem, mesh

    m = mesh.create_box(((0, 0, 0), (1, 1, 1)), n, reorder=reorder)
    Vd = fem.functionspace(m, ("Lagrange", deg))          # built on the device
    Vh = fem.functionspace(m, ("Lagrange", deg), device="cpu")
    assert Vd._dofmap_dev is not None
    assert Vd.num_nodes == Vh.num_nodes
    np.testing.assert_array_equal(Vd.dofmap, Vh.dofmap)
    np.testing.assert_array_equal(Vd.dofmap_device().cpu().numpy(), Vh.dofmap)
    dm, nn = oracle.dofmap_tet(m.cells, deg)
    assert nn == Vd.num_nodes
    np.testing.assert_array_equal(Vd.dofmap, dm)


def test_device_dofmap_p2_64_matches_golden(cuda, capi):
    """The 64^3 P2 dofmap built on the device has the golden digest."""
    import hashlib
    import json
    import os

    from dolfinx_gb300 import fem, mesh

    ref = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                                      "config_structure.json")))["c2_p2_unit_cube_64"]
    V = fem.functionspace(mesh.create_unit_cube(64, 64, 64), ("Lagrange", 2))
    assert V._dofmap_dev is not None and V.num_nodes == ref["num_nodes"]
    got = hashlib.sha256(np.ascontiguousarray(V.dofmap_device().cpu().numpy()).tobytes())
    assert got.hexdigest() == ref["dofmap"]


def test_device_dofmap_rejects_bad_vertices(cuda, capi):
    import ctypes as C

    import torch

    cells = torch.tensor([[0, 1, 2, 7]], dtype=torch.int32, device="cuda")
    lib = capi.lib()
    wb = int(lib.dfx_dofmap_device_workspace_bytes(1, 4, 2))
    work = torch.empty(wb, dtype=torch.uint8, device="cuda")
    dm = torch.empty((1, 10), dtype=torch.int32, device="cuda")
    n = C.c_int32(0)
    rc = lib.dfx_dofmap_create_tet_device(1, C.c_void_p(cells.data_ptr()), 4, 2,
                                          C.c_void_p(dm.data_ptr()), C.byref(n),
                                          C.c_void_p(work.data_ptr()), wb, None)
    assert rc == capi.DFX_ERR_INVALID
