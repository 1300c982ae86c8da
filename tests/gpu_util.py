"""Shared set-up for the GPU parity tests: the same seeded problem fed to
the oracle (numpy) and to the device path."""

import numpy as np


def problem(oracle, n, deg, seed=0, sigma=1.0, bs=1):
    from dolfinx_gb300 import fem, mesh

    m = mesh.create_unit_cube(*n)
    V = fem.functionspace(m, ("Lagrange", deg, (3,) if bs == 3 else None))
    rng = np.random.default_rng(seed)
    kappa = np.exp(rng.normal(0.0, sigma, m.num_cells))
    f = rng.uniform(-1, 1, m.num_nodes)
    rp, cols = oracle.sparsity(V.num_nodes, V.dofmap)
    return m, V, kappa, f, rp, cols


def assert_close(gpu, ref, rtol=1e-12):
    """Entry-wise agreement to rtol relative to the largest entry."""
    gpu = np.asarray(gpu)
    ref = np.asarray(ref)
    scale = max(np.abs(ref).max(), 1e-300)
    err = np.abs(gpu - ref).max() / scale
    assert err <= rtol, f"max relative error {err:.3e} > {rtol:.1e}"
    return err
