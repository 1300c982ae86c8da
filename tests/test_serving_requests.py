"""Host logic of the serving loop (no GPU): the synthetic request stream
follows the serving config - Poisson arrivals at the given rate, n
log-uniform in [8, 96], P1 or P2 with equal probability, k^2 uniform in
[0, 10] - and is reproducible from its seed."""

import math

import numpy as np


def test_request_stream_statistics():
    from dolfinx_gb300 import serving

    reqs = serving.make_requests(20000, rate=500.0, seed=3)
    t = np.array([r.arrival for r in reqs])
    assert (np.diff(t) >= 0).all()
    gaps = np.diff(np.concatenate([[0.0], t]))
    assert abs(gaps.mean() - 1 / 500.0) < 0.05 / 500.0  # exponential gaps, mean 1/rate
    n = np.array([r.n for r in reqs])
    assert n.min() >= 8 and n.max() <= 96
    # log-uniform: the median of n sits near the geometric mean of the range
    assert abs(math.log(np.median(n)) - 0.5 * (math.log(8) + math.log(96))) < 0.05
    deg = np.array([r.degree for r in reqs])
    assert set(deg) == {1, 2} and abs((deg == 2).mean() - 0.5) < 0.02
    k2 = np.array([r.k2 for r in reqs])
    assert k2.min() >= 0.0 and k2.max() <= 10.0 and abs(k2.mean() - 5.0) < 0.1
    assert len({r.seed for r in reqs}) > 19990  # per-request seeds


def test_request_stream_is_reproducible_and_rate_independent_in_content():
    from dolfinx_gb300 import serving

    a = serving.make_requests(50, rate=200.0, seed=1, n_range=(8, 48))
    b = serving.make_requests(50, rate=200.0, seed=1, n_range=(8, 48))
    c = serving.make_requests(50, rate=5000.0, seed=1, n_range=(8, 48))
    assert [(r.n, r.degree, r.k2, r.seed, r.arrival) for r in a] == \
        [(r.n, r.degree, r.k2, r.seed, r.arrival) for r in b]
    # the same requests arrive faster at a higher rate
    assert [(r.n, r.degree, r.k2, r.seed) for r in a] == [(r.n, r.degree, r.k2, r.seed) for r in c]
    assert c[-1].arrival < a[-1].arrival


def test_unit_cube_boundary_nodes_equal_isclose():
    """The serving structures' boundary nodes (two column passes) are the
    nodes np.isclose finds at 0 or 1, for P1/P2 boxes of several sizes and
    for points at and just inside the tolerances."""
    from dolfinx_gb300 import fem, mesh, serving

    for n in (1, 3, 7, 49):
        m = mesh.create_unit_cube(n, n, n)
        for deg in (1, 2):
            X = fem.functionspace(m, ("Lagrange", deg), device="cpu").tabulate_dof_coordinates()
            ref = np.flatnonzero(np.isclose(X, 0.0).any(1) | np.isclose(X, 1.0).any(1))
            np.testing.assert_array_equal(serving.unit_cube_boundary_nodes(X), ref)
    t = 1e-8 + 1e-5
    X = np.array([[0.5, 0.5, 1e-8], [0.5, 0.5, 1.1e-8], [1 - t, 0.5, 0.5],
                  [1 - 1.01 * t, 0.5, 0.5], [1.0, 1.0, 1.0], [0.3, 0.6, 0.9]])
    ref = np.flatnonzero(np.isclose(X, 0.0).any(1) | np.isclose(X, 1.0).any(1))
    np.testing.assert_array_equal(serving.unit_cube_boundary_nodes(X), ref)
