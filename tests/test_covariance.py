"""Host parts of the operator build (no GPU): the von Karman covariance by
the trapezoidal K_{5/6} rule the device build uses, against scipy's ``kv``
(through the oracle), and the sparse-stencil geometry."""

import numpy as np

from cases import rel_l2


def test_phase_covariance_matches_scipy_kv():
    from oracle.extrusion import phase_covariance as ref
    from pyturb_gb300.covariance import phase_covariance

    r = np.concatenate([[0.0], np.logspace(-5, 3, 500)])
    for L0 in (1.0, 25.0, 100.0):
        got, want = phase_covariance(r, 0.15, L0), ref(r, 0.15, L0)
        ok = want > 1e-300
        assert np.max(np.abs(got[ok] - want[ok]) / np.abs(want[ok])) < 1e-12
    # array shapes are kept
    assert phase_covariance(np.zeros((3, 4)), 0.1, 25.0).shape == (3, 4)


def test_sparse_points_rule():
    from oracle.extrusion import sparse_points as ref
    from pyturb_gb300.covariance import sparse_points

    assert sparse_points(1449, 2, 0) == []
    pts = sparse_points(1449, 2, 2)
    assert pts == ref(1449, 2, 2)
    assert sorted({d for d, _ in pts}) == [4, 8, 16, 32, 64, 128, 256, 512, 1024]
    assert sorted({c for _, c in pts}) == [483, 965]
    assert all(d > 3 for d, _ in sparse_points(40, 3, 1))
    assert max(d for d, _ in sparse_points(1449, 2, 2, max_depth=100)) == 64


def test_smooth_seed_sizes():
    from pyturb_gb300.extrude import _smooth_size

    for n in (1, 2, 5, 48, 1449, 2473):
        v = _smooth_size(n)
        assert v >= n
        while v % 2 == 0:
            v //= 2
        while v % 3 == 0:
            v //= 3
        assert v == 1
    assert _smooth_size(1449) == 1458 and _smooth_size(2473) == 2592
    assert rel_l2(np.ones(3), np.ones(3)) == 0.0
