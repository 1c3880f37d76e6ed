"""The FP64 device build of the Assemat-Wilson operator against the float64
oracle (the reference's host recipe restated): ``A`` directly, ``B B^T``
(the factor itself is not unique), the reference's eigen-square-root ``B``
in the parity mode, and the stencil factor ``S S^T = C_zz``; for the
rows-only stencil and for full rows plus sparse columns."""

import time

import numpy as np
import pytest

from cases import rel_l2

pytestmark = pytest.mark.gpu

# float64 builds differ by the conditioning of C_zz times rounding (the
# stencil covariance is smooth): measured ~3e-9 for A and ~1e-9 for B B^T
TOL_A = 1e-7
TOL_BBT = 1e-8


def _oracle(W, m, dx, L0, sparse=()):
    from oracle.extrusion import build_extrusion

    return build_extrusion(W, m, dx, L0, sparse=sparse)


@pytest.mark.parametrize("W,m,dx,L0,columns", [(48, 2, 1.0 / 32, 25.0, 0), (301, 2, 0.02, 20.0, 0),
                                               (48, 2, 1.0 / 32, 25.0, 2),
                                               (200, 3, 0.01, 10.0, 2)])
def test_operator_matches_float64_oracle(W, m, dx, L0, columns):
    from pyturb_gb300.covariance import build_operator, sparse_points

    sparse = sparse_points(W, m, columns)
    a_ref, b_ref = _oracle(W, m, dx, L0, sparse)
    op = build_operator(W, m, dx, L0, sparse, want_float64=True, want_seed=True)
    a, b = op.host()
    assert a.shape == a_ref.shape and b.shape == (W, W)
    assert rel_l2(a, a_ref) < TOL_A, rel_l2(a, a_ref)
    assert rel_l2(b @ b.T, b_ref @ b_ref.T) < TOL_BBT
    assert np.allclose(np.triu(b, 1), 0.0)  # the build's own factor is triangular
    # float32 operator = the float64 one rounded
    assert rel_l2(op.M.double().cpu().numpy(), np.concatenate([a, b], 1)) < 1e-7
    # stencil factor: S S^T = C_zz
    from oracle.extrusion import phase_covariance

    yz, xz = np.mgrid[0:m, 0:W]
    pts = np.column_stack((xz.ravel(), yz.ravel())).astype(float)
    if sparse:
        pts = np.concatenate([pts, np.array([(c, m - d) for d, c in sparse], dtype=float)])
    czz = phase_covariance(np.hypot(pts[:, None, 0] - pts[None, :, 0],
                                    pts[:, None, 1] - pts[None, :, 1]) * dx, 1.0, L0)
    S = op.S.double().cpu().numpy()
    assert rel_l2(S @ S.T, czz) < 1e-6


@pytest.mark.parametrize("W,columns", [(48, 0), (64, 0), (48, 2)])
def test_eigen_factor_reproduces_the_reference_B(W, columns):
    """The parity mode's B (eigen square root of the device-built conditional
    covariance) equals the reference's own B column for column."""
    from pyturb_gb300.covariance import build_operator, sparse_points

    sparse = sparse_points(W, 2, columns)
    _a_ref, b_ref = _oracle(W, 2, 1.0 / 32, 25.0, sparse)
    _a, b = build_operator(W, 2, 1.0 / 32, 25.0, sparse, b_factor="eigh",
                           want_float64=True).host()
    assert rel_l2(b, b_ref) < 1e-7, rel_l2(b, b_ref)


def test_benchmark_width_build_against_oracle_and_time():
    """W = 1449 (n = 1024 extruder), rows-only and 2 rows + 2 sparse columns:
    A and B B^T against the oracle, and the device build time."""
    import torch

    from pyturb_gb300.covariance import build_operator, sparse_points

    W, m, dx, L0 = 1449, 2, 8.0 / 1024, 25.0
    for columns in (0, 2):
        sparse = sparse_points(W, m, columns)
        build_operator(W, m, dx, L0, sparse)  # warm-up (module load)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        op = build_operator(W, m, dx, L0, sparse, want_float64=True)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        a, b = op.host()
        a_ref, b_ref = _oracle(W, m, dx, L0, sparse)
        ea, eb = rel_l2(a, a_ref), rel_l2(b @ b.T, b_ref @ b_ref.T)
        print(f"W={W} sparse={len(sparse)}: device build {dt * 1e3:.1f} ms, "
              f"A rel {ea:.2e}, BB^T rel {eb:.2e}")
        assert ea < TOL_A and eb < TOL_BBT
        assert dt < 5.0

