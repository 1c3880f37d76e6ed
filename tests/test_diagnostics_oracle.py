"""The diagnostics oracle against the reference's own functions, and the
product's host Zernike basis against the oracle (CPU)."""

import sys
from pathlib import Path

import numpy as np
import pytest

from oracle import diagnostics as od


def _reference():
    src = Path("/root/reference/src")
    if not src.exists():
        pytest.skip("reference sources not present")
    sys.path.insert(0, str(src))
    try:
        import pyturb.analysis as ra
        import pyturb.utils as ru
    except Exception as exc:  # pragma: no cover
        pytest.skip(f"reference not importable: {exc}")
    finally:
        sys.path.remove(str(src))
    return ra, ru


def test_oracle_matches_reference():
    ra, ru = _reference()
    rng = np.random.default_rng(2)
    ph = rng.standard_normal((3, 40, 40)).cumsum(axis=1)
    r1, d1 = ru.structure_function(ph, 0.1, 9)
    r2, d2 = od.structure_function(ph, 0.1, 9)
    np.testing.assert_allclose(r1, r2)
    np.testing.assert_allclose(d1, d2, rtol=1e-13)
    for j in range(1, 67):
        assert ra.noll_to_zernike(j) == od.noll(j)
    np.testing.assert_allclose(ra.zernike_basis(21, 33), od.zernike_basis(21, 33), atol=1e-12)
    np.testing.assert_allclose(ra.zernike_decompose(ph, 15), od.zernike_decompose(ph, 15),
                               rtol=1e-10, atol=1e-12)
    f1, p1 = ra.temporal_psd(ph, 0.01)
    f2, p2 = od.temporal_psd(ph, 0.01)
    np.testing.assert_allclose(f1, f2)
    np.testing.assert_allclose(p1, p2, rtol=1e-12)


def test_product_basis_matches_oracle():
    from pyturb_gb300 import analysis as pa

    for j in range(1, 91):
        assert pa.noll_to_zernike(j) == od.noll(j)
    np.testing.assert_allclose(pa.zernike_basis(28, 48), od.zernike_basis(28, 48), atol=1e-12)
    np.testing.assert_allclose(pa.zernike_basis(10, 31, 25.0), od.zernike_basis(10, 31, 25.0),
                               atol=1e-12)
