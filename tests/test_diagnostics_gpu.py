"""Device diagnostics against the float64 oracle."""

import numpy as np
import pytest

from oracle import diagnostics as od

pytestmark = pytest.mark.gpu


def _stack(seed, shape):
    rng = np.random.default_rng(seed)
    return rng.standard_normal(shape).cumsum(axis=-2).cumsum(axis=-1).astype(np.float32)


@pytest.mark.parametrize("shape,ms", [((8, 96, 96), None), ((6, 64, 80), 63), ((1, 33, 33), 1),
                                      ((4, 512, 512), 128)])
def test_structure_function(shape, ms):
    from pyturb_gb300.analysis import structure_function

    ph = _stack(1, shape)
    r, D = structure_function(ph, 0.02, ms)
    r2, D2 = od.structure_function(ph.astype(np.float64), 0.02, ms)
    np.testing.assert_allclose(r, r2)
    np.testing.assert_allclose(D, D2, rtol=1e-6)


def test_structure_function_on_a_device_tensor_of_a_single_screen():
    import torch

    from pyturb_gb300.analysis import structure_function

    ph = _stack(2, (1, 64, 64))[0]
    r, D = structure_function(torch.tensor(ph, device="cuda"))
    np.testing.assert_allclose(D, od.structure_function(ph.astype(np.float64))[1], rtol=1e-6)


@pytest.mark.parametrize("n,modes,count", [(64, 21, 5), (128, 36, 1), (255, 10, 3)])
def test_zernike_decompose(n, modes, count):
    from pyturb_gb300.analysis import zernike_decompose

    ph = _stack(3, (count, n, n))
    ph /= np.abs(ph).max()
    got = zernike_decompose(ph if count > 1 else ph[0], modes)
    want = od.zernike_decompose(ph.astype(np.float64) if count > 1 else ph[0].astype(np.float64),
                                modes)
    np.testing.assert_allclose(got, want, rtol=2e-4, atol=2e-5 * np.abs(want).max())


@pytest.mark.parametrize("shape", [(50, 200), (3, 7, 97), (2, 4096), (9, 2000)])
def test_temporal_psd(shape):
    from pyturb_gb300.analysis import temporal_psd

    x = np.random.default_rng(4).standard_normal(shape).cumsum(axis=-1).astype(np.float32)
    f, p = temporal_psd(x, 1e-3)
    f2, p2 = od.temporal_psd(x.astype(np.float64), 1e-3)
    np.testing.assert_allclose(f, f2)
    np.testing.assert_allclose(p, p2, rtol=2e-4, atol=1e-6 * p2.max())


def test_argument_errors():
    from pyturb_gb300.analysis import structure_function, temporal_psd

    with pytest.raises(ValueError):
        structure_function(np.zeros((16, 16), np.float32), max_separation=16)
    with pytest.raises(ValueError):
        temporal_psd(np.zeros(10, np.float32), 0.0)
