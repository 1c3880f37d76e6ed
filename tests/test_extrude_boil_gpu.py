"""Extrusion boiling with in-kernel noise: decorrelates frames faster than
frozen flow while keeping the screen statistics."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _frames(tau, seed=5, steps=12):
    import warnings

    import pyturb_gb300 as G
    from pyturb_gb300.backend import to_numpy

    warnings.simplefilter("ignore")
    layers = [G.Layer(0.0, 0.7, 4.0, 30.0, 20.0), G.Layer(6000.0, 0.3, 6.0, 200.0, 20.0)]
    atm = G.Atmosphere(layers, r0=0.12, diameter=1.0, n=48, engine="extrude", interp="linear",
                       tau_boil=tau, seed=seed)
    return np.stack([to_numpy(f).astype(np.float64) for _, f in atm.frames(0.01, steps)])


def test_boiling_decorrelates_and_keeps_variance():
    frozen = _frames(None)
    boiled = _frames([0.02, 0.02])

    def corr(a, b):
        a = a - a.mean()
        b = b - b.mean()
        return float((a * b).sum() / np.sqrt((a * a).sum() * (b * b).sum()))

    c_frozen = np.mean([corr(frozen[k], frozen[k + 6]) for k in range(6)])
    c_boiled = np.mean([corr(boiled[k], boiled[k + 6]) for k in range(6)])
    assert c_boiled < c_frozen - 0.2, (c_frozen, c_boiled)
    v_frozen, v_boiled = frozen.var(axis=(1, 2)).mean(), boiled.var(axis=(1, 2)).mean()
    assert 0.3 < v_boiled / v_frozen < 3.0
    assert np.all(np.isfinite(boiled))


def test_frozen_layers_are_untouched_by_other_layers_boiling():
    a = _frames([np.inf, np.inf], steps=4)
    b = _frames(None, steps=4)
    np.testing.assert_array_equal(a, b)
