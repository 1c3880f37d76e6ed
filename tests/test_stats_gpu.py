"""Production (in-kernel Philox) screens against turbulence theory, and the
exact frozen-flow identities (seed reproducibility, integer shifts)."""

import warnings

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def structure_function(phase, max_sep):
    phase = np.asarray(phase, dtype=np.float64)
    out = []
    for s in range(1, max_sep + 1):
        a = phase[..., s:, :] - phase[..., :-s, :]
        b = phase[..., :, s:] - phase[..., :, :-s]
        out.append(0.5 * (np.mean(a**2) + np.mean(b**2)))
    return np.arange(1, max_sep + 1), np.array(out)


def test_kolmogorov_structure_function():
    import pyturb_gb300 as G
    from pyturb_gb300.backend import to_numpy

    r0, dx = 0.1, 0.02
    g = G.PhaseScreen(n=256, pixel_scale=dx, r0=r0, L0=np.inf, seed=7)
    screens = to_numpy(g.generate(64))
    sep, d = structure_function(screens, 24)
    theory = 6.88 * (sep * dx / r0) ** (5.0 / 3.0)
    ratio = d[3:] / theory[3:]
    assert np.all(ratio > 0.85) and np.all(ratio < 1.15)
    assert abs(ratio.mean() - 1.0) < 0.08


def test_seed_reproducibility_and_independence():
    import pyturb_gb300 as G
    from pyturb_gb300.backend import to_numpy

    a = to_numpy(G.PhaseScreen(n=64, pixel_scale=0.05, r0=0.1, seed=42).generate(3))
    b = to_numpy(G.PhaseScreen(n=64, pixel_scale=0.05, r0=0.1, seed=42).generate(3))
    c = to_numpy(G.PhaseScreen(n=64, pixel_scale=0.05, r0=0.1, seed=43).generate(3))
    np.testing.assert_array_equal(a, b)
    assert not np.array_equal(a, c)
    batch = to_numpy(G.PhaseScreen(n=32, pixel_scale=0.02, r0=0.1, seed=1).generate(400))
    flat = batch.reshape(400, -1).astype(np.float64)
    flat -= flat.mean(axis=1, keepdims=True)
    x, y = flat[0::2], flat[1::2]
    corr = (x * y).sum(1) / np.sqrt((x**2).sum(1) * (y**2).sum(1))
    assert abs(corr.mean()) < 0.1


def test_von_karman_saturation():
    import pyturb_gb300 as G
    from pyturb_gb300.backend import to_numpy

    r0, dx = 0.1, 0.02
    screens = to_numpy(G.PhaseScreen(n=256, pixel_scale=dx, r0=r0, L0=1.0, seed=3).generate(16))
    sep, d = structure_function(screens, 60)
    assert d[-1] < 0.5 * 6.88 * (sep[-1] * dx / r0) ** (5.0 / 3.0)
    assert d[-1] == pytest.approx(2.0 * 0.0863 * (1.0 / r0) ** (5.0 / 3.0), rel=0.35)


def test_integer_pixel_translation_is_a_roll():
    import pyturb_gb300 as G
    from pyturb_gb300.backend import to_numpy

    warnings.simplefilter("ignore")
    t = G.PhaseScreen(n=128, pixel_scale=0.05, r0=0.1, subharmonics=0, seed=2)
    f = G.FourierFlowScreen(t, seed=4)
    a = to_numpy(f.translate(0.0, 0.0))
    b = to_numpy(f.translate(3 * 0.05, -2 * 0.05))
    np.testing.assert_allclose(b, np.roll(a, (-3, 2), axis=(0, 1)), atol=2e-5 * np.abs(a).max())


def test_sample_structure_function_matches_total_r0():
    import pyturb_gb300 as G
    from pyturb_gb300.backend import to_numpy

    lys = [G.Layer(0, 0.6, 10, 0, L0=np.inf), G.Layer(5000, 0.4, 20, 90, L0=np.inf)]
    atm = G.Atmosphere(lys, r0=0.15, n=256, diameter=5.12, subharmonics=8, seed=4)
    opd = to_numpy(atm.sample(48))
    phase = opd * (2 * np.pi / 500e-9)
    sep, d = structure_function(phase, 20)
    theory = 6.88 * (sep * atm.pixel_scale / atm.r0) ** (5.0 / 3.0)
    ratio = d[3:] / theory[3:]
    assert abs(ratio.mean() - 1.0) < 0.1


def test_extrude_engine_statistics_and_determinism():
    import pyturb_gb300 as G
    from pyturb_gb300.backend import to_numpy

    lys = [G.Layer(0, 1.0, 10, 35)]
    a = G.Atmosphere(lys, r0=0.15, n=64, diameter=2.0, engine="extrude", seed=3)
    b = G.Atmosphere(lys, r0=0.15, n=64, diameter=2.0, engine="extrude", seed=3)
    fa = [to_numpy(f) for _, f in a.frames(dt=0.01, steps=5)]
    fb = [to_numpy(f) for _, f in b.frames(dt=0.01, steps=5)]
    for x, y in zip(fa, fb):
        np.testing.assert_array_equal(x, y)
    assert np.std(fa[-1]) > 0
