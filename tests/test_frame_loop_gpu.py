"""The CUDA-graph frame loop: replays at any start time equal direct rendering."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _atm(n=64, chunk=16, seed=4):
    import pyturb_gb300 as G

    layers = [G.Layer(0.0, 0.6, 9.0, 20.0, 25.0), G.Layer(4000.0, 0.25, 17.0, 135.0, 25.0),
              G.Layer(11000.0, 0.15, 28.0, 250.0, 25.0)]
    return G.Atmosphere(layers, r0=0.15, diameter=2.0, n=n, seed=seed, zenith_angle=30.0,
                        frames_chunk=chunk)


def _rel(a, b):
    a = a.double().cpu().numpy()
    b = b.double().cpu().numpy()
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("t0", [0.0, 0.37, 1000.0])
def test_frame_loop_matches_direct_rendering(t0):
    import warnings

    warnings.simplefilter("ignore")
    atm = _atm()
    loop = atm.frame_loop(2e-3, 37)       # 37 frames: three chunks of 16, 16, 5
    got = loop.render(t0).clone()
    want = atm.render(t0 + loop.times)
    assert _rel(got, want) < 2e-6
    # a second replay at another start time reuses the same graph
    got2 = loop.render(t0 + 0.5).clone()
    assert _rel(got2, atm.render(t0 + 0.5 + loop.times)) < 2e-6


def test_frame_loop_reads_the_current_layer_state():
    import warnings

    warnings.simplefilter("ignore")
    atm = _atm(seed=7)
    loop = atm.frame_loop(1e-3, 8)
    a = loop.render(0.1).clone()
    other = _atm(seed=8)
    atm._spec.spectra.copy_(other._spec.spectra)     # a new realisation, same geometry
    atm._spec.sh_coef.copy_(other._spec.sh_coef)
    b = loop.render(0.1).clone()
    assert _rel(b, other.render(0.1 + loop.times)) < 2e-6
    assert _rel(a, b) > 0.1


def test_frame_loop_refuses_unsupported_configurations():
    import pyturb_gb300 as G

    atm = _atm()
    with pytest.raises(ValueError):
        atm.frame_loop(0.0, 4)
    lgs = G.Atmosphere([G.Layer(0.0, 1.0, 5.0, 0.0, 25.0)], r0=0.15, diameter=2.0, n=32,
                       lgs_altitude=90e3, seed=1)
    with pytest.raises(ValueError):
        lgs.frame_loop(1e-3, 4)
