"""Argument validation happens before any device work (runs without a GPU)."""

import numpy as np
import pytest

import pyturb_gb300 as G


def test_phase_screen_validation():
    with pytest.raises(ValueError, match="integer"):
        G.PhaseScreen(n=1, pixel_scale=0.01, r0=0.1)
    with pytest.raises(ValueError, match="integer"):
        G.PhaseScreen(n=32.0, pixel_scale=0.01, r0=0.1)
    with pytest.raises(ValueError, match="pixel_scale"):
        G.PhaseScreen(n=32, pixel_scale=-1, r0=0.1)
    with pytest.raises(ValueError, match="L0"):
        G.PhaseScreen(n=32, pixel_scale=0.01, r0=0.1, L0=-5)
    with pytest.raises(ValueError, match="r0"):
        G.PhaseScreen(n=32, pixel_scale=0.01, r0=0.0)
    with pytest.raises(ValueError, match="dtype"):
        G.PhaseScreen(n=32, pixel_scale=0.01, r0=0.1, dtype="int32")
    with pytest.raises(ValueError, match="dtype"):
        G.PhaseScreen(n=32, pixel_scale=0.01, r0=0.1, dtype="float16")
    with pytest.raises(ValueError, match="float32"):
        G.PhaseScreen(n=32, pixel_scale=0.01, r0=0.1, dtype="float64")
    with pytest.raises(ValueError, match="subharmonics"):
        G.PhaseScreen(n=32, pixel_scale=0.01, r0=0.1, subharmonics=-1)
    with pytest.raises(ValueError, match="power_law"):
        G.PhaseScreen(n=32, pixel_scale=0.01, r0=0.1, power_law=2.0)
    with pytest.raises(ValueError, match="inner_scale"):
        G.PhaseScreen(n=32, pixel_scale=0.01, r0=0.1, inner_scale=-1.0)


def test_cpu_device_is_refused():
    with pytest.raises(ValueError, match="CPU"):
        G.PhaseScreen(n=32, pixel_scale=0.01, r0=0.1, device="cpu")
    with pytest.raises(ValueError, match="Unknown device"):
        G.PhaseScreen(n=32, pixel_scale=0.01, r0=0.1, device="tpu")


def test_infinite_validation():
    with pytest.raises(ValueError, match="finite"):
        G.InfinitePhaseScreen(n=32, pixel_scale=0.01, r0=0.1, L0=np.inf)
    with pytest.raises(ValueError, match="stencil_rows"):
        G.InfinitePhaseScreen(n=32, pixel_scale=0.01, r0=0.1, stencil_rows=0)
    with pytest.raises(ValueError, match="interp"):
        G.InfinitePhaseScreen(n=32, pixel_scale=0.01, r0=0.1, interp="nearest")


def test_atmosphere_validation():
    lys = [G.Layer(0.0, 1.0)]
    with pytest.raises(ValueError, match="exactly one"):
        G.Atmosphere(lys)
    with pytest.raises(ValueError, match="exactly one"):
        G.Atmosphere(lys, r0=0.1, seeing=0.8)
    with pytest.raises(ValueError, match="zenith"):
        G.Atmosphere(lys, r0=0.1, zenith_angle=90.0)
    with pytest.raises(ValueError, match="engine"):
        G.Atmosphere(lys, r0=0.1, engine="fast")
    with pytest.raises(ValueError, match="power_law"):
        G.Atmosphere(lys, r0=0.1, engine="extrude", power_law=3.0)
    with pytest.raises(ValueError, match="inner_scale"):
        G.Atmosphere(lys, r0=0.1, engine="extrude", inner_scale=0.01)
    with pytest.raises(ValueError, match="finite outer scale"):
        G.Atmosphere([G.Layer(0.0, 1.0, L0=np.inf)], r0=0.1, engine="extrude")
    with pytest.raises(ValueError, match="wet_fraction"):
        G.Atmosphere(lys, r0=0.1, wet_fraction=0.2)
    with pytest.raises(ValueError, match="tau_boil"):
        G.Atmosphere(lys, r0=0.1, tau_boil=-1.0)
    with pytest.raises(ValueError, match="at least one layer"):
        G.Atmosphere([], r0=0.1)
    with pytest.raises(ValueError, match="cn2_fraction"):
        G.Atmosphere([G.Layer(0.0, -1.0)], r0=0.1)


def test_extruded_validation():
    common = dict(layer_r0=[0.15], layer_L0=[25.0], layer_wind=[(1.0, 0.0)],
                  layer_altitude_los=[0.0])
    with pytest.raises(ValueError, match="integer"):
        G.ExtrudedAtmosphere(n=32.0, pixel_scale=0.1, **common)
    with pytest.raises(ValueError, match="pixel_scale"):
        G.ExtrudedAtmosphere(n=32, pixel_scale=0.0, **common)
    with pytest.raises(ValueError, match="field_of_view_pix"):
        G.ExtrudedAtmosphere(n=32, pixel_scale=0.1, field_of_view_pix=[0.0, 1.0], **common)
    with pytest.raises(ValueError, match="seeds"):
        G.ExtrudedAtmosphere(n=32, pixel_scale=0.1, seeds=[1, 2], **common)
    with pytest.raises(ValueError, match="tau_boil"):
        G.ExtrudedAtmosphere(n=32, pixel_scale=0.1, tau_boil=[0.1, 0.2], **common)
    with pytest.raises(ValueError, match="equal"):
        G.ExtrudedAtmosphere(n=32, pixel_scale=0.1, layer_r0=[0.1, 0.2], layer_L0=[25.0],
                             layer_wind=[(1.0, 0.0)], layer_altitude_los=[0.0])


def test_output_scale_matches_reference_formula():
    from pyturb_gb300.optics import output_scale

    assert output_scale(500e-9, None) == pytest.approx(500e-9 / (2 * np.pi))
    assert output_scale(500e-9, 500e-9) == pytest.approx(1.0)
    # ciddor with no water is edlen
    assert output_scale(500e-9, 1.6e-6, "ciddor", 0.0) == pytest.approx(
        output_scale(500e-9, 1.6e-6, "edlen", 0.0))
