"""Scalar optics helpers used by the OPD conversion.

``Atmosphere._to_opd`` (``src/pyturb/atmosphere.py:764-799``) turns phase at
the reference wavelength into OPD or into phase at another wavelength, with an
optional chromatic scale from published dispersion formulas (restated here):
Edlen (1966) for dry air and Ciddor (1996) for the water-vapour shape
(``src/pyturb/utils.py:25-116``). All host-side FP64 scalars.
"""

from __future__ import annotations

from typing import Optional

import numpy as np

ARCSEC_TO_RAD = np.pi / (180.0 * 3600.0)


def air_refractivity(wavelength: float) -> float:
    """Dry-air ``n - 1`` (Edlen 1966): ``1e-8 (8342.13 + 2406030/(130 - s^2) +
    15997/(38.9 - s^2))`` with ``s = 1/lambda`` in inverse microns."""
    s2 = (1.0 / (float(wavelength) * 1e6)) ** 2
    return (8342.13 + 2406030.0 / (130.0 - s2) + 15997.0 / (38.9 - s2)) * 1e-8


def water_vapour_refractivity(wavelength: float) -> float:
    """Water-vapour dispersion shape (Ciddor 1996): ``1.022e-8 (295.235 +
    2.6422 s^2 - 0.032380 s^4 + 0.004028 s^6)``."""
    s2 = (1.0 / (float(wavelength) * 1e6)) ** 2
    return 1.022e-8 * (295.235 + 2.6422 * s2 - 0.032380 * s2**2 + 0.004028 * s2**3)


def seeing_from_r0(r0: float, wavelength: float = 500e-9) -> float:
    return 0.98 * wavelength / r0 / ARCSEC_TO_RAD


def r0_at_wavelength(r0: float, wavelength_in: float, wavelength_out: float) -> float:
    return r0 * (wavelength_out / wavelength_in) ** (6.0 / 5.0)


def chromatic_scale(dispersion: Optional[str], wet_fraction: float, ref_wavelength: float,
                    wavelength: float) -> float:
    """OPD scale from the reference wavelength to ``wavelength``
    (``src/pyturb/atmosphere.py:780-799``)."""
    if dispersion is None:
        return 1.0
    dry = air_refractivity(wavelength) / air_refractivity(ref_wavelength)
    if dispersion == "edlen":
        return dry
    wet = water_vapour_refractivity(wavelength) / water_vapour_refractivity(ref_wavelength)
    return (1.0 - wet_fraction) * dry + wet_fraction * wet


def output_scale(ref_wavelength: float, wavelength: Optional[float],
                 dispersion: Optional[str] = None, wet_fraction: float = 0.0) -> float:
    """Factor from phase [rad] at ``ref_wavelength`` to OPD [m] (``wavelength``
    None) or to phase [rad] at ``wavelength`` (``src/pyturb/atmosphere.py:764-778``)."""
    scale = ref_wavelength / (2.0 * np.pi)
    if wavelength is None:
        return scale
    wl = float(wavelength)
    return scale * chromatic_scale(dispersion, wet_fraction, ref_wavelength, wl) * (2.0 * np.pi / wl)
