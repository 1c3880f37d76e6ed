"""The turbulent-layer value type the hot path consumes.

Only what the phase-screen path needs is here: the :class:`Layer` record
(``src/pyturb/profiles.py:54-85``) and Cn2-fraction normalisation
(``src/pyturb/profiles.py:608-615``). Named site profiles and the integrated
seeing quantities are host-side scalars outside the GPU path; build a layer
list directly, or pass pyturb's own profile layers (any object with the same
five attributes works).
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import List, Sequence, Tuple

import numpy as np


@dataclass
class Layer:
    """One turbulent layer: altitude [m] at zenith, Cn2 weight, wind speed
    [m/s], wind direction [deg from axis 0 toward axis 1], outer scale [m]."""

    altitude: float
    cn2_fraction: float
    wind_speed: float = 10.0
    wind_direction: float = 0.0
    L0: float = 25.0

    @property
    def wind_vector(self) -> Tuple[float, float]:
        theta = np.deg2rad(self.wind_direction)
        return self.wind_speed * np.cos(theta), self.wind_speed * np.sin(theta)


def _fractions(layers: Sequence) -> np.ndarray:
    frac = np.asarray([layer.cn2_fraction for layer in layers], dtype=np.float64)
    if np.any(frac < 0):
        raise ValueError("cn2_fraction values must be non-negative")
    total = frac.sum()
    if total <= 0:
        raise ValueError("cn2_fraction values must sum to a positive number")
    return frac / total


def as_layers(layers: Sequence) -> List[Layer]:
    """Copy any layer-like objects into :class:`Layer` records."""
    return [Layer(float(ly.altitude), float(ly.cn2_fraction), float(ly.wind_speed),
                  float(ly.wind_direction), float(ly.L0)) for ly in layers]
