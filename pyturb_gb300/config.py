"""Argument validation, performed before any device work.

Same contract as the reference's frozen configuration dataclasses
(``src/pyturb/config.py:21-416``): every argument error is a ``ValueError``
raised before the GPU is touched, with the same conditions. One deliberate
difference: the arithmetic type is float32 only (``dtype="float64"`` is
refused — FP64 on the GB300 runs at a small fraction of the FP32 rate, and the
float64 results of the reference are this package's parity oracle instead).
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import Any, Optional, Sequence, Tuple, Union

import numpy as np

from .backend import check_device
from .profiles import Layer, _fractions


def r0_from_seeing(seeing: float, wavelength: float = 500e-9) -> float:
    """Fried parameter [m] from seeing FWHM [arcsec]: ``FWHM = 0.98 lambda / r0``
    (``src/pyturb/utils.py:137-142``)."""
    return 0.98 * wavelength / (seeing * np.pi / (180.0 * 3600.0))


def _check_dtype(dtype: Any) -> np.dtype:
    try:
        d = np.dtype(dtype)
    except TypeError as exc:
        raise ValueError("dtype must be float32") from exc
    if d == np.dtype("float64"):
        raise ValueError(
            "dtype must be float32: pyturb_gb300 computes in float32 on the GPU "
            "(use pyturb's CPU path for float64)"
        )
    if d != np.dtype("float32"):
        raise ValueError("dtype must be float32")
    return d


@dataclass(frozen=True)
class GridConfig:
    """``src/pyturb/config.py:21-45``."""

    n: int
    pixel_scale: float
    device: str
    dtype: np.dtype

    @classmethod
    def create(cls, n: int, pixel_scale: float, device: str, dtype: Any) -> "GridConfig":
        if not isinstance(n, (int, np.integer)) or isinstance(n, bool) or n < 2:
            raise ValueError("n must be an integer of at least 2")
        if not np.isfinite(pixel_scale) or pixel_scale <= 0:
            raise ValueError("pixel_scale must be positive and finite")
        d = _check_dtype(dtype)
        return cls(int(n), float(pixel_scale), check_device(device), d)


@dataclass(frozen=True)
class ScreenConfig:
    """``src/pyturb/config.py:69-116``."""

    n: int
    pixel_scale: float
    r0: float
    L0: float
    device: str
    dtype: np.dtype

    @classmethod
    def create(cls, n, pixel_scale, r0, L0, device, dtype, *, finite_outer_scale: bool):
        grid = GridConfig.create(n, pixel_scale, device, dtype)
        if not np.isfinite(r0) or r0 <= 0:
            raise ValueError("r0 must be positive and finite")
        outer = np.inf if L0 is None else L0
        if np.isnan(outer) or outer <= 0:
            raise ValueError("L0 must be positive (use numpy.inf for Kolmogorov)")
        if finite_outer_scale and not np.isfinite(outer):
            raise ValueError("InfinitePhaseScreen requires a finite positive outer scale L0")
        return cls(grid.n, grid.pixel_scale, float(r0), float(outer), grid.device, grid.dtype)


@dataclass(frozen=True)
class LayerConfig:
    altitude: float
    cn2_fraction: float
    wind_speed: float
    wind_direction: float
    L0: float

    def to_layer(self) -> Layer:
        return Layer(self.altitude, self.cn2_fraction, self.wind_speed,
                     self.wind_direction, self.L0)


@dataclass(frozen=True)
class AtmosphereConfig:
    """``src/pyturb/config.py:119-293``."""

    layers: Tuple[LayerConfig, ...]
    r0_zenith: float
    wavelength: float
    zenith_angle: float
    diameter: float
    grid: GridConfig
    L0_override: Optional[float]
    power_law: float
    inner_scale: float
    subharmonics: int
    field_of_view: float
    tau_boil: Tuple[float, ...]
    has_tau_boil: bool
    engine: str
    interp: str
    lgs_altitude: Optional[float]
    dispersion: Optional[str]
    wet_fraction: float
    seed: Optional[int]

    @classmethod
    def create(cls, layers, r0, seeing, wavelength, zenith_angle, diameter, n, L0,
               power_law, inner_scale, subharmonics, field_of_view, tau_boil, engine,
               interp, lgs_altitude, dispersion, wet_fraction, device, dtype, seed):
        model_layers = list(layers)
        if not model_layers:
            raise ValueError("at least one layer is required")
        if (r0 is None) == (seeing is None):
            raise ValueError("give exactly one of r0 or seeing")
        if not np.isfinite(wavelength) or wavelength <= 0:
            raise ValueError("wavelength must be positive and finite [m]")
        if not np.isfinite(zenith_angle) or not 0.0 <= zenith_angle < 90.0:
            raise ValueError("zenith_angle must be in [0, 90) degrees")
        if not np.isfinite(diameter) or diameter <= 0:
            raise ValueError("diameter must be positive and finite")
        if not isinstance(n, (int, np.integer)) or isinstance(n, bool) or n < 2:
            raise ValueError("n must be an integer of at least 2")
        grid = GridConfig.create(n, float(diameter) / n, device, dtype)
        if not np.isfinite(field_of_view) or field_of_view < 0:
            raise ValueError("field_of_view must be finite and >= 0 arcsec")
        if engine not in ("spectral", "extrude"):
            raise ValueError("engine must be 'spectral' or 'extrude'")
        if interp not in ("cubic", "linear", "lanczos"):
            raise ValueError("interp must be 'cubic', 'linear', or 'lanczos'")
        if not np.isfinite(power_law) or power_law <= 2.0:
            raise ValueError("power_law must be > 2 and finite (Kolmogorov is 11/3)")
        if not np.isfinite(inner_scale) or inner_scale < 0:
            raise ValueError("inner_scale must be >= 0 and finite (0 disables it)")
        if not isinstance(subharmonics, (int, np.integer)) or subharmonics < 0:
            raise ValueError("subharmonics must be an integer >= 0")
        if subharmonics > 16:
            raise ValueError("subharmonics must be <= 16 on the GPU backend")
        if L0 is not None and (np.isnan(L0) or L0 <= 0):
            raise ValueError("L0 override must be positive (use numpy.inf for Kolmogorov)")
        if engine == "extrude" and power_law != 11.0 / 3.0:
            raise ValueError(
                "non-Kolmogorov power_law requires engine='spectral': the extruder's "
                "recurrence is the closed-form von Karman conditional distribution "
                "(power_law=11/3)."
            )
        if engine == "extrude" and inner_scale > 0:
            raise ValueError(
                "inner_scale requires engine='spectral': the extruder's covariance "
                "has no inner-scale term."
            )
        if lgs_altitude is not None and (not np.isfinite(lgs_altitude) or lgs_altitude <= 0):
            raise ValueError("lgs_altitude must be positive and finite [m]")
        if dispersion not in (None, "edlen", "ciddor"):
            raise ValueError("dispersion must be None, 'edlen', or 'ciddor'")
        if not np.isfinite(wet_fraction) or not 0.0 <= wet_fraction <= 1.0:
            raise ValueError("wet_fraction must be finite and in [0, 1]")
        if wet_fraction > 0.0 and dispersion != "ciddor":
            raise ValueError("wet_fraction > 0 requires dispersion='ciddor'")
        if seeing is not None:
            if not np.isfinite(seeing) or seeing <= 0:
                raise ValueError("seeing must be positive and finite [arcsec]")
            r0 = r0_from_seeing(seeing, wavelength)
        if not np.isfinite(r0) or r0 <= 0:
            raise ValueError("r0 (or the r0 implied by seeing) must be positive and finite [m]")
        fractions = _fractions(model_layers)
        configured = tuple(
            LayerConfig(
                altitude=layer.altitude,
                cn2_fraction=float(fraction),
                wind_speed=layer.wind_speed,
                wind_direction=layer.wind_direction,
                L0=layer.L0 if L0 is None else float(L0),
            )
            for layer, fraction in zip(model_layers, fractions)
        )
        if engine == "extrude" and any(not np.isfinite(ly.L0) for ly in configured):
            raise ValueError(
                "engine='extrude' requires a finite outer scale L0 for every layer"
            )
        if tau_boil is None:
            tau = np.full(len(configured), np.inf)
        else:
            tau = np.broadcast_to(np.asarray(tau_boil, dtype=np.float64),
                                  (len(configured),)).astype(np.float64)
        if np.any(~np.isfinite(tau) & ~np.isinf(tau)) or np.any(tau <= 0):
            raise ValueError("tau_boil must be positive (or None for frozen flow)")
        return cls(
            layers=configured, r0_zenith=float(r0), wavelength=float(wavelength),
            zenith_angle=float(zenith_angle), diameter=float(diameter), grid=grid,
            L0_override=None if L0 is None else float(L0), power_law=float(power_law),
            inner_scale=float(inner_scale), subharmonics=int(subharmonics),
            field_of_view=float(field_of_view), tau_boil=tuple(float(v) for v in tau),
            has_tau_boil=tau_boil is not None, engine=engine, interp=interp,
            lgs_altitude=None if lgs_altitude is None else float(lgs_altitude),
            dispersion=dispersion, wet_fraction=float(wet_fraction), seed=seed,
        )


@dataclass(frozen=True)
class ExtrusionConfig:
    """``src/pyturb/config.py:296-416``."""

    grid: GridConfig
    layer_r0: Tuple[float, ...]
    layer_L0: Tuple[float, ...]
    layer_wind: Tuple[Tuple[float, float], ...]
    layer_altitude_los: Tuple[float, ...]
    field_of_view_pix: Tuple[float, ...]
    stencil_rows: int
    interp: str
    lgs_altitude_los: Optional[float]
    seeds: Tuple[Any, ...]
    tau_boil: Tuple[float, ...]
    boil_seed: Optional[Any]

    @classmethod
    def create(cls, n, pixel_scale, layer_r0, layer_L0, layer_wind, layer_altitude_los,
               field_of_view_pix, stencil_rows, interp, lgs_altitude_los, device, dtype,
               seeds, tau_boil, boil_seed):
        grid = GridConfig.create(n, pixel_scale, device, dtype)
        r0s = tuple(float(v) for v in layer_r0)
        L0s = tuple(float(v) for v in layer_L0)
        winds = tuple((float(vx), float(vy)) for vx, vy in layer_wind)
        alts = tuple(float(v) for v in layer_altitude_los)
        nl = len(r0s)
        if nl == 0:
            raise ValueError("at least one extrusion layer is required")
        if not (len(L0s) == len(winds) == len(alts) == nl):
            raise ValueError(
                "layer_r0, layer_L0, layer_wind and layer_altitude_los must have equal "
                f"length (got {nl}, {len(L0s)}, {len(winds)}, {len(alts)})"
            )
        if any(not np.isfinite(v) or v <= 0 for v in r0s):
            raise ValueError("every layer_r0 value must be positive and finite")
        if any(not np.isfinite(v) or v <= 0 for v in L0s):
            raise ValueError("every layer_L0 value must be positive and finite")
        if any(not np.isfinite(v) for w in winds for v in w):
            raise ValueError("every layer_wind component must be finite")
        if any(not np.isfinite(v) for v in alts):
            raise ValueError("every layer_altitude_los value must be finite")
        if np.ndim(field_of_view_pix) == 0:
            fov = (float(field_of_view_pix),) * nl
        else:
            fov = tuple(float(v) for v in field_of_view_pix)
        if len(fov) != nl:
            raise ValueError("field_of_view_pix must be scalar or one value per layer")
        if any(not np.isfinite(v) or v < 0 for v in fov):
            raise ValueError("field_of_view_pix values must be finite and >= 0")
        if (not isinstance(stencil_rows, (int, np.integer)) or isinstance(stencil_rows, bool)
                or not 1 <= stencil_rows < grid.n):
            raise ValueError("stencil_rows must be in [1, n)")
        if interp not in ("cubic", "linear", "lanczos"):
            raise ValueError("interp must be 'cubic', 'linear', or 'lanczos'")
        if lgs_altitude_los is not None and (
            not np.isfinite(lgs_altitude_los) or lgs_altitude_los <= 0
        ):
            raise ValueError("lgs_altitude_los must be positive and finite")
        if lgs_altitude_los is not None and any(a >= lgs_altitude_los for a in alts):
            raise ValueError("lgs_altitude_los must exceed every layer altitude")
        if seeds is None:
            seed_values = (None,) * nl
        else:
            seed_values = tuple(seeds)
            if len(seed_values) != nl:
                raise ValueError("seeds must contain one value per layer")
        if tau_boil is None:
            taus = (float("inf"),) * nl
        elif np.ndim(tau_boil) == 0:
            taus = (float(tau_boil),) * nl
        else:
            taus = tuple(float(v) for v in tau_boil)
            if len(taus) != nl:
                raise ValueError("tau_boil must be scalar or one value per layer")
        if any(np.isnan(v) or v <= 0 for v in taus):
            raise ValueError("tau_boil values must be positive")
        return cls(grid, r0s, L0s, winds, alts, fov, int(stencil_rows), interp,
                   None if lgs_altitude_los is None else float(lgs_altitude_los),
                   seed_values, taus, boil_seed)
