"""FFT phase screens on the GB300 (drop-in for ``pyturb.PhaseScreen``).

Host side (FP64, once per configuration, as in the reference): the von Karman
PSD amplitude filter with band-integrated near-DC cells and the 3x3-per-level
subharmonic tables (``src/pyturb/fourier.py:131-228``). Device side, one
native call per :meth:`PhaseScreen.generate`: noise x filter, the 2-D inverse
FFT with the Re/Im screen pairing, and the subharmonic sum minus its screen
mean fused into the transform's last pass (``src/pyturb/fourier.py:233-282``).
"""

from __future__ import annotations

import ctypes as C
from functools import lru_cache
from typing import Any, Optional, Tuple

import numpy as np

from . import _lib
from .backend import NoiseStream, cuda_device, dptr, stream_handle, torch_module, upload
from .config import ScreenConfig

__all__ = ["PhaseScreen", "psd", "amplitude_table", "subharmonic_tables", "Grid"]


def psd(f_squared, r0: float, L0: float, power_law: float = 11.0 / 3.0,
        inner_scale: float = 0.0):
    """Modified von Karman phase PSD [rad^2 m^2] (``src/pyturb/fourier.py:131-149``):
    ``0.023 r0^{-5/3} (f^2 + 1/L0^2)^{-power_law/2} exp(-f^2/fm^2)``."""
    f0_sq = 0.0 if np.isinf(L0) else 1.0 / L0**2
    out = 0.023 * r0 ** (-5.0 / 3.0) * (f_squared + f0_sq) ** (-power_law / 2.0)
    if inner_scale > 0.0:
        fm = 5.92 / (2.0 * np.pi * inner_scale)
        out = out * np.exp(-f_squared / fm**2)
    return out


def band_amplitude(fx: float, fy: float, width: float, r0: float, L0: float,
                   power_law: float, inner_scale: float, samples: int = 33) -> float:
    """Amplitude of one mode standing for a whole frequency cell
    (``src/pyturb/fourier.py:151-172``): ``amp^2 = int(PSD f^2) / f_c^2`` by
    ``samples`` x ``samples`` midpoint quadrature."""
    offsets = ((np.arange(samples) + 0.5) / samples - 0.5) * width
    f_sq = (fx + offsets[:, None]) ** 2 + (fy + offsets[None, :]) ** 2
    p = psd(f_sq, r0, L0, power_law, inner_scale)
    band_power = p.mean() * width**2
    f_sq_eff = (p * f_sq).sum() / p.sum()
    return float(np.sqrt(band_power * f_sq_eff / (fx**2 + fy**2)))


@lru_cache(maxsize=32)
def _unit_amplitude(n: int, dx: float, L0: float, power_law: float,
                    inner_scale: float) -> np.ndarray:
    df = 1.0 / (n * dx)
    f = np.fft.fftfreq(n, d=dx)
    f_sq = f[:, None] ** 2 + f[None, :] ** 2
    f_sq[0, 0] = 1.0
    amp = np.sqrt(psd(f_sq, 1.0, L0, power_law, inner_scale)) * df
    amp[0, 0] = 0.0
    k_max = min(8, (n - 1) // 2)
    for i in range(-k_max, k_max + 1):
        for j in range(-k_max, k_max + 1):
            if i == 0 and j == 0:
                continue
            amp[i, j] = band_amplitude(f[i], f[j], df, 1.0, L0, power_law, inner_scale)
    amp.setflags(write=False)
    return amp


def amplitude_table(n: int, dx: float, r0: float, L0: float, power_law: float = 11.0 / 3.0,
                    inner_scale: float = 0.0) -> np.ndarray:
    """FP64 ``(n, n)`` filter ``sqrt(PSD) df`` with DC zeroed and the
    ``|i|,|j| <= 8`` cells band-integrated (``src/pyturb/fourier.py:174-191``).
    Computed once per (n, dx, L0, shape) at unit r0 and scaled by r0^{-5/6}."""
    return _unit_amplitude(int(n), float(dx), float(L0), float(power_law),
                           float(inner_scale)) * float(r0) ** (-5.0 / 6.0)


@lru_cache(maxsize=32)
def _unit_subharmonics(n: int, dx: float, P: int, L0: float, power_law: float,
                       inner_scale: float) -> Tuple[np.ndarray, np.ndarray]:
    df = 1.0 / (n * dx)
    freqs = np.zeros((P, 3))
    amps = np.zeros((P, 3, 3))
    for p in range(1, P + 1):
        df_p = df / 3.0**p
        f_p = np.array([-1.0, 0.0, 1.0]) * df_p
        freqs[p - 1] = f_p
        for i in range(3):
            for j in range(3):
                if i == 1 and j == 1:
                    continue
                amps[p - 1, i, j] = band_amplitude(f_p[i], f_p[j], df_p, 1.0, L0,
                                                   power_law, inner_scale)
    freqs.setflags(write=False)
    amps.setflags(write=False)
    return freqs, amps


def subharmonic_tables(n: int, dx: float, r0: float, L0: float, P: int,
                       power_law: float = 11.0 / 3.0,
                       inner_scale: float = 0.0) -> Tuple[np.ndarray, np.ndarray]:
    """``(freqs (P, 3), amps (P, 3, 3))``: level p has modes at
    ``{-1, 0, 1} df / 3^p`` with band amplitudes, centre cell excluded
    (``src/pyturb/fourier.py:196-219``)."""
    freqs, amps = _unit_subharmonics(int(n), float(dx), int(P), float(L0), float(power_law),
                                     float(inner_scale))
    return freqs, amps * float(r0) ** (-5.0 / 6.0)


class Grid:
    """Owner of one native ``pt_grid`` plan plus a workspace sized for it."""

    def __init__(self, ns: int, dx: float, sh_freq: np.ndarray, n_layers: int = 1,
                 workspace: bool = True) -> None:
        self._lib = _lib.load()
        torch = torch_module()
        self.device = cuda_device()
        self.ns = int(ns)
        self.dx = float(dx)
        freq = np.ascontiguousarray(sh_freq, dtype=np.float64).reshape(-1, 3)
        self.P = int(freq.shape[0])
        self._freq = freq
        handle = C.c_void_p()
        _lib.call("pt_grid_create", C.byref(handle), self.ns, self.dx, self.P,
                  _lib.as_dptr(freq) if self.P else None)
        self.handle = handle
        self.work_bytes = int(self._lib.pt_grid_workspace_bytes(handle, max(1, int(n_layers))))
        # without a workspace the owner passes a shared one to each call
        self.work = (torch.empty(self.work_bytes, dtype=torch.uint8, device=self.device)
                     if workspace else None)

    def ensure_workspace(self, n_layers: int) -> None:
        """Grow the workspace to what ``n_layers`` layers need (never shrinks)."""
        need = int(self._lib.pt_grid_workspace_bytes(self.handle, max(1, int(n_layers))))
        if need > self.work_bytes:
            torch = torch_module()
            self.work = torch.empty(need, dtype=torch.uint8, device=self.device)
            self.work_bytes = need

    def __del__(self) -> None:
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                self._lib.pt_grid_destroy(h)
            except Exception:
                pass
            self.handle = None


class PhaseScreen:
    """Independent von Karman / Kolmogorov screens (``src/pyturb/fourier.py:31-294``).

    Same constructor and :meth:`generate` contract as the reference; the result
    is a float32 CUDA ``torch.Tensor`` of radians. ``host_noise`` (a factory
    ``seed -> generator``, e.g. ``numpy.random.default_rng``) switches from the
    in-kernel Philox stream to host normals drawn in the reference's order —
    with it, a screen equals the reference's float64 screen for the same seed
    to float32 rounding.
    """

    def __init__(self, n: int, pixel_scale: float, r0: float, L0: float = 25.0,
                 subharmonics: int = 8, power_law: float = 11.0 / 3.0,
                 inner_scale: float = 0.0, seed: Any = None, device: str = "gpu",
                 dtype: Any = "float32", host_noise=None, _stream=None) -> None:
        config = ScreenConfig.create(n, pixel_scale, r0, L0, device, dtype,
                                     finite_outer_scale=False)
        if not isinstance(subharmonics, (int, np.integer)) or subharmonics < 0:
            raise ValueError("subharmonics must be >= 0")
        if subharmonics > 16:
            raise ValueError("subharmonics must be <= 16 on the GPU backend")
        if not np.isfinite(power_law) or power_law <= 2.0:
            raise ValueError("power_law must be > 2 and finite (Kolmogorov is 11/3)")
        if not np.isfinite(inner_scale) or inner_scale < 0:
            raise ValueError("inner_scale must be >= 0 and finite (0 disables it)")
        self.n = config.n
        self.pixel_scale = config.pixel_scale
        self.r0 = config.r0
        self.L0 = config.L0
        self.subharmonics = int(subharmonics)
        self.power_law = float(power_law)
        self.inner_scale = float(inner_scale)
        self.device = config.device
        self.dtype = config.dtype
        self._host_noise_factory = host_noise
        # an extruder's seed screen shares its layer's stream (src/pyturb/extrude.py:408-417)
        self._rng = _stream if _stream is not None else NoiseStream(seed, host_noise)
        amp = amplitude_table(self.n, self.pixel_scale, self.r0, self.L0, self.power_law,
                              self.inner_scale)
        self._sh_freqs, self._sh_amps = subharmonic_tables(
            self.n, self.pixel_scale, self.r0, self.L0, self.subharmonics, self.power_law,
            self.inner_scale)
        self._amplitude_host = amp
        self._grid = Grid(self.n, self.pixel_scale, self._sh_freqs)
        self._amplitude = upload(amp)
        self._sh_amp_dev = upload(self._sh_amps) if self.subharmonics else None

    # -- the native call, shared with Atmosphere.sample ---------------------
    def _generate_into(self, out, count: int, crop: int, n_out: int, scale: float,
                       accumulate: bool) -> None:
        n, P = self.n, self.subharmonics
        noise = sh_noise = None
        if self._rng.injected:
            n_fft = (count + 1) // 2
            noise = upload(self._rng.draw((2, n_fft, n, n)))
            if P:
                sh = np.stack([self._rng.draw((2, count, 3, 3)) for _ in range(P)])
                sh_noise = upload(sh)
        call = self._rng.next_call()
        _lib.call("pt_generate", self._grid.handle, int(count), dptr(self._amplitude),
                  dptr(self._sh_amp_dev), dptr(noise), dptr(sh_noise), self._rng.key, call,
                  int(crop), int(n_out), float(scale), int(bool(accumulate)), dptr(out),
                  dptr(self._grid.work), self._grid.work_bytes, stream_handle())

    def autotune(self, count: int) -> dict:
        """Tune this screen's transform schedule for batches of ``count``
        (radix plan or column variant, cached on disk per device, size and
        batch; results are unchanged beyond float32 rounding). The noise
        stream is left where it was. Needs in-kernel noise."""
        if self._rng.injected:
            raise ValueError("autotune needs in-kernel noise (host_noise draws cannot be replayed)")
        from .tuning import tune_grid

        torch = torch_module()
        count = int(count)
        out = torch.empty((count, self.n, self.n), dtype=torch.float32, device=self._grid.device)
        call = self._rng.call
        try:
            return tune_grid(self._grid, lambda: self._generate_into(out, count, 0, self.n, 1.0,
                                                                     False), count)
        finally:
            self._rng.call = call

    def generate(self, count: Optional[int] = None):
        """``count`` independent screens ``(count, n, n)`` (or one ``(n, n)``)."""
        squeeze = count is None
        count = 1 if squeeze else int(count)
        if count < 1:
            raise ValueError("count must be >= 1")
        torch = torch_module()
        out = torch.empty((count, self.n, self.n), dtype=torch.float32, device=self._grid.device)
        self._generate_into(out, count, 0, self.n, 1.0, False)
        return out[0] if squeeze else out

    @property
    def _f(self) -> np.ndarray:
        return np.fft.fftfreq(self.n, d=self.pixel_scale)

    def __repr__(self) -> str:
        extra = ""
        if self.power_law != 11.0 / 3.0:
            extra += f", power_law={self.power_law}"
        if self.inner_scale > 0.0:
            extra += f", inner_scale={self.inner_scale}"
        return (f"PhaseScreen(n={self.n}, pixel_scale={self.pixel_scale}, r0={self.r0}, "
                f"L0={self.L0}, subharmonics={self.subharmonics}{extra}, "
                f"device={self.device!r}, dtype={self.dtype.name!r})")

