"""One frozen-flow spectral layer (drop-in for ``pyturb.flow.FourierFlowScreen``).

A fixed spectrum realisation evaluated at any continuous translation by the
shift theorem (``src/pyturb/flow.py:34-139``): one native call fills the
spectrum and subharmonic coefficients, one native call per :meth:`translate`
applies the phasors, inverse-transforms and adds the shifted subharmonics.
"""

from __future__ import annotations

from typing import Any

import numpy as np

from . import _lib
from .backend import NoiseStream, dptr, stream_handle, torch_module, upload
from .fourier import Grid, PhaseScreen

__all__ = ["FourierFlowScreen", "SpectralLayers"]


class SpectralLayers:
    """L fixed spectra ``(L, ns, ns)`` complex + subharmonic coefficients
    ``(P, L, 3, 3)`` complex on the device, with the native frame readout.

    The stacked state of ``Atmosphere._build_batched``
    (``src/pyturb/atmosphere.py:532-579``)."""

    def __init__(self, ns: int, dx: float, sh_freq: np.ndarray, amplitudes: np.ndarray,
                 sh_amps: np.ndarray, streams) -> None:
        torch = torch_module()
        self.L = int(amplitudes.shape[0])
        self.ns = int(ns)
        self.P = int(np.asarray(sh_freq).reshape(-1, 3).shape[0])
        self.grid = Grid(ns, dx, sh_freq, n_layers=self.L)
        dev = self.grid.device
        self.amplitude = upload(amplitudes)                     # (L, ns, ns)
        self.sh_amp = upload(sh_amps) if self.P else None        # (P, L, 3, 3)
        self.spectra = torch.empty((self.L, ns, ns, 2), dtype=torch.float32, device=dev)
        self.sh_coef = torch.empty((max(self.P, 1), self.L, 3, 3, 2), dtype=torch.float32,
                                   device=dev)
        self.fill(streams)

    def fill(self, streams) -> None:
        """Draw every layer's realisation: (2, ns, ns) then (2, 3, 3) per level,
        from each layer's own stream (``src/pyturb/flow.py:71-94``)."""
        L, ns, P = self.L, self.ns, self.P
        noise = sh_noise = None
        seeds = np.array([s.next_key() for s in streams], dtype=np.uint64)
        if all(s.injected for s in streams):
            main, sub = [], []
            for s in streams:
                main.append(s.draw((2, ns, ns)))
                sub.append(np.stack([s.draw((2, 3, 3)) for _ in range(P)]) if P else None)
            noise = upload(np.stack(main))
            if P:
                sh_noise = upload(np.stack(sub))
        _lib.call("pt_layers_fill", self.grid.handle, L, dptr(self.amplitude),
                  dptr(self.sh_amp), dptr(noise), dptr(sh_noise),
                  seeds.ctypes.data_as(_lib.C.POINTER(_lib.C.c_uint64)),
                  dptr(self.spectra), dptr(self.sh_coef), stream_handle())

    def frames(self, sx: np.ndarray, sy: np.ndarray, crop: int, n_out: int, scale: float,
               out=None):
        """Layer-summed frames at displacements ``sx, sy`` of shape (F, L) [m]."""
        torch = torch_module()
        sx = np.ascontiguousarray(sx, dtype=np.float64).reshape(-1, self.L)
        sy = np.ascontiguousarray(sy, dtype=np.float64).reshape(-1, self.L)
        F = sx.shape[0]
        if out is None:
            out = torch.empty((F, n_out, n_out), dtype=torch.float32, device=self.grid.device)
        _lib.call("pt_frames", self.grid.handle, self.L, dptr(self.spectra),
                  dptr(self.sh_coef) if self.P else None, F, _lib.as_dptr(sx),
                  _lib.as_dptr(sy), 0, int(crop), int(n_out), float(scale), dptr(out),
                  dptr(self.grid.work), self.grid.work_bytes, stream_handle())
        return out

    def layer_screens(self, sx: np.ndarray, sy: np.ndarray, out=None):
        """Per-layer (uncropped, unscaled) screens ``(L, ns, ns)`` at one shift per layer."""
        torch = torch_module()
        sx = np.ascontiguousarray(sx, dtype=np.float64).reshape(self.L)
        sy = np.ascontiguousarray(sy, dtype=np.float64).reshape(self.L)
        if out is None:
            out = torch.empty((self.L, self.ns, self.ns), dtype=torch.float32,
                              device=self.grid.device)
        _lib.call("pt_frames", self.grid.handle, self.L, dptr(self.spectra),
                  dptr(self.sh_coef) if self.P else None, self.L, _lib.as_dptr(sx),
                  _lib.as_dptr(sy), 1, 0, self.ns, 1.0, dptr(out), dptr(self.grid.work),
                  self.grid.work_bytes, stream_handle())
        return out


class FourierFlowScreen:
    """One frozen layer at arbitrary continuous offsets (``src/pyturb/flow.py:34-139``).

    ``template`` is a :class:`pyturb_gb300.PhaseScreen`; the layer inherits its
    grid, filters and noise mode. :meth:`translate` returns a float32 CUDA
    tensor ``(n, n)`` of radians.
    """

    def __init__(self, template: PhaseScreen, seed: Any = None) -> None:
        self.template = template
        self.n = template.n
        self.pixel_scale = template.pixel_scale
        self.r0 = template.r0
        self.L0 = template.L0
        self.device = template.device
        self.dtype = template.dtype
        self._host_noise = template._host_noise_factory
        self._rng = NoiseStream(seed, self._host_noise)
        self._layers = None
        self.reseed()

    def reseed(self, seed: Any = None) -> "FourierFlowScreen":
        if seed is not None:
            self._rng = NoiseStream(seed, self._host_noise)
        t = self.template
        amp = t._amplitude_host[None]
        sh = t._sh_amps[:, None] if t.subharmonics else np.zeros((0, 1, 3, 3))
        if self._layers is None:
            self._layers = SpectralLayers(self.n, self.pixel_scale, t._sh_freqs, amp, sh,
                                          [self._rng])
        else:
            self._layers.fill([self._rng])
        return self

    def translate(self, sx: float, sy: float):
        """The screen blown by ``(sx, sy)`` metres along axes (0, 1), shape ``(n, n)``."""
        out = self._layers.frames(np.array([[float(sx)]]), np.array([[float(sy)]]), 0,
                                  self.n, 1.0)
        return out[0]

    def __repr__(self) -> str:
        return (f"FourierFlowScreen(n={self.n}, pixel_scale={self.pixel_scale}, "
                f"r0={self.r0}, L0={self.L0}, device={self.device!r})")
