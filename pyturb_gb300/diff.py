"""Differentiable multi-layer readout: gradients for fitting Cn2 and winds.

The forward model is the reference spectral engine's LGS cone readout
(``Atmosphere._build_lgs_zoom`` / ``_lgs_zoom``, src/pyturb/atmosphere.py:
581-616, 1048-1090) applied to given layer screens, with the frozen-flow and
direction displacement (``disp = v * t + alt * offset``, atmosphere.py:
1012-1022) done as a periodic bilinear shift so that it is differentiable in
the wind: for screens ``phi (B, L, S, S)`` and per-layer weights ``w``,

    out[b, t, d] = sum_l w_l * phi[b, l](centre + mag_dl * (i - (n-1)/2)
                                         + (v_l t + alt_l theta_d) / dx).

The reference has no gradients; the adjoints here are hand-written kernels
(``pt_lr_grad_screens``: the transpose of the bilinear gather as a
deterministic tile gather; ``pt_lr_grad_params``: block reductions for the
weights and positions) behind :class:`torch.autograd.Function`. Torch carries
the chain rule from positions to winds (a few hundred float64 scalars).
"""

from __future__ import annotations

import math
from typing import Optional, Sequence

import numpy as np

from . import _lib
from .backend import check_device, cuda_device, stream_handle


def _ptr(t) -> int:
    return t.data_ptr()


class _LayerReadoutFn:
    """Holder for the autograd Function (built lazily so that importing the
    package does not import torch)."""

    fn = None

    @classmethod
    def get(cls):
        if cls.fn is not None:
            return cls.fn
        import torch

        class LayerReadout(torch.autograd.Function):
            @staticmethod
            def forward(ctx, screens, weights, pos0, mag, n):
                B, L, S, S2 = screens.shape
                T, D = pos0.shape[0], pos0.shape[1]
                if S2 != S or tuple(pos0.shape) != (T, D, L, 2) or mag.shape != (D, L):
                    raise ValueError("layer_readout: inconsistent shapes")
                if screens.dtype != torch.float32 or weights.dtype != torch.float32:
                    raise ValueError("layer_readout: screens and weights must be float32")
                if pos0.dtype != torch.float64:
                    raise ValueError("layer_readout: pos0 must be float64")
                screens = screens.contiguous()
                weights = weights.contiguous()
                pos0 = pos0.contiguous()
                dev = screens.device
                s = stream_handle()
                magc = np.ascontiguousarray(mag, dtype=np.float64)
                fix = torch.empty(3 * T * D * L, dtype=torch.int64, device=dev)
                _lib.call("pt_lr_fix", T, D, L, S, n, _ptr(pos0), _lib.as_dptr(magc), _ptr(fix), s)
                out = torch.empty((B, T, D, n, n), dtype=torch.float32, device=dev)
                _lib.call("pt_lr_forward", B, L, S, T, D, n, _lib.as_dptr(magc), _ptr(screens),
                          _ptr(weights), _ptr(fix), _ptr(out), s)
                ctx.save_for_backward(screens, weights, fix)
                ctx.mag = magc
                ctx.n = n
                return out

            @staticmethod
            def backward(ctx, g):
                screens, weights, fix = ctx.saved_tensors
                magc, n = ctx.mag, ctx.n
                B, L, S, _ = screens.shape
                D = magc.shape[0]
                T = fix.numel() // (3 * D * L)
                g = g.contiguous()
                dev = g.device
                s = stream_handle()
                gs = gw = gp = None
                if ctx.needs_input_grad[0]:
                    gs = torch.empty_like(screens)
                    _lib.call("pt_lr_grad_screens", B, L, S, T, D, n, _lib.as_dptr(magc),
                              _ptr(weights), _ptr(fix), _ptr(g), _ptr(gs), s)
                if ctx.needs_input_grad[1] or ctx.needs_input_grad[2]:
                    cnt = int(_lib.load().pt_lr_partial_count(B, L, T, D, n))
                    part = torch.empty(cnt, dtype=torch.float32, device=dev)
                    _lib.call("pt_lr_grad_params", B, L, S, T, D, n, _lib.as_dptr(magc),
                              _ptr(screens), _ptr(weights), _ptr(fix), _ptr(g), _ptr(part), s)
                    nb = (n + 63) // 64
                    p = part.view(B, T * D, nb, L, 3).double()
                    if ctx.needs_input_grad[1]:
                        gw = p[..., 0].sum(dim=(0, 1, 2)).float()
                    if ctx.needs_input_grad[2]:
                        gp = p[..., 1:].sum(dim=(0, 2)).reshape(T, D, L, 2)
                return gs, gw, gp, None, None

        cls.fn = LayerReadout
        return cls.fn


def layer_readout(screens, weights, pos0, mag, n: int):
    """``out (B, T, D, n, n)`` from ``screens (B, L, S, S)`` float32,
    ``weights (L,)`` float32, ``pos0 (T, D, L, 2)`` float64 (device) and the
    host magnification table ``mag (D, L)``; differentiable in the first three."""
    return _LayerReadoutFn.get().apply(screens, weights, pos0, np.asarray(mag, np.float64), int(n))


class DifferentiableReadout:
    """Cone-zoomed, wind-shifted readout of layer screens in D directions.

    ``altitudes`` (L,) m along the line of sight; ``directions`` (D, 2) rad
    (x, y) offsets; ``source_altitudes`` (D,) m, ``None`` or ``inf`` for a
    natural guide star (magnification 1), else the LGS cone magnification
    ``1 - h/H`` per layer (atmosphere.py:486-487); ``times`` (T,) s. Screens
    are ``(B, L, n_screen, n_screen)`` at ``pixel_scale`` m/px and the pupil is
    ``n x n`` at the same pixel scale.
    """

    def __init__(self, n: int, n_screen: int, pixel_scale: float, altitudes: Sequence[float],
                 directions, times, source_altitudes: Optional[Sequence] = None,
                 device: str = "gpu") -> None:
        import torch

        self.n = int(n)
        self.n_screen = int(n_screen)
        self.pixel_scale = float(pixel_scale)
        if self.n < 1 or self.n_screen < 2 or not self.pixel_scale > 0:
            raise ValueError("n, n_screen and pixel_scale must be positive")
        self.altitudes = np.asarray(altitudes, np.float64).reshape(-1)
        self.directions = np.asarray(directions, np.float64).reshape(-1, 2)
        self.times = np.asarray(times, np.float64).reshape(-1)
        D, L = self.directions.shape[0], self.altitudes.size
        src = [None] * D if source_altitudes is None else list(source_altitudes)
        if len(src) != D:
            raise ValueError("source_altitudes must give one entry per direction")
        mag = np.ones((D, L))
        for d, H in enumerate(src):
            if H is not None and math.isfinite(float(H)):
                if not float(H) > self.altitudes.max():
                    raise ValueError("a laser guide star must lie above every layer")
                mag[d] = 1.0 - self.altitudes / float(H)
        self.mag = mag
        span = mag.max() * (self.n - 1) + 2.0
        if span >= self.n_screen:
            raise ValueError(f"the pupil footprint ({span:.0f} px) must be smaller than "
                             f"n_screen={self.n_screen}")
        check_device(device)
        self.device = cuda_device()
        dev = self.device
        self._base = torch.as_tensor(
            (self.n_screen - 1) / 2.0 - mag * (self.n - 1) / 2.0, dtype=torch.float64,
            device=dev)                                                     # (D, L)
        self._t = torch.as_tensor(self.times, dtype=torch.float64, device=dev)
        self._alt_th = torch.as_tensor(
            self.altitudes[None, :, None] * self.directions[:, None, :], dtype=torch.float64,
            device=dev)                                                     # (D, L, 2)

    def positions(self, winds):
        """``pos0 (T, D, L, 2)`` float64 from ``winds (L, 2)`` (m/s), differentiable."""
        v = winds.to(self.device, dtype=self._t.dtype)
        disp = v[None, None] * self._t[:, None, None, None] + self._alt_th[None]
        return self._base[None, :, :, None] + disp / self.pixel_scale

    def __call__(self, screens, weights, winds):
        """``out (B, T, D, n, n)`` float32 OPD in the screens' units."""
        return layer_readout(screens, weights, self.positions(winds), self.mag, self.n)


def fit_layers(readout: DifferentiableReadout, screens, target, weights0, winds0,
               steps: int = 100, lr: float = 0.01):
    """Adam fit of the per-layer weights and winds to a target OPD sequence
    (mean-squared error). Returns ``(weights, winds, losses)``."""
    import torch

    w = weights0.detach().clone().float().requires_grad_(True)
    v = winds0.detach().clone().double().requires_grad_(True)
    opt = torch.optim.Adam([w, v], lr=lr)
    losses = []
    for _ in range(int(steps)):
        opt.zero_grad(set_to_none=True)
        loss = torch.nn.functional.mse_loss(readout(screens, w, v), target)
        loss.backward()
        opt.step()
        losses.append(float(loss.detach()))
    return w.detach(), v.detach(), losses


# ------------------------------------------------------------- spectral synthesis


class _SynthFn:
    """Holder for the spectral-synthesis autograd Function (built lazily)."""

    fn = None

    @classmethod
    def get(cls):
        if cls.fn is not None:
            return cls.fn
        import torch

        class SpectralSynthesis(torch.autograd.Function):
            @staticmethod
            def forward(ctx, spectra, weights, shifts, grid, crop, n_out, scale):
                L, ns, ns2 = spectra.shape
                F = shifts.shape[0]
                if ns2 != ns or ns != grid.ns or grid.P != 0:
                    raise ValueError("spectral_synthesis: spectra must be (L, ns, ns) on a grid "
                                     "without subharmonics")
                if tuple(shifts.shape) != (F, L, 2) or shifts.dtype != torch.float64:
                    raise ValueError("spectral_synthesis: shifts must be float64 (F, L, 2)")
                if spectra.dtype != torch.complex64 or weights.dtype != torch.float32:
                    raise ValueError("spectral_synthesis: complex64 spectra, float32 weights")
                s = stream_handle()
                grid.ensure_workspace(L)
                sw = torch.view_as_real(spectra * weights.to(torch.complex64)[:, None, None])
                sw = sw.contiguous()
                sh = shifts.detach().cpu().numpy()
                sx = np.ascontiguousarray(sh[..., 0])
                sy = np.ascontiguousarray(sh[..., 1])
                out = torch.empty((F, n_out, n_out), dtype=torch.float32, device=spectra.device)
                _lib.call("pt_frames", grid.handle, L, _ptr(sw), None, F, _lib.as_dptr(sx),
                          _lib.as_dptr(sy), 0, int(crop), int(n_out), float(scale), _ptr(out),
                          _ptr(grid.work), grid.work_bytes, s)
                ctx.save_for_backward(spectra, weights, shifts)
                ctx.grid, ctx.crop, ctx.n_out, ctx.scale = grid, int(crop), int(n_out), float(scale)
                return out

            @staticmethod
            def backward(ctx, g):
                spectra, weights, shifts = ctx.saved_tensors
                grid = ctx.grid
                L, ns, _ = spectra.shape
                F = shifts.shape[0]
                dev = g.device
                s = stream_handle()
                g = g.contiguous()
                P2 = (F + 1) // 2
                z = torch.empty((P2, ns, ns, 2), dtype=torch.float32, device=dev)
                _lib.call("pt_synth_adj_pack", ns, F, ctx.crop, ctx.n_out, ctx.scale, _ptr(g),
                          _ptr(z), s)
                _lib.call("pt_ifft2", grid.handle, _ptr(z), _ptr(z), P2, _ptr(grid.work),
                          grid.work_bytes, s)
                sx = shifts[..., 0].contiguous()
                sy = shifts[..., 1].contiguous()
                ph = torch.empty((L, F, 2, ns, 2), dtype=torch.float32, device=dev)
                _lib.call("pt_synth_adj_phasors", ns, grid.dx, L, F, _ptr(sx), _ptr(sy), _ptr(ph), s)
                w = weights.contiguous()
                gS = gw = gsh = None
                if ctx.needs_input_grad[0]:
                    gSr = torch.empty((L, ns, ns, 2), dtype=torch.float32, device=dev)
                    _lib.call("pt_synth_adj_spectra", ns, L, F, _ptr(w), _ptr(z), _ptr(ph),
                              _ptr(gSr), s)
                    gS = torch.view_as_complex(gSr)
                if ctx.needs_input_grad[1] or ctx.needs_input_grad[2]:
                    sr = torch.view_as_real(spectra.contiguous()).contiguous()
                    part = torch.empty((L, F, 3), dtype=torch.float64, device=dev)
                    _lib.call("pt_synth_adj_params", ns, grid.dx, L, F, _ptr(w), _ptr(sr), _ptr(z),
                              _ptr(ph), _ptr(part), s)
                    if ctx.needs_input_grad[1]:
                        gw = part[..., 0].sum(dim=1).float()
                    if ctx.needs_input_grad[2]:
                        gsh = part[..., 1:].transpose(0, 1).contiguous()
                return gS, gw, gsh, None, None, None, None

        cls.fn = SpectralSynthesis
        return cls.fn


def spectral_synthesis(spectra, weights, shifts, grid, crop: int, n_out: int, scale: float = 1.0):
    """``(F, n_out, n_out)`` frames ``scale * crop(Re IDFT(sum_l w_l S_l Phi_fl))`` (no
    subharmonics), differentiable in ``spectra (L, ns, ns)`` complex64, ``weights (L,)``
    and ``shifts (F, L, 2)`` float64 [m] (x along axis 0). ``grid`` is a
    :class:`pyturb_gb300.fourier.Grid` built with no subharmonic levels."""
    return _SynthFn.get().apply(spectra, weights, shifts, grid, int(crop), int(n_out),
                                float(scale))


class DifferentiableSpectralFrames:
    """Spectral frozen-flow frames differentiable in the layer noise, the
    per-layer weights (sqrt of the Cn2 fractions) and the winds.

    The layers share one ``n_screen`` grid at ``pixel_scale`` and the von
    Karman amplitude of ``r0`` / ``L0`` (``fourier.py:174-228`` of the
    reference, without subharmonic levels); layer ``l``'s spectrum is
    ``amplitude * noise[l]`` with ``noise`` complex N(0, 1). Frame ``(t, d)``
    displaces layer ``l`` by ``v_l t + alt_l theta_d`` (``atmosphere.py:
    1012-1015``) and is cropped to the central ``n x n`` pupil.
    """

    def __init__(self, n: int, n_screen: int, pixel_scale: float, r0: float, L0: float,
                 altitudes: Sequence[float], times, directions=None, scale: float = 1.0,
                 device: str = "gpu") -> None:
        import torch

        from .fourier import Grid, amplitude_table

        check_device(device)
        self.device = cuda_device()
        self.n, self.n_screen = int(n), int(n_screen)
        if not 1 <= self.n <= self.n_screen:
            raise ValueError("need 1 <= n <= n_screen")
        self.pixel_scale = float(pixel_scale)
        self.altitudes = np.asarray(altitudes, np.float64).reshape(-1)
        self.times = np.asarray(times, np.float64).reshape(-1)
        dirs = np.zeros((1, 2)) if directions is None else np.asarray(directions, np.float64)
        self.directions = dirs.reshape(-1, 2)
        self.scale = float(scale)
        self.crop = (self.n_screen - self.n) // 2
        self.grid = Grid(self.n_screen, self.pixel_scale, np.zeros((0, 3)), n_layers=1)
        amp = amplitude_table(self.n_screen, self.pixel_scale, r0, L0)
        self.amplitude = torch.as_tensor(amp, dtype=torch.float32, device=self.device)
        dev = self.device
        self._t = torch.as_tensor(self.times, dtype=torch.float64, device=dev)
        self._alt_th = torch.as_tensor(
            self.altitudes[None, :, None] * self.directions[:, None, :], dtype=torch.float64,
            device=dev)                                                     # (D, L, 2)

    def shifts(self, winds):
        """``(T * D, L, 2)`` float64 displacements [m] from ``winds (L, 2)``."""
        v = winds.to(self.device, dtype=self._t.dtype)
        disp = v[None, None] * self._t[:, None, None, None] + self._alt_th[None]
        return disp.reshape(-1, self.altitudes.size, 2)

    def spectra(self, noise):
        """``amplitude * noise`` for complex ``noise (L, ns, ns)``."""
        return noise * self.amplitude.to(noise.dtype)[None]

    def __call__(self, noise, weights, winds):
        """``(T * D, n, n)`` frames, frame index ``t * D + d``."""
        return spectral_synthesis(self.spectra(noise), weights, self.shifts(winds), self.grid,
                                  self.crop, self.n, self.scale)
