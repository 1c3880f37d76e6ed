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
