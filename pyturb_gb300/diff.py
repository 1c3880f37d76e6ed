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

Checkpointed losses (:func:`readout_mse`, :meth:`DifferentiableSpectralFrames.mse`)
never hold the whole frame sequence: the forward keeps only the loss, and the
backward recomputes the frames from the layer state (screens, or spectra =
amplitude x noise) ``frames_per_chunk`` at a time, so memory is one chunk of
frames instead of the sequence and its gradient.
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
                              _ptr(weights), _ptr(fix), _ptr(g), 0, _ptr(gs), s)
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


def _lr_chunk(screens, weights, pos0c, magc, n):
    """Frames (B, Tc, D, n, n) of one time chunk and its fixed-point table."""
    import torch

    B, L, S, _ = screens.shape
    Tc, D = pos0c.shape[0], pos0c.shape[1]
    s = stream_handle()
    fix = torch.empty(3 * Tc * D * L, dtype=torch.int64, device=screens.device)
    _lib.call("pt_lr_fix", Tc, D, L, S, n, _ptr(pos0c), _lib.as_dptr(magc), _ptr(fix), s)
    out = torch.empty((B, Tc, D, n, n), dtype=torch.float32, device=screens.device)
    _lib.call("pt_lr_forward", B, L, S, Tc, D, n, _lib.as_dptr(magc), _ptr(screens),
              _ptr(weights), _ptr(fix), _ptr(out), s)
    return out, fix


class _ReadoutMSEFn:
    """Holder for the checkpointed readout loss (built lazily)."""

    fn = None

    @classmethod
    def get(cls):
        if cls.fn is not None:
            return cls.fn
        import torch

        class ReadoutMSE(torch.autograd.Function):
            @staticmethod
            def forward(ctx, screens, weights, pos0, target, mag, n, chunk):
                B, L, S, S2 = screens.shape
                T, D = pos0.shape[0], pos0.shape[1]
                if S2 != S or tuple(pos0.shape) != (T, D, L, 2) or mag.shape != (D, L):
                    raise ValueError("readout_mse: inconsistent shapes")
                if tuple(target.shape) != (B, T, D, n, n) or target.dtype != torch.float32:
                    raise ValueError("readout_mse: target must be float32 (B, T, D, n, n)")
                if screens.dtype != torch.float32 or weights.dtype != torch.float32:
                    raise ValueError("readout_mse: screens and weights must be float32")
                if pos0.dtype != torch.float64:
                    raise ValueError("readout_mse: pos0 must be float64")
                screens, weights, pos0 = screens.contiguous(), weights.contiguous(), pos0.contiguous()
                magc = np.ascontiguousarray(mag, dtype=np.float64)
                total = torch.zeros((), dtype=torch.float64, device=screens.device)
                for t0 in range(0, T, chunk):
                    t1 = min(T, t0 + chunk)
                    out, _ = _lr_chunk(screens, weights, pos0[t0:t1], magc, n)
                    total += (out - target[:, t0:t1]).double().square().sum()
                ctx.save_for_backward(screens, weights, pos0, target)
                ctx.mag, ctx.n, ctx.chunk = magc, n, chunk
                return (total / target.numel()).float()

            @staticmethod
            def backward(ctx, gl):
                screens, weights, pos0, target = ctx.saved_tensors
                magc, n, chunk = ctx.mag, ctx.n, ctx.chunk
                B, L, S, _ = screens.shape
                T, D = pos0.shape[0], pos0.shape[1]
                s = stream_handle()
                dev = screens.device
                need_s = ctx.needs_input_grad[0]
                need_p = ctx.needs_input_grad[1] or ctx.needs_input_grad[2]
                gs = torch.empty_like(screens) if need_s else None
                gw = torch.zeros(L, dtype=torch.float64, device=dev)
                gp = torch.zeros((T, D, L, 2), dtype=torch.float64, device=dev)
                k = 2.0 / target.numel()
                nb = (n + 63) // 64
                for t0 in range(0, T, chunk):
                    t1 = min(T, t0 + chunk)
                    Tc = t1 - t0
                    out, fix = _lr_chunk(screens, weights, pos0[t0:t1], magc, n)
                    g = ((out - target[:, t0:t1]) * (gl.float() * k)).contiguous()
                    del out
                    if need_s:
                        _lib.call("pt_lr_grad_screens", B, L, S, Tc, D, n, _lib.as_dptr(magc),
                                  _ptr(weights), _ptr(fix), _ptr(g), int(t0 > 0), _ptr(gs), s)
                    if need_p:
                        cnt = int(_lib.load().pt_lr_partial_count(B, L, Tc, D, n))
                        part = torch.empty(cnt, dtype=torch.float32, device=dev)
                        _lib.call("pt_lr_grad_params", B, L, S, Tc, D, n, _lib.as_dptr(magc),
                                  _ptr(screens), _ptr(weights), _ptr(fix), _ptr(g), _ptr(part), s)
                        pv = part.view(B, Tc * D, nb, L, 3).double()
                        gw += pv[..., 0].sum(dim=(0, 1, 2))
                        gp[t0:t1] = pv[..., 1:].sum(dim=(0, 2)).reshape(Tc, D, L, 2)
                return (gs, gw.float() if ctx.needs_input_grad[1] else None,
                        gp if ctx.needs_input_grad[2] else None, None, None, None, None)

        cls.fn = ReadoutMSE
        return cls.fn


def readout_mse(screens, weights, pos0, target, mag, n: int, frames_per_chunk: int = 8):
    """``mean((layer_readout(screens, weights, pos0, mag, n) - target)^2)`` without
    holding the frames: the forward keeps the loss only and the backward
    recomputes ``frames_per_chunk`` time steps at a time (the screens stay the
    checkpoint). Differentiable in ``screens``, ``weights`` and ``pos0``."""
    if int(frames_per_chunk) < 1:
        raise ValueError("frames_per_chunk must be >= 1")
    return _ReadoutMSEFn.get().apply(screens, weights, pos0, target,
                                     np.asarray(mag, np.float64), int(n), int(frames_per_chunk))


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

    def mse(self, screens, weights, winds, target, frames_per_chunk: int = 8):
        """``mean((self(screens, weights, winds) - target)^2)``, checkpointed
        (see :func:`readout_mse`)."""
        return readout_mse(screens, weights, self.positions(winds), target, self.mag, self.n,
                           frames_per_chunk)


def fit_layers(readout: DifferentiableReadout, screens, target, weights0, winds0,
               steps: int = 100, lr: float = 0.01, frames_per_chunk: Optional[int] = None):
    """Adam fit of the per-layer weights and winds to a target OPD sequence
    (mean-squared error). With ``frames_per_chunk`` the loss is the
    checkpointed :meth:`DifferentiableReadout.mse`. Returns ``(weights, winds,
    losses)``."""
    import torch

    w = weights0.detach().clone().float().requires_grad_(True)
    v = winds0.detach().clone().double().requires_grad_(True)
    opt = torch.optim.Adam([w, v], lr=lr)
    losses = []
    for _ in range(int(steps)):
        opt.zero_grad(set_to_none=True)
        if frames_per_chunk:
            loss = readout.mse(screens, w, v, target, frames_per_chunk=int(frames_per_chunk))
        else:
            loss = torch.nn.functional.mse_loss(readout(screens, w, v), target)
        loss.backward()
        opt.step()
        losses.append(float(loss.detach()))
    return w.detach(), v.detach(), losses


# ------------------------------------------------------------- spectral synthesis


def _synth_frames(grid, sw, shc, sx, sy, crop, n_out, scale):
    """Frames (F, n_out, n_out) from weighted spectra ``sw`` (L, ns, ns, 2) and
    weighted subharmonic coefficients ``shc`` (P, L, 3, 3, 2) or None."""
    import torch

    F, L = sx.shape
    out = torch.empty((F, n_out, n_out), dtype=torch.float32, device=sw.device)
    _lib.call("pt_frames", grid.handle, L, _ptr(sw), _ptr(shc) if shc is not None else None, F,
              _lib.as_dptr(sx), _lib.as_dptr(sy), 0, int(crop), int(n_out), float(scale),
              _ptr(out), _ptr(grid.work), grid.work_bytes, stream_handle())
    return out


def _sh_beta(grid):
    """Grid means of the subharmonic basis rows, (P, 3) complex128 (host)."""
    x = (np.arange(grid.ns) - grid.ns / 2.0) * grid.dx
    return np.exp(2j * np.pi * grid._freq[:, :, None] * x[None, None, :]).mean(axis=-1)


class _SynthAdjoint:
    """Accumulates the synthesis VJP over chunks of frames (pt_synth_adj_*):
    spectra, weights, shifts and, with subharmonic levels, the level
    coefficients."""

    def __init__(self, grid, spectra, weights, sh_coef, shifts, crop, n_out, scale, need):
        import torch

        self.torch = torch
        self.grid, self.crop, self.n_out, self.scale = grid, crop, n_out, scale
        self.L, self.ns = spectra.shape[0], spectra.shape[1]
        self.F = shifts.shape[0]
        self.dev = spectra.device
        self.need_S, self.need_p, self.need_c = need
        self.w = weights.contiguous()
        self.sr = torch.view_as_real(spectra.contiguous()).contiguous() if self.need_p else None
        self.shifts = shifts
        self.gSr = (torch.empty((self.L, self.ns, self.ns, 2), dtype=torch.float32,
                                device=self.dev) if self.need_S else None)
        self.gw = torch.zeros(self.L, dtype=torch.float64, device=self.dev)
        self.gsh = torch.zeros((self.F, self.L, 2), dtype=torch.float64, device=self.dev)
        self.sh = sh_coef
        if sh_coef is not None:
            self.fp = torch.as_tensor(grid._freq, dtype=torch.float64, device=self.dev)
            beta = torch.as_tensor(_sh_beta(grid), device=self.dev)
            self.bb = beta[:, :, None] * beta[:, None, :]                       # (P, 3, 3)
            self.cl = sh_coef.detach().to(torch.complex128).permute(1, 0, 2, 3)  # (L, P, 3, 3)
            self.gc = torch.zeros_like(self.cl)
        self.first = True

    def add(self, f0, g):
        """The VJP of frames [f0, f0 + len(g)) for upstream ``g`` (Fc, n_out, n_out)."""
        torch = self.torch
        grid, ns, L = self.grid, self.ns, self.L
        Fc = g.shape[0]
        s = stream_handle()
        g = g.contiguous()
        P2 = (Fc + 1) // 2
        z = torch.empty((P2, ns, ns, 2), dtype=torch.float32, device=self.dev)
        _lib.call("pt_synth_adj_pack", ns, Fc, self.crop, self.n_out, self.scale, _ptr(g), _ptr(z),
                  s)
        _lib.call("pt_ifft2", grid.handle, _ptr(z), _ptr(z), P2, _ptr(grid.work), grid.work_bytes, s)
        sh = self.shifts[f0:f0 + Fc]
        sx, sy = sh[..., 0].contiguous(), sh[..., 1].contiguous()
        ph = torch.empty((L, Fc, 2, ns, 2), dtype=torch.float32, device=self.dev)
        _lib.call("pt_synth_adj_phasors", ns, grid.dx, L, Fc, _ptr(sx), _ptr(sy), _ptr(ph), s)
        if self.need_S:
            _lib.call("pt_synth_adj_spectra", ns, L, Fc, _ptr(self.w), _ptr(z), _ptr(ph),
                      int(not self.first), _ptr(self.gSr), s)
        if self.need_p:
            part = torch.empty((L, Fc, 3), dtype=torch.float64, device=self.dev)
            _lib.call("pt_synth_adj_params", ns, grid.dx, L, Fc, _ptr(self.w), _ptr(self.sr),
                      _ptr(z), _ptr(ph), _ptr(part), s)
            self.gw += part[..., 0].sum(dim=1)
            self.gsh[f0:f0 + Fc] += part[..., 1:].transpose(0, 1)
        if self.sh is not None and (self.need_p or self.need_c):
            P = grid.P
            proj = torch.empty((Fc, 18 * P + 1), dtype=torch.float64, device=self.dev)
            _lib.call("pt_synth_adj_sh", grid.handle, Fc, self.crop, self.n_out, _ptr(g),
                      _ptr(proj), s)
            G = torch.complex(proj[:, 0:18 * P:2], proj[:, 1:18 * P:2]).reshape(Fc, P, 3, 3)
            Q = self.scale * (G - self.bb[None] * proj[:, 18 * P, None, None, None])
            ex = torch.exp(2j * np.pi * sx.double()[:, :, None, None] * self.fp[None, None])
            ey = torch.exp(2j * np.pi * sy.double()[:, :, None, None] * self.fp[None, None])
            E = ex[..., :, None] * ey[..., None, :]                             # (Fc, L, P, 3, 3)
            EQ = E * Q[:, None]
            if self.need_p:
                M = self.cl[None] * EQ
                self.gw += M.real.sum(dim=(0, 2, 3, 4))
                wMi = (self.w.double()[None, :, None, None, None] * M).imag
                self.gsh[f0:f0 + Fc, :, 0] -= 2 * np.pi * torch.einsum("pi,flpij->fl", self.fp, wMi)
                self.gsh[f0:f0 + Fc, :, 1] -= 2 * np.pi * torch.einsum("pj,flpij->fl", self.fp, wMi)
            if self.need_c:
                self.gc += torch.conj(self.w.double()[:, None, None, None] * EQ.sum(dim=0))
        self.first = False

    def grads(self):
        torch = self.torch
        gS = torch.view_as_complex(self.gSr) if self.need_S else None
        gc = (self.gc.permute(1, 0, 2, 3).to(torch.complex64).contiguous()
              if self.sh is not None and self.need_c else None)
        return gS, self.gw.float(), self.gsh, gc


def _synth_inputs(spectra, weights, sh_coef, shifts, grid, who):
    import torch

    L, ns, ns2 = spectra.shape
    F = shifts.shape[0]
    if ns2 != ns or ns != grid.ns:
        raise ValueError(f"{who}: spectra must be (L, ns, ns) on the grid")
    if tuple(shifts.shape) != (F, L, 2) or shifts.dtype != torch.float64:
        raise ValueError(f"{who}: shifts must be float64 (F, L, 2)")
    if spectra.dtype != torch.complex64 or weights.dtype != torch.float32:
        raise ValueError(f"{who}: complex64 spectra, float32 weights")
    if (sh_coef is None) != (grid.P == 0):
        raise ValueError(f"{who}: sh_coef (P, L, 3, 3) must be given exactly when the grid "
                         "has subharmonic levels")
    if sh_coef is not None and (tuple(sh_coef.shape) != (grid.P, L, 3, 3)
                                or sh_coef.dtype != torch.complex64):
        raise ValueError(f"{who}: sh_coef must be complex64 (P, L, 3, 3)")
    grid.ensure_workspace(L)
    wc = weights.to(torch.complex64)
    sw = torch.view_as_real(spectra * wc[:, None, None]).contiguous()
    shc = (torch.view_as_real(sh_coef * wc[None, :, None, None]).contiguous()
           if sh_coef is not None else None)
    sh = shifts.detach().cpu().numpy()
    return sw, shc, np.ascontiguousarray(sh[..., 0]), np.ascontiguousarray(sh[..., 1])


class _SynthFn:
    """Holder for the spectral-synthesis autograd Functions (built lazily)."""

    fn = None
    mse = None

    @classmethod
    def get(cls):
        if cls.fn is not None:
            return cls.fn
        import torch

        class SpectralSynthesis(torch.autograd.Function):
            @staticmethod
            def forward(ctx, spectra, weights, shifts, sh_coef, grid, crop, n_out, scale, chunk):
                sw, shc, sx, sy = _synth_inputs(spectra, weights, sh_coef, shifts, grid,
                                                "spectral_synthesis")
                out = _synth_frames(grid, sw, shc, sx, sy, crop, n_out, scale)
                ctx.save_for_backward(spectra, weights, shifts,
                                      sh_coef if sh_coef is not None else torch.empty(0))
                ctx.has_sh = sh_coef is not None
                ctx.grid, ctx.crop, ctx.n_out, ctx.scale = grid, int(crop), int(n_out), float(scale)
                ctx.chunk = chunk
                return out

            @staticmethod
            def backward(ctx, g):
                spectra, weights, shifts, shc = ctx.saved_tensors
                need = (ctx.needs_input_grad[0],
                        ctx.needs_input_grad[1] or ctx.needs_input_grad[2],
                        ctx.has_sh and ctx.needs_input_grad[3])
                adj = _SynthAdjoint(ctx.grid, spectra, weights, shc if ctx.has_sh else None,
                                    shifts, ctx.crop, ctx.n_out, ctx.scale, need)
                F = shifts.shape[0]
                for f0 in range(0, F, ctx.chunk):
                    adj.add(f0, g[f0:f0 + ctx.chunk])
                gS, gw, gsh, gc = adj.grads()
                return (gS, gw if ctx.needs_input_grad[1] else None,
                        gsh if ctx.needs_input_grad[2] else None, gc,
                        None, None, None, None, None)

        class SynthesisMSE(torch.autograd.Function):
            @staticmethod
            def forward(ctx, spectra, weights, shifts, sh_coef, target, grid, crop, n_out, scale,
                        chunk):
                F = shifts.shape[0]
                if tuple(target.shape) != (F, n_out, n_out) or target.dtype != torch.float32:
                    raise ValueError("synthesis_mse: target must be float32 (F, n_out, n_out)")
                sw, shc, sx, sy = _synth_inputs(spectra, weights, sh_coef, shifts, grid,
                                                "synthesis_mse")
                total = torch.zeros((), dtype=torch.float64, device=spectra.device)
                for f0 in range(0, F, chunk):
                    f1 = min(F, f0 + chunk)
                    out = _synth_frames(grid, sw, shc, sx[f0:f1], sy[f0:f1], crop, n_out, scale)
                    total += (out - target[f0:f1]).double().square().sum()
                ctx.save_for_backward(spectra, weights, shifts,
                                      sh_coef if sh_coef is not None else torch.empty(0), target)
                ctx.has_sh = sh_coef is not None
                ctx.grid, ctx.crop, ctx.n_out, ctx.scale = grid, int(crop), int(n_out), float(scale)
                ctx.chunk = chunk
                return (total / target.numel()).float()

            @staticmethod
            def backward(ctx, gl):
                spectra, weights, shifts, shc, target = ctx.saved_tensors
                grid, chunk = ctx.grid, ctx.chunk
                need = (ctx.needs_input_grad[0],
                        ctx.needs_input_grad[1] or ctx.needs_input_grad[2],
                        ctx.has_sh and ctx.needs_input_grad[3])
                sh_coef = shc if ctx.has_sh else None
                adj = _SynthAdjoint(grid, spectra, weights, sh_coef, shifts, ctx.crop, ctx.n_out,
                                    ctx.scale, need)
                sw, shw, sx, sy = _synth_inputs(spectra, weights, sh_coef, shifts, grid,
                                                "synthesis_mse")
                k = gl.float() * (2.0 / target.numel())
                F = shifts.shape[0]
                for f0 in range(0, F, chunk):   # recompute each chunk of frames
                    f1 = min(F, f0 + chunk)
                    out = _synth_frames(grid, sw, shw, sx[f0:f1], sy[f0:f1], ctx.crop, ctx.n_out,
                                        ctx.scale)
                    adj.add(f0, (out - target[f0:f1]) * k)
                gS, gw, gsh, gc = adj.grads()
                return (gS, gw if ctx.needs_input_grad[1] else None,
                        gsh if ctx.needs_input_grad[2] else None, gc,
                        None, None, None, None, None, None)

        cls.fn = SpectralSynthesis
        cls.mse = SynthesisMSE
        return cls.fn


def spectral_synthesis(spectra, weights, shifts, grid, crop: int, n_out: int, scale: float = 1.0,
                       sh_coef=None, frames_per_chunk: int = 64):
    """``(F, n_out, n_out)`` frames ``scale * crop(Re IDFT(sum_l w_l S_l Phi_fl) + low_f)``,
    differentiable in ``spectra (L, ns, ns)`` complex64, ``weights (L,)``,
    ``shifts (F, L, 2)`` float64 [m] (x along axis 0) and, on a grid with
    subharmonic levels, ``sh_coef (P, L, 3, 3)`` complex64 (``low_f`` the
    zero-mean low-order sum of the reference, ``atmosphere.py:921-935``). The
    backward runs ``frames_per_chunk`` frames at a time."""
    if int(frames_per_chunk) < 1:
        raise ValueError("frames_per_chunk must be >= 1")
    return _SynthFn.get().apply(spectra, weights, shifts, sh_coef, grid, int(crop), int(n_out),
                                float(scale), int(frames_per_chunk))


def synthesis_mse(spectra, weights, shifts, target, grid, crop: int, n_out: int,
                  scale: float = 1.0, sh_coef=None, frames_per_chunk: int = 16):
    """``mean((spectral_synthesis(...) - target)^2)`` without holding the frames:
    the forward keeps the loss only, and the backward recomputes the frames
    from the spectra ``frames_per_chunk`` at a time."""
    if int(frames_per_chunk) < 1:
        raise ValueError("frames_per_chunk must be >= 1")
    _SynthFn.get()
    return _SynthFn.mse.apply(spectra, weights, shifts, sh_coef, target, grid, int(crop),
                              int(n_out), float(scale), int(frames_per_chunk))


class DifferentiableSpectralFrames:
    """Spectral frozen-flow frames differentiable in the layer noise, the
    per-layer weights (sqrt of the Cn2 fractions) and the winds.

    The layers share one ``n_screen`` grid at ``pixel_scale`` and the von
    Karman amplitude of ``r0`` / ``L0`` (``fourier.py:174-228`` of the
    reference); layer ``l``'s spectrum is ``amplitude * noise[l]`` with
    ``noise`` complex N(0, 1), and with ``subharmonics = P`` levels its
    low-order coefficients are ``sh_amp * sh_noise[l]`` (``sh_noise (L, P, 3,
    3)`` complex). Frame ``(t, d)`` displaces layer ``l`` by ``v_l t + alt_l
    theta_d`` (``atmosphere.py:1012-1015``) and is cropped to the central
    ``n x n`` pupil.
    """

    def __init__(self, n: int, n_screen: int, pixel_scale: float, r0: float, L0: float,
                 altitudes: Sequence[float], times, directions=None, scale: float = 1.0,
                 subharmonics: int = 0, device: str = "gpu") -> None:
        import torch

        from .fourier import Grid, amplitude_table, subharmonic_tables

        check_device(device)
        self.device = cuda_device()
        self.n, self.n_screen = int(n), int(n_screen)
        if not 1 <= self.n <= self.n_screen:
            raise ValueError("need 1 <= n <= n_screen")
        if not 0 <= int(subharmonics) <= 16:
            raise ValueError("subharmonics must be in [0, 16]")
        self.pixel_scale = float(pixel_scale)
        self.altitudes = np.asarray(altitudes, np.float64).reshape(-1)
        self.times = np.asarray(times, np.float64).reshape(-1)
        dirs = np.zeros((1, 2)) if directions is None else np.asarray(directions, np.float64)
        self.directions = dirs.reshape(-1, 2)
        self.scale = float(scale)
        self.crop = (self.n_screen - self.n) // 2
        self.P = int(subharmonics)
        freqs, sh_amp = subharmonic_tables(self.n_screen, self.pixel_scale, r0, L0, self.P)
        self.grid = Grid(self.n_screen, self.pixel_scale, freqs if self.P else np.zeros((0, 3)),
                         n_layers=1)
        amp = amplitude_table(self.n_screen, self.pixel_scale, r0, L0)
        self.amplitude = torch.as_tensor(amp, dtype=torch.float32, device=self.device)
        self.sh_amp = (torch.as_tensor(np.asarray(sh_amp).reshape(self.P, 3, 3),
                                       dtype=torch.float32, device=self.device)
                       if self.P else None)
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

    def sh_coef(self, sh_noise):
        """``(P, L, 3, 3)`` level coefficients ``sh_amp * sh_noise`` for
        ``sh_noise (L, P, 3, 3)`` complex, or None without levels."""
        if not self.P:
            if sh_noise is not None:
                raise ValueError("sh_noise given, but the frames have no subharmonic levels")
            return None
        if sh_noise is None:
            raise ValueError("sh_noise (L, P, 3, 3) is required with subharmonic levels")
        return (sh_noise * self.sh_amp.to(sh_noise.dtype)[None]).permute(1, 0, 2, 3)

    def __call__(self, noise, weights, winds, sh_noise=None):
        """``(T * D, n, n)`` frames, frame index ``t * D + d``."""
        return spectral_synthesis(self.spectra(noise), weights, self.shifts(winds), self.grid,
                                  self.crop, self.n, self.scale, self.sh_coef(sh_noise))

    def mse(self, noise, weights, winds, target, sh_noise=None, frames_per_chunk: int = 16):
        """``mean((self(noise, weights, winds, sh_noise) - target)^2)``, checkpointed:
        the frames are recomputed from the noise in the backward
        ``frames_per_chunk`` at a time (see :func:`synthesis_mse`)."""
        return synthesis_mse(self.spectra(noise), weights, self.shifts(winds), target, self.grid,
                             self.crop, self.n, self.scale, self.sh_coef(sh_noise),
                             frames_per_chunk)
