"""Float64 restatement of the weighted spectral frame synthesis and its
vector-Jacobian product (test oracle).

Test infrastructure only: imported by ``tests/`` and nothing on the product
path. The forward is ``Atmosphere._integrate`` without subharmonics
(src/pyturb/atmosphere.py:882-938: per-layer phasors ``exp(2 pi i f s)`` with
``f = fftfreq(ns, dx)``, x along axis 0, summed spectra, ``ifft2 * ns^2``,
real part, crop) with a weight per layer. The reference has no gradients; the
VJP here is the analytic one, checked against float64 central differences and
torch autograd in ``tests/test_synth_diff_oracle.py``.
"""

from __future__ import annotations

import numpy as np


def _phasors(ns, dx, sx, sy):
    f = np.fft.fftfreq(ns, dx)
    px = np.exp(2j * np.pi * f[None, None, :] * np.asarray(sx)[..., None])   # (F, L, ns)
    py = np.exp(2j * np.pi * f[None, None, :] * np.asarray(sy)[..., None])
    return f, px, py


def synth_frames(spectra, w, sx, sy, dx, crop, n_out, scale):
    """``(F, n_out, n_out)``: ``scale * crop(Re(ifft2(sum_l w_l S_l Phi) ns^2))``."""
    S = np.asarray(spectra, np.complex128)
    L, ns, _ = S.shape
    _, px, py = _phasors(ns, dx, sx, sy)
    F = px.shape[0]
    out = np.empty((F, n_out, n_out))
    for f in range(F):
        X = np.einsum("l,lij,li,lj->ij", np.asarray(w, np.float64), S, px[f], py[f])
        y = np.real(np.fft.ifft2(X)) * ns * ns
        out[f] = scale * y[crop:crop + n_out, crop:crop + n_out]
    return out


def synth_vjp(spectra, w, sx, sy, dx, crop, n_out, scale, g):
    """``(dS (L, ns, ns) complex as dL/dRe + i dL/dIm, dw (L,), dsx (F, L), dsy (F, L))``."""
    S = np.asarray(spectra, np.complex128)
    w = np.asarray(w, np.float64)
    L, ns, _ = S.shape
    f, px, py = _phasors(ns, dx, sx, sy)
    F = px.shape[0]
    gS = np.zeros_like(S)
    gw = np.zeros(L)
    gsx = np.zeros((F, L))
    gsy = np.zeros((F, L))
    for fr in range(F):
        pad = np.zeros((ns, ns))
        pad[crop:crop + n_out, crop:crop + n_out] = g[fr]
        G = scale * np.fft.fft2(pad)                     # dL/dX_f
        for l in range(L):
            phi = px[fr, l][:, None] * py[fr, l][None, :]
            gS[l] += w[l] * G * np.conj(phi)
            q = np.conj(G) * S[l] * phi
            gw[l] += np.sum(q.real)
            gsx[fr, l] = -2 * np.pi * w[l] * np.sum(f[:, None] * q.imag)
            gsy[fr, l] = -2 * np.pi * w[l] * np.sum(f[None, :] * q.imag)
    return gS, gw, gsx, gsy
