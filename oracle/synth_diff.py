"""Float64 restatement of the weighted spectral frame synthesis and its
vector-Jacobian product (test oracle).

Test infrastructure only: imported by ``tests/`` and nothing on the product
path. The forward is ``Atmosphere._integrate`` (src/pyturb/atmosphere.py:
882-938: per-layer phasors ``exp(2 pi i f s)`` with ``f = fftfreq(ns, dx)``,
x along axis 0, summed spectra, ``ifft2 * ns^2``, real part; optionally the
subharmonic low-order sum of atmosphere.py:921-935, each level's 3 x 3
coefficients shifted by ``exp(2 pi i f_p s)``, evaluated on the bases
``exp(2 pi i f_p (x - ns/2) dx)`` and made zero-mean over the grid; crop)
with a weight per layer. The reference has no gradients; the
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


def _sh_parts(sh, w, sx, sy, ns, dx):
    """Bases (P, 3, ns) and per-frame layer terms for ``sh = (coef (P, L, 3, 3)
    complex, freqs (P, 3))``: ``E[f, l, p, i, j] = exp(2 pi i (sx[f, l] f_pi +
    sy[f, l] f_pj))`` and ``C[f, p, i, j] = sum_l w_l coef[p, l, i, j] E``."""
    coef = np.asarray(sh[0], np.complex128)
    fp = np.asarray(sh[1], np.float64)
    x = (np.arange(ns) - ns / 2.0) * dx
    basis = np.exp(2j * np.pi * fp[:, :, None] * x[None, None, :])
    ex = np.exp(2j * np.pi * np.asarray(sx)[:, :, None, None] * fp[None, None])   # (F, L, P, 3)
    ey = np.exp(2j * np.pi * np.asarray(sy)[:, :, None, None] * fp[None, None])
    E = ex[..., :, None] * ey[..., None, :]                                         # (F, L, P, 3, 3)
    C = np.einsum("l,plij,flpij->fpij", np.asarray(w, np.float64), coef, E)
    return coef, fp, basis, E, C


def synth_frames(spectra, w, sx, sy, dx, crop, n_out, scale, sh=None):
    """``(F, n_out, n_out)``: ``scale * crop(Re(ifft2(sum_l w_l S_l Phi) ns^2) +
    low)``, ``low`` the zero-mean subharmonic sum when ``sh`` is given."""
    S = np.asarray(spectra, np.complex128)
    L, ns, _ = S.shape
    _, px, py = _phasors(ns, dx, sx, sy)
    F = px.shape[0]
    if sh is not None:
        _, _, basis, _, C = _sh_parts(sh, w, sx, sy, ns, dx)
    out = np.empty((F, n_out, n_out))
    for f in range(F):
        X = np.einsum("l,lij,li,lj->ij", np.asarray(w, np.float64), S, px[f], py[f])
        y = np.real(np.fft.ifft2(X)) * ns * ns
        if sh is not None:
            low = np.real(np.einsum("pix,pij,pjy->xy", basis, C[f], basis))
            y = y + (low - low.mean())
        out[f] = scale * y[crop:crop + n_out, crop:crop + n_out]
    return out


def synth_vjp(spectra, w, sx, sy, dx, crop, n_out, scale, g, sh=None):
    """``(dS (L, ns, ns) complex as dL/dRe + i dL/dIm, dw (L,), dsx (F, L), dsy (F, L))``,
    and ``dcoef (P, L, 3, 3)`` (same convention) last when ``sh`` is given."""
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
    if sh is None:
        return gS, gw, gsx, gsy
    # low_f = Re sum_pij C[f,p,i,j] (b_pi(x) b_pj(y) - mean), so dL/dC = conj(Q) with
    # Q[f,p,i,j] = scale * sum_xy pad(g_f) (b_pi(x) b_pj(y) - beta_pi beta_pj)
    coef, fp, basis, E, _ = _sh_parts(sh, w, sx, sy, ns, dx)
    beta = basis.mean(axis=-1)                                                   # (P, 3)
    Q = np.empty((F,) + coef.shape[:1] + (3, 3), np.complex128)
    for fr in range(F):
        pad = np.zeros((ns, ns))
        pad[crop:crop + n_out, crop:crop + n_out] = g[fr]
        Gq = np.einsum("pix,xy,pjy->pij", basis, pad, basis)
        Q[fr] = scale * (Gq - beta[:, :, None] * beta[:, None, :] * pad.sum())
    M = np.einsum("plij,flpij,fpij->flpij", coef, E, Q)                         # c E Q
    gw = gw + M.real.sum(axis=(0, 2, 3, 4))
    wM = w[None, :, None, None, None] * M
    gsx = gsx - 2 * np.pi * np.einsum("pi,flpij->fl", fp, wM.imag)
    gsy = gsy - 2 * np.pi * np.einsum("pj,flpij->fl", fp, wM.imag)
    gcoef = np.conj(np.einsum("l,flpij,fpij->plij", w, E, Q))
    return gS, gw, gsx, gsy, gcoef
