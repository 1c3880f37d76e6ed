"""Float64 restatements of the validation diagnostics (test oracle only):
``structure_function`` (src/pyturb/utils.py:159-201), ``zernike_basis`` /
``zernike_decompose`` (src/pyturb/analysis.py:56-162) and ``temporal_psd``
(analysis.py:183-208). Imported by ``tests/`` only; pinned against the
reference's own functions in ``tests/test_diagnostics_oracle.py``."""

from __future__ import annotations

from math import comb

import numpy as np


def structure_function(phase, pixel_scale=1.0, max_separation=None):
    p = np.asarray(phase, dtype=np.float64)
    if p.ndim == 2:
        p = p[None]
    n = min(p.shape[-2:])
    ms = n // 4 if max_separation is None else int(max_separation)
    D = np.empty(ms)
    for s in range(1, ms + 1):
        a = np.mean((p[:, s:, :] - p[:, :-s, :]) ** 2)
        b = np.mean((p[:, :, s:] - p[:, :, :-s]) ** 2)
        D[s - 1] = 0.5 * (a + b)
    return np.arange(1, ms + 1) * pixel_scale, D


def noll(j):
    """(n, m) by walking the Noll triangle row by row."""
    n, left = 0, j
    while left > n + 1:
        left -= n + 1
        n += 1
    ms = sorted({abs(m) for m in range(-n, n + 1, 2)})
    order = [0] if n % 2 == 0 else []
    for a in ms:
        if a:
            order += [a, a]
    am = order[left - 1]
    return n, (0 if am == 0 else (am if j % 2 == 0 else -am))


def radial(n, am, rho):
    # R_n^m(rho) = sum_s (-1)^s C(n-s, s) C(n-2s, (n-am)/2 - s) rho^(n-2s)
    out = np.zeros_like(rho)
    for s in range((n - am) // 2 + 1):
        out += (-1) ** s * comb(n - s, s) * comb(n - 2 * s, (n - am) // 2 - s) * rho ** (n - 2 * s)
    return out


def zernike_basis(n_modes, n_pixels, diameter_pixels=None):
    radius = (n_pixels if diameter_pixels is None else diameter_pixels) / 2.0
    u = (np.arange(n_pixels) - (n_pixels - 1) / 2.0) / radius
    x, y = np.meshgrid(u, u, indexing="ij")
    rho, th = np.hypot(x, y), np.arctan2(y, x)
    out = np.zeros((n_modes, n_pixels, n_pixels))
    for q in range(n_modes):
        n, m = noll(q + 1)
        ang = np.cos(m * th) if m >= 0 else np.sin(-m * th)
        z = np.sqrt(n + 1.0) * (1.0 if m == 0 else np.sqrt(2.0)) * radial(n, abs(m), rho) * ang
        out[q] = np.where(rho <= 1.0, z, 0.0)
    return out


def zernike_decompose(phase, n_modes, basis=None):
    p = np.asarray(phase, dtype=np.float64)
    single = p.ndim == 2
    if single:
        p = p[None]
    b = zernike_basis(n_modes, p.shape[-1]) if basis is None else basis
    mask = b[0] != 0
    c, *_ = np.linalg.lstsq(b[:, mask].T, p[:, mask].T, rcond=None)
    return c.T[0] if single else c.T


def temporal_psd(series, dt):
    x = np.asarray(series, dtype=np.float64)
    x = x - x.mean(axis=-1, keepdims=True)
    T = x.shape[-1]
    p = np.abs(np.fft.rfft(x, axis=-1)) ** 2 * (2.0 * dt / T)
    p = p.reshape(-1, p.shape[-1]).mean(axis=0)
    return np.fft.rfftfreq(T, d=dt)[1:], p[1:]
