"""Float64 restatement of the differentiable multi-layer readout (test oracle).

Test infrastructure only: imported by ``tests/`` and nothing on the product
path. The geometry is the LGS cone zoom of the reference's spectral engine,
``Atmosphere._build_lgs_zoom`` / ``_lgs_zoom`` (src/pyturb/atmosphere.py:
581-616, 1048-1090: the pupil grid ``centre + (i - (n-1)/2) * mag``, rows
first), with the displacement of ``_integrate_lgs`` (atmosphere.py:1012-1022,
``disp = v * t + alt * offset``, x displacing rows) applied as a periodic
bilinear shift instead of a phase ramp. The reference has no adjoint, so the
vector-Jacobian product here is the analytic transpose, written as a scatter
(``np.add.at``) so that it shares no structure with the device gather, and is
itself checked against float64 central differences and torch autograd.
"""

from __future__ import annotations

import numpy as np


def positions(n, n_screen, pixel_scale, altitudes, directions, mag, winds, times):
    """``pos0 (T, D, L, 2)``: screen position (px) of pupil pixel (0, 0).

    ``directions (D, 2)`` rad, ``mag (D, L)``, ``winds (L, 2)`` m/s,
    ``times (T,)`` s. Axis 0 (rows) takes the x displacement, as the
    reference's ``phasor_x`` multiplies the row axis (atmosphere.py:1019-1021).
    """
    alt = np.asarray(altitudes, np.float64)
    th = np.asarray(directions, np.float64)
    v = np.asarray(winds, np.float64)
    t = np.asarray(times, np.float64)
    m = np.asarray(mag, np.float64)
    centre = (n_screen - 1) / 2.0
    disp = v[None, None, :, :] * t[:, None, None, None] + alt[None, None, :, None] * th[None, :, None, :]
    return centre - m[None, :, :, None] * (n - 1) / 2.0 + disp / pixel_scale


def _axis(p0, m, n, S):
    """Cells and fractions of ``u_i = p0 + m * i`` (i < n) on a periodic axis of
    S samples, from the 32.32 fixed-point positions the device forms
    (``p0`` reduced into [0, S), both rounded to 2^-32 px). The values agree
    with float64 arithmetic to ~1e-10 px; the fixed point decides which cell a
    sample lying exactly on a grid line belongs to, and so the one-sided
    position derivative there (LGS magnifications such as 1 - h/H = 37/45 put
    whole rows and columns of samples on grid lines)."""
    one = 2.0 ** 32
    x = p0 - np.floor(p0 / S) * S
    v = int(np.rint(x * one))
    span = S << 32
    v = v + span if v < 0 else (v - span if v >= span else v)
    u = v + np.arange(n, dtype=np.int64) * int(np.rint(m * one))
    i0 = u >> 32
    i0 = np.where(i0 >= S, i0 - S, i0)
    f = (u & 0xFFFFFFFF).astype(np.float64) / one
    return i0, (i0 + 1) % S, f


def layer_readout(screens, w, pos0, mag, n):
    """Forward: ``out (B, T, D, n, n)`` in float64."""
    screens = np.asarray(screens, np.float64)
    B, L, S, _ = screens.shape
    T, D = pos0.shape[:2]
    out = np.zeros((B, T, D, n, n))
    for t in range(T):
        for d in range(D):
            for l in range(L):
                r0, r1, fr = _axis(pos0[t, d, l, 0], mag[d, l], n, S)
                c0, c1, fc = _axis(pos0[t, d, l, 1], mag[d, l], n, S)
                s = screens[:, l]
                top = s[:, r0][:, :, c0] * (1 - fc) + s[:, r0][:, :, c1] * fc
                bot = s[:, r1][:, :, c0] * (1 - fc) + s[:, r1][:, :, c1] * fc
                out[:, t, d] += w[l] * (top * (1 - fr)[:, None] + bot * fr[:, None])
    return out


def layer_readout_vjp(screens, w, pos0, mag, n, g):
    """Vector-Jacobian product for upstream ``g (B, T, D, n, n)``.

    Returns ``(d screens (B, L, S, S), d w (L,), d pos0 (T, D, L, 2))``; the
    position derivative is that of the bilinear cell each sample lies in.
    """
    screens = np.asarray(screens, np.float64)
    g = np.asarray(g, np.float64)
    B, L, S, _ = screens.shape
    T, D = pos0.shape[:2]
    gs = np.zeros_like(screens)
    gw = np.zeros(L)
    gp = np.zeros((T, D, L, 2))
    for t in range(T):
        for d in range(D):
            gi = g[:, t, d]
            for l in range(L):
                r0, r1, fr = _axis(pos0[t, d, l, 0], mag[d, l], n, S)
                c0, c1, fc = _axis(pos0[t, d, l, 1], mag[d, l], n, S)
                s = screens[:, l]
                v00, v01 = s[:, r0][:, :, c0], s[:, r0][:, :, c1]
                v10, v11 = s[:, r1][:, :, c0], s[:, r1][:, :, c1]
                FR, FC = fr[:, None], fc[None, :]
                top = v00 * (1 - FC) + v01 * FC
                bot = v10 * (1 - FC) + v11 * FC
                val = top * (1 - FR) + bot * FR
                gw[l] += np.sum(gi * val)
                gp[t, d, l, 0] += w[l] * np.sum(gi * (bot - top))
                gp[t, d, l, 1] += w[l] * np.sum(gi * ((v01 - v00) * (1 - FR) + (v11 - v10) * FR))
                R0, R1 = r0[:, None], r1[:, None]
                C0, C1 = c0[None, :], c1[None, :]
                for rr, cc, wt in ((R0, C0, (1 - FR) * (1 - FC)), (R0, C1, (1 - FR) * FC),
                                   (R1, C0, FR * (1 - FC)), (R1, C1, FR * FC)):
                    rr_b = np.broadcast_to(rr, (n, n))
                    cc_b = np.broadcast_to(cc, (n, n))
                    for b in range(B):
                        np.add.at(gs[b, l], (rr_b, cc_b), w[l] * wt * gi[b])
    return gs, gw, gp
