"""Oracle (test infrastructure only): Assemat-Wilson extrusion, the ring
buffer with compaction and the rotated sub-pixel readout, in float64.

Follows ``src/pyturb/infinite.py``, ``src/pyturb/extrude.py`` and
``src/pyturb/ring.py``.
"""

from __future__ import annotations

from math import floor

import numpy as np
from scipy import linalg
from scipy.special import gamma, kv

from .spectral import OraclePhaseScreen, interp_taps


def phase_covariance(r, r0, L0):
    """``src/pyturb/infinite.py:88-117``."""
    r = np.asarray(r, dtype=np.float64)
    pref = ((L0 / r0) ** (5.0 / 3.0) * (2.0 ** (-5.0 / 6.0) * gamma(11.0 / 6.0) / np.pi ** (8.0 / 3.0))
            * ((24.0 / 5.0) * gamma(6.0 / 5.0)) ** (5.0 / 6.0))
    x = 2.0 * np.pi * r / L0
    core = np.full_like(x, 2.0 ** (-1.0 / 6.0) * gamma(5.0 / 6.0))
    nz = x > 0
    core[nz] = x[nz] ** (5.0 / 6.0) * kv(5.0 / 6.0, x[nz])
    return pref * core


def sparse_points(width, m, columns, max_depth=None):
    """Sparse stencil points ``(depth, column)`` beside the m full rows (no
    reference counterpart; the package's rule restated): ``columns`` columns
    at round((c + 1)(W - 1)/(columns + 1)), at every depth 2^j with
    m < 2^j <= max_depth (default the largest power of two <= W)."""
    if columns <= 0:
        return []
    dmax = max_depth if max_depth is not None else 1 << (int(width).bit_length() - 1)
    depths = [1 << j for j in range(1, 31) if m < (1 << j) <= dmax]
    cols = [int(round((c + 1) * (width - 1) / (columns + 1))) for c in range(columns)]
    return [(d, c) for d in depths for c in cols]


def build_extrusion(width, m, dx, L0, r0=1.0, sparse=()):
    """``src/pyturb/extrude.py:250-304`` / ``src/pyturb/infinite.py:231-269``;
    ``sparse`` appends points (column, m - depth) to the stencil (rows-only
    when empty, as the reference)."""
    yz, xz = np.mgrid[0:m, 0:width]
    st = np.column_stack((xz.ravel(), yz.ravel())).astype(float)
    if len(sparse):
        extra = np.array([(c, m - d) for d, c in sparse], dtype=float)
        st = np.concatenate([st, extra])
    nr = np.column_stack((np.arange(width, dtype=float), np.full(width, float(m))))

    def cov(a, b):
        return phase_covariance(np.hypot(a[:, None, 0] - b[None, :, 0],
                                         a[:, None, 1] - b[None, :, 1]) * dx, r0, L0)

    czz, cxz, cxx = cov(st, st), cov(nr, st), cov(nr, nr)
    try:
        a = linalg.cho_solve(linalg.cho_factor(czz), cxz.T).T
    except np.linalg.LinAlgError:
        a = np.linalg.lstsq(czz, cxz.T, rcond=None)[0].T
    res = cxx - a @ cxz.T
    res = (res + res.T) / 2.0
    w, v = np.linalg.eigh(res)
    return a, v * np.sqrt(np.clip(w, 0.0, None))


def seed_factor(width, m, dx, L0, r0=1.0):
    """``S`` with ``S S^T = C_zz`` of the m stencil rows, the seed of boiling's
    fresh windows (``src/pyturb/extrude.py:290-303``): Cholesky of the
    symmetrised covariance, an eigen square root if that fails."""
    yz, xz = np.mgrid[0:m, 0:width]
    st = np.column_stack((xz.ravel(), yz.ravel())).astype(float)
    czz = phase_covariance(np.hypot(st[:, None, 0] - st[None, :, 0],
                                    st[:, None, 1] - st[None, :, 1]) * dx, r0, L0)
    czz = (czz + czz.T) / 2.0
    try:
        return np.linalg.cholesky(czz)
    except np.linalg.LinAlgError:
        w, v = np.linalg.eigh(czz)
        return v * np.sqrt(np.clip(w, 0.0, None))


def compact_row_ring(buf, base, fill, m, first_readable_row):
    """``src/pyturb/ring.py:9-28``."""
    target = int(floor(first_readable_row)) - 1
    stencil = base + fill - m
    keep_from = max(1, min(target, stencil) - base)
    keep = fill - keep_from
    buf[:keep] = buf[keep_from:fill].copy()
    return base + keep_from, keep


def _smooth_size(n):
    """Smallest 2^a 3^b >= n."""
    return min(v for v in (2 ** a * 3 ** b for a in range(40) for b in range(25)) if v >= n)


class _Layer:
    """``src/pyturb/extrude.py:307-496`` (frozen flow). With sparse points the
    buffer also keeps ``history`` older rows below the readable window and
    the seed screen is ``seed_side`` square (cropped to W columns)."""

    def __init__(self, n, W, dx, r0, L0, vx, vy, alt, m, rng, a, b_unit, cap, mag, fov,
                 sparse=(), history=0, seed_side=None):
        self.n, self.W, self.dx, self.m, self.rng = n, W, dx, m, rng
        speed = float(np.hypot(vx, vy))
        self.speed = speed
        self.c = vx / speed if speed > 0 else 1.0
        self.s = vy / speed if speed > 0 else 0.0
        self.alt_pix = alt / dx
        self.a = a
        self.b = b_unit * r0 ** (-5.0 / 6.0)
        g = (np.arange(n, dtype=float) - (n - 1) / 2.0) * mag
        along = g[:, None] * self.c + g[None, :] * self.s
        perp = -g[:, None] * self.s + g[None, :] * self.c
        self.along, self.perp = along, perp + W / 2.0
        self.amin, self.amax = float(along.min()), float(along.max())
        self.fov = float(fov)
        self.buf = np.empty((cap, W))
        self.cap = cap
        emin = self.amin - self.fov
        span = int(np.ceil(self.amax + self.fov)) - int(np.floor(emin)) + 3
        self.sparse = list(sparse)
        self.depth = max([m] + [d for d, _ in self.sparse])
        self.base = int(np.floor(emin)) - 2 - history
        side = W if seed_side is None else seed_side
        init = OraclePhaseScreen(side, dx, r0, L0, rng=rng).generate()
        self.buf[:span + history] = init[:span + history, :W]
        self.fill = span + history
        self.travel = 0.0

    def extrude_one(self):
        if self.fill == self.cap:
            self.base, self.fill = compact_row_ring(self.buf, self.base, self.fill, self.depth,
                                                    self.amin - self.fov + self.travel)
        z = self.buf[self.fill - self.m:self.fill].ravel()
        if self.sparse:
            z = np.concatenate([z, [self.buf[self.fill - d, c] for d, c in self.sparse]])
        beta = self.rng.standard_normal(self.W)
        self.buf[self.fill] = self.a @ z + self.b @ beta
        self.fill += 1

    def set_travel(self, travel):
        self.travel = float(travel)
        top = int(np.ceil(self.amax + self.fov + self.travel)) + 2
        while self.base + self.fill - 1 < top:
            self.extrude_one()

    def offsets(self, thx, thy):
        dxp, dyp = self.alt_pix * thx, self.alt_pix * thy
        return dxp * self.c + dyp * self.s, -dxp * self.s + dyp * self.c


class OracleExtruded:
    """``ExtrudedAtmosphere`` (``src/pyturb/extrude.py:499-915``) with the
    looped readout (``_integrate_looped`` 883-915), frozen flow."""

    def __init__(self, n, pixel_scale, layer_r0, layer_L0, layer_wind, layer_altitude_los,
                 field_of_view_pix=0.0, stencil_rows=2, interp="cubic", lgs_altitude_los=None,
                 seeds=None, rng_factory=np.random.default_rng, tau_boil=None, boil_seed=None,
                 stencil_columns=0, sparse_depth=None):
        self.n, self.dx, self.interp, self.m = int(n), float(pixel_scale), interp, stencil_rows
        L = len(layer_r0)
        fov = ([float(field_of_view_pix)] * L if np.ndim(field_of_view_pix) == 0
               else list(field_of_view_pix))
        mags = ([1.0 - a / lgs_altitude_los for a in layer_altitude_los]
                if lgs_altitude_los is not None else [1.0] * L)
        exts, spans = [], []
        for (vx, vy), mag, fv in zip(layer_wind, mags, fov):
            sp = float(np.hypot(vx, vy))
            c = vx / sp if sp > 0 else 1.0
            s = vy / sp if sp > 0 else 0.0
            e = (n - 1) / 2.0 * mag * (abs(c) + abs(s))
            exts.append(e)
            spans.append(int(np.ceil(e + fv)) - int(np.floor(-e - fv)) + 3)
        self.W = int(np.ceil(2.0 * max(exts) + 2.0 * max(fov))) + 4
        self.sparse = sparse_points(self.W, self.m, stencil_columns, sparse_depth)
        history = max([0] + [d for d, _ in self.sparse])
        self.cap = max(spans) + self.n + self.m + 32 + history
        side = self.W if not self.sparse else _smooth_size(max(self.W, max(spans) + history))
        cache = {}
        seeds = seeds if seeds is not None else [None] * L
        self.layers = []
        for r0, L0, (vx, vy), alt, sd, mag, fv in zip(layer_r0, layer_L0, layer_wind,
                                                      layer_altitude_los, seeds, mags, fov):
            key = round(float(L0), 9)
            if key not in cache:
                cache[key] = build_extrusion(self.W, self.m, self.dx, L0, sparse=self.sparse)
            a, b = cache[key]
            self.layers.append(_Layer(self.n, self.W, self.dx, r0, L0, vx, vy, alt, self.m,
                                      rng_factory(sd), a, b, self.cap, mag, fv, self.sparse,
                                      history, side))
        # boiling (src/pyturb/extrude.py:472-496, 643-650, 695-753, the NumPy path)
        self.tau = [float("inf")] * L if tau_boil is None else [
            float("inf") if t is None else float(t) for t in tau_boil]
        self.boiling = any(np.isfinite(t) for t in self.tau)
        if self.boiling:
            seeds_by_L0 = {}
            for ly, r0, L0 in zip(self.layers, layer_r0, layer_L0):
                key = round(float(L0), 9)
                if key not in seeds_by_L0:
                    seeds_by_L0[key] = seed_factor(self.W, self.m, self.dx, L0)
                ly.seed = seeds_by_L0[key] * r0 ** (-5.0 / 6.0)
            self.boil_rng = rng_factory(boil_seed)

    def boil_step(self, dt):
        """Blend every boiling layer's readable rows toward an independent
        fresh window: ``buf[lo:hi] = a buf + b fresh``, a = exp(-dt/tau)."""
        if not self.boiling:
            return
        regions = []
        for i, ly in enumerate(self.layers):
            if not np.isfinite(self.tau[i]):
                continue
            a = float(np.exp(-dt / self.tau[i]))
            b = float(np.sqrt(max(0.0, 1.0 - a * a)))
            lo = max(0, int(np.floor(ly.amin + ly.travel)) - ly.base - 3)
            hi = ly.fill
            if hi > lo:
                regions.append((ly, lo, hi, a, b))
        W, m = self.W, self.m
        for ly, lo, hi, a, b in regions:
            h = hi - lo
            fresh = np.empty((h, W))
            seed = (ly.seed @ self.boil_rng.standard_normal(m * W)).reshape(m, W)
            fresh[:min(m, h)] = seed[:min(m, h)]
            for k in range(m, h):
                fresh[k] = ly.a @ fresh[k - m:k].ravel() + ly.b @ self.boil_rng.standard_normal(W)
            ly.buf[lo:hi] = a * ly.buf[lo:hi] + b * fresh

    def set_time(self, t):
        for ly in self.layers:
            ly.set_travel(ly.speed * t / self.dx)

    def integrate(self, thx=0.0, thy=0.0):
        total = np.zeros((self.n, self.n))
        for ly in self.layers:
            oa, op = ly.offsets(thx, thy)
            row = ly.along + ((ly.travel - ly.base) + oa)
            col = ly.perp + op
            r0 = np.floor(row).astype(int)
            c0 = np.floor(col).astype(int)
            offr, wr = interp_taps(self.interp, row - r0)
            offc, wc = interp_taps(self.interp, col - c0)
            for dr, w_r in zip(offr, wr):
                rr = np.clip(r0 + dr, 0, ly.fill - 1)
                rt = np.zeros_like(total)
                for dc, w_c in zip(offc, wc):
                    cc = np.clip(c0 + dc, 0, self.W - 1)
                    rt += w_c * ly.buf[rr, cc]
                total += w_r * rt
        return total


class OracleInfinite:
    """``InfinitePhaseScreen`` (``src/pyturb/infinite.py:120-395``)."""

    def __init__(self, n, pixel_scale, r0, L0=25.0, stencil_rows=2, interp="cubic", rng=None):
        self.n, self.dx, self.r0, self.L0, self.m, self.interp = n, pixel_scale, r0, L0, stencil_rows, interp
        self.a, self.b = build_extrusion(n, stencil_rows, pixel_scale, L0, r0=r0)
        self.rng = rng
        self.cap = n + stencil_rows + 6
        self.buf = np.empty((self.cap, n))
        self.buf[:n] = OraclePhaseScreen(n, pixel_scale, r0, L0, rng=rng).generate()
        self.base, self.fill, self.travel = 0, n, 0.0
        self._advance_to(0.0)

    def _extrude_one(self):
        if self.fill == self.cap:
            self.base, self.fill = compact_row_ring(self.buf, self.base, self.fill, self.m,
                                                    self.travel)
        z = self.buf[self.fill - self.m:self.fill].ravel()
        beta = self.rng.standard_normal(self.n)
        self.buf[self.fill] = self.a @ z + self.b @ beta
        self.fill += 1

    def _advance_to(self, travel):
        self.travel = float(travel)
        top = int(np.floor(self.travel)) + self.n + 2
        while self.base + self.fill - 1 < top:
            self._extrude_one()
        pos = (self.travel - self.base) + np.arange(self.n)
        i0 = np.floor(pos).astype(int)
        t = (pos - i0)[:, None]
        offs, ws = interp_taps(self.interp, t)
        self.screen = sum(w * self.buf[np.clip(i0 + o, 0, self.fill - 1)] for o, w in zip(offs, ws))

    def step(self, steps=1):
        self._advance_to(self.travel + steps)
        return self.screen

    def advance(self, pixels):
        self._advance_to(self.travel + pixels)
        return self.screen
