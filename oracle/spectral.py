"""Oracle (test infrastructure only): spectral synthesis and the spectral
frozen-flow engine of the reference, in float64.

Follows ``src/pyturb/fourier.py``, ``src/pyturb/flow.py`` and the spectral
parts of ``src/pyturb/atmosphere.py``.
"""

from __future__ import annotations

from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np
import scipy.fft

_ARCSEC = np.pi / (180.0 * 3600.0)


def psd(f_sq, r0, L0, power_law=11.0 / 3.0, inner_scale=0.0):
    """``src/pyturb/fourier.py:131-149``."""
    f0 = 0.0 if np.isinf(L0) else 1.0 / L0**2
    out = 0.023 * r0 ** (-5.0 / 3.0) * (f_sq + f0) ** (-power_law / 2.0)
    if inner_scale > 0.0:
        fm = 5.92 / (2.0 * np.pi * inner_scale)
        out = out * np.exp(-f_sq / fm**2)
    return out


def band_amplitude(fx, fy, width, r0, L0, power_law=11.0 / 3.0, inner_scale=0.0, samples=33):
    """``src/pyturb/fourier.py:151-172``."""
    off = ((np.arange(samples) + 0.5) / samples - 0.5) * width
    f_sq = (fx + off[:, None]) ** 2 + (fy + off[None, :]) ** 2
    p = psd(f_sq, r0, L0, power_law, inner_scale)
    power = p.mean() * width**2
    f_eff = (p * f_sq).sum() / p.sum()
    return np.sqrt(power * f_eff / (fx**2 + fy**2))


def build_filters(n, dx, r0, L0, P, power_law=11.0 / 3.0, inner_scale=0.0):
    """Amplitude (n, n), grid frequencies (n,), and per level (amp (3,3),
    basis (3, n) complex, freqs (3,)) — ``src/pyturb/fourier.py:174-228``."""
    df = 1.0 / (n * dx)
    f = np.fft.fftfreq(n, d=dx)
    f_sq = f[:, None] ** 2 + f[None, :] ** 2
    f_sq[0, 0] = 1.0
    amp = np.sqrt(psd(f_sq, r0, L0, power_law, inner_scale)) * df
    amp[0, 0] = 0.0
    k = min(8, (n - 1) // 2)
    for i in range(-k, k + 1):
        for j in range(-k, k + 1):
            if i == 0 and j == 0:
                continue
            amp[i, j] = band_amplitude(f[i], f[j], df, r0, L0, power_law, inner_scale)
    coords = (np.arange(n) - n / 2.0) * dx
    levels = []
    for p in range(1, P + 1):
        df_p = df / 3.0**p
        f_p = np.array([-1.0, 0.0, 1.0]) * df_p
        a = np.zeros((3, 3))
        for i in range(3):
            for j in range(3):
                if i == 1 and j == 1:
                    continue
                a[i, j] = band_amplitude(f_p[i], f_p[j], df_p, r0, L0, power_law, inner_scale)
        basis = np.exp(2j * np.pi * f_p[:, None] * coords[None, :])
        levels.append((a, basis, f_p))
    return amp, f, levels


def _low(coef, basis):
    """Re(basis^T (coef @ basis)) for one level: (3,3) x (3,n) -> (n,n)."""
    return (basis.T @ (coef @ basis)).real


class OraclePhaseScreen:
    """``src/pyturb/fourier.py:31-294`` with an injected generator ``rng``."""

    def __init__(self, n, pixel_scale, r0, L0=25.0, subharmonics=8, power_law=11.0 / 3.0,
                 inner_scale=0.0, rng=None):
        self.n, self.dx, self.r0, self.L0 = int(n), float(pixel_scale), float(r0), float(L0)
        self.P = int(subharmonics)
        self.rng = rng
        self.amplitude, self.f, self.levels = build_filters(
            self.n, self.dx, self.r0, self.L0, self.P, power_law, inner_scale)

    def generate(self, count=None):
        """``src/pyturb/fourier.py:233-282``."""
        squeeze = count is None
        count = 1 if squeeze else int(count)
        n = self.n
        n_fft = (count + 1) // 2
        noise = self.rng.standard_normal((2, n_fft, n, n))
        spec = (noise[0] + 1j * noise[1]) * self.amplitude
        field = scipy.fft.ifft2(spec, axes=(-2, -1)) * (n * n)
        screens = np.concatenate((field.real, field.imag))[:count]
        if self.P:
            cn = []
            for a, _b, _f in self.levels:
                z = self.rng.standard_normal((2, count, 3, 3))
                cn.append((z[0] + 1j * z[1]) * a)
            low = np.zeros((count, n, n))
            for c in range(count):
                for p, (_a, b, _f) in enumerate(self.levels):
                    low[c] += _low(cn[p][c], b)
            low -= low.mean(axis=(-2, -1), keepdims=True)
            screens = screens + low
        return screens[0] if squeeze else screens


class OracleFlow:
    """``src/pyturb/flow.py:34-139``: fixed spectrum + shift theorem."""

    def __init__(self, template: OraclePhaseScreen, rng):
        self.t = template
        self.rng = rng
        self.reseed()

    def reseed(self):
        n = self.t.n
        z = self.rng.standard_normal((2, n, n))
        self.spectrum = (z[0] + 1j * z[1]) * self.t.amplitude
        self.sh = []
        for a, _b, _f in self.t.levels:
            z = self.rng.standard_normal((2, 3, 3))
            self.sh.append((z[0] + 1j * z[1]) * a)
        return self

    def translate(self, sx, sy):
        t = self.t
        n = t.n
        px = np.exp(2j * np.pi * sx * t.f)
        py = np.exp(2j * np.pi * sy * t.f)
        field = scipy.fft.ifft2(self.spectrum * px[:, None] * py[None, :]) * (n * n)
        screen = field.real
        if t.P:
            low = np.zeros((n, n))
            for c, (_a, b, f_p) in zip(self.sh, t.levels):
                shifted = c * np.exp(2j * np.pi * sx * f_p)[:, None] * np.exp(2j * np.pi * sy * f_p)[None, :]
                low += _low(shifted, b)
            screen = screen + (low - low.mean())
        return screen


class OracleAtmosphere:
    """Spectral engine, sampling, directions, LGS cone and boiling of
    ``src/pyturb/atmosphere.py:305-1243`` (``engine='spectral'``), float64.

    ``rng_factory(seed)`` builds each stream (``numpy.random.default_rng`` to
    reproduce the reference). ``layers`` is a sequence of objects with
    altitude, cn2_fraction, wind_speed, wind_direction, L0."""

    def __init__(self, layers, r0, wavelength=500e-9, zenith_angle=0.0, diameter=8.0, n=512,
                 subharmonics=8, field_of_view=0.0, tau_boil=None, interp="cubic",
                 lgs_altitude=None, seed=None, rng_factory=np.random.default_rng,
                 power_law=11.0 / 3.0, inner_scale=0.0):
        frac = np.array([ly.cn2_fraction for ly in layers], dtype=np.float64)
        frac = frac / frac.sum()
        self.layers = list(layers)
        self.wavelength = wavelength
        self.n = int(n)
        self.dx = diameter / n
        self.P = int(subharmonics)
        self.interp = interp
        cos_z = np.cos(np.deg2rad(zenith_angle))
        airmass = 1.0 / cos_z
        self.r0_los = r0 * cos_z ** (3.0 / 5.0)
        max_alt = max(ly.altitude for ly in layers) * airmass
        margin = int(np.ceil(max_alt * np.tan(field_of_view * _ARCSEC) / self.dx))
        self.margin = margin
        self.ns = self.n + 2 * margin
        self.fov = field_of_view
        L = len(layers)
        self.tau = (np.full(L, np.inf) if tau_boil is None
                    else np.broadcast_to(np.asarray(tau_boil, float), (L,)).astype(float))
        master = np.random.SeedSequence(seed)
        children = master.spawn(L)
        self.boil_seed = int(master.spawn(1)[0].generate_state(1)[0])
        master.spawn(1)  # extrude-engine boiling seed (unused by the spectral engine)
        self.boil_rng = rng_factory(self.boil_seed)
        self.gens, self.flows, r0s = [], [], []
        self.vx, self.vy, self.alt = [], [], []
        for ly, fr, child in zip(layers, frac, children):
            r0_i = self.r0_los * fr ** (-3.0 / 5.0)
            g, fl, _e = child.spawn(3)
            gen = OraclePhaseScreen(self.ns, self.dx, r0_i, ly.L0, self.P, power_law,
                                    inner_scale, rng=rng_factory(int(g.generate_state(1)[0])))
            self.gens.append(gen)
            self.flows.append(OracleFlow(gen, rng_factory(int(fl.generate_state(1)[0]))))
            th = np.deg2rad(ly.wind_direction)
            self.vx.append(ly.wind_speed * np.cos(th))
            self.vy.append(ly.wind_speed * np.sin(th))
            self.alt.append(ly.altitude * airmass)
            r0s.append(r0_i)
        self.vx, self.vy, self.alt = map(np.asarray, (self.vx, self.vy, self.alt))
        groups: Dict[float, List[int]] = {}
        for i, ly in enumerate(layers):
            groups.setdefault(round(float(ly.L0), 9), []).append(i)
        self.sample_gens = []
        for idxs, child in zip(groups.values(), master.spawn(len(groups))):
            if len(idxs) == 1:
                self.sample_gens.append(self.gens[idxs[0]])
                continue
            r0_agg = sum(r0s[i] ** (-5.0 / 3.0) for i in idxs) ** (-3.0 / 5.0)
            self.sample_gens.append(OraclePhaseScreen(
                self.ns, self.dx, r0_agg, layers[idxs[0]].L0, self.P, power_law, inner_scale,
                rng=rng_factory(int(child.generate_state(1)[0]))))
        self.lgs_mag = None
        if lgs_altitude is not None:
            self.lgs_mag = 1.0 - self.alt / (lgs_altitude * airmass)
        self.spectra = np.stack([f.spectrum for f in self.flows])
        self.sh = ([np.stack([f.sh[p] for f in self.flows]) for p in range(self.P)])
        self.t = 0.0
        if np.any(np.isfinite(self.tau)):
            self._tau_maps()

    # -- ``src/pyturb/atmosphere.py:618-658``
    def _tau_maps(self):
        L0s = np.array([ly.L0 for ly in self.layers], dtype=float)
        df = 1.0 / (self.ns * self.dx)
        f_ref = np.where(np.isfinite(L0s), 1.0 / np.where(L0s > 0, L0s, np.inf), df)
        f = self.gens[0].f
        fr = np.hypot(f[:, None], f[None, :])
        self.main_tau = self.tau[:, None, None] * np.clip(fr[None] / f_ref[:, None, None], 1.0, None) ** (-2.0 / 3.0)
        self.sh_tau = []
        for _a, _b, f_p in self.gens[0].levels:
            frs = np.hypot(f_p[:, None], f_p[None, :])
            self.sh_tau.append(self.tau[:, None, None] * np.clip(frs[None] / f_ref[:, None, None], 1.0, None) ** (-2.0 / 3.0))

    def _layer_low(self, sx, sy, l):
        n = self.ns
        low = np.zeros((n, n))
        for p, (_a, b, f_p) in enumerate(self.gens[0].levels):
            c = self.sh[p][l] * np.exp(2j * np.pi * sx * f_p)[:, None] * np.exp(2j * np.pi * sy * f_p)[None, :]
            low += _low(c, b)
        return low

    def phase(self, t, ox=0.0, oy=0.0):
        """``_integrate`` (``src/pyturb/atmosphere.py:882-938``) or
        ``_integrate_lgs`` (1000-1045), float64."""
        ns = self.ns
        f = self.gens[0].f
        sx = self.vx * t + self.alt * ox
        sy = self.vy * t + self.alt * oy
        if self.lgs_mag is not None:
            screens = []
            for l in range(len(self.layers)):
                spec = self.spectra[l] * np.exp(2j * np.pi * sx[l] * f)[:, None] * np.exp(2j * np.pi * sy[l] * f)[None, :]
                s = (scipy.fft.ifft2(spec) * ns * ns).real
                if self.P:
                    low = self._layer_low(sx[l], sy[l], l)
                    s = s + (low - low.mean())
                screens.append(s)
            return self._lgs_zoom(np.stack(screens))
        spec = np.zeros((ns, ns), dtype=complex)
        for l in range(len(self.layers)):
            spec += self.spectra[l] * np.exp(2j * np.pi * sx[l] * f)[:, None] * np.exp(2j * np.pi * sy[l] * f)[None, :]
        total = (scipy.fft.ifft2(spec) * ns * ns).real
        if self.P:
            low = np.zeros((ns, ns))
            for l in range(len(self.layers)):
                low += self._layer_low(sx[l], sy[l], l)
            total = total + (low - low.mean())
        m = self.margin
        return total[m:m + self.n, m:m + self.n]

    def _lgs_zoom(self, screens):
        """``src/pyturb/atmosphere.py:581-616, 1047-1090``."""
        n, ns = self.n, self.ns
        centre = (ns - 1) / 2.0
        base = np.arange(n, dtype=float) - (n - 1) / 2.0
        total = np.zeros((n, n))
        for l, mag in enumerate(self.lgs_mag):
            pos = centre + base * mag
            p0 = np.floor(pos).astype(int)
            fr = pos - p0
            offs, ws = interp_taps(self.interp, fr)
            idx = [np.clip(p0 + o, 0, ns - 1) for o in offs]
            out = np.zeros((n, n))
            for a in range(len(offs)):
                band = screens[l][idx[a]]
                rt = np.zeros((n, n))
                for b in range(len(offs)):
                    rt += ws[b][None, :] * band[:, idx[b]]
                out += ws[a][:, None] * rt
            total += out
        return total

    def opd(self, t=0.0, directions=None):
        scale = self.wavelength / (2.0 * np.pi)
        if directions is None:
            return self.phase(t) * scale
        return np.stack([self.phase(t, np.tan(a * _ARCSEC), np.tan(b * _ARCSEC))
                         for a, b in directions]) * scale

    def boil_step(self, dt):
        """``src/pyturb/atmosphere.py:1092-1126``."""
        with np.errstate(divide="ignore"):
            alpha = np.where(np.isfinite(self.tau), np.exp(-dt / self.tau), 1.0)
        if np.all(alpha >= 1.0):
            return
        L = len(self.layers)
        a = np.exp(-dt / self.main_tau)
        b = np.sqrt(np.clip(1.0 - a * a, 0.0, None))
        z = self.boil_rng.standard_normal((2, L, self.ns, self.ns))
        amps = np.stack([g.amplitude for g in self.gens])
        self.spectra = a * self.spectra + b * ((z[0] + 1j * z[1]) * amps)
        if self.P:
            z = self.boil_rng.standard_normal((2, self.P, L, 3, 3))
            for p in range(self.P):
                ap = np.exp(-dt / self.sh_tau[p])
                bp = np.sqrt(np.clip(1.0 - ap * ap, 0.0, None))
                amp_p = np.stack([g.levels[p][0] for g in self.gens])
                self.sh[p] = ap * self.sh[p] + bp * ((z[0, p] + 1j * z[1, p]) * amp_p)

    def frames(self, dt, steps):
        """``src/pyturb/atmosphere.py:1128-1154``."""
        out = []
        for _ in range(steps):
            t = self.t
            out.append((t, self.opd(t)))
            self.t += dt
            if np.any(np.isfinite(self.tau)):
                self.boil_step(dt)
        return out

    def sample(self, count=None):
        """``src/pyturb/atmosphere.py:1191-1219``."""
        total = None
        for g in self.sample_gens:
            s = g.generate(count)
            total = s if total is None else total + s
        m = self.margin
        return total[..., m:m + self.n, m:m + self.n] * (self.wavelength / (2.0 * np.pi))


def interp_taps(interp, fr):
    """(offsets, weights) for linear / Catmull-Rom / Lanczos-3 at fraction fr
    (``src/pyturb/extrude.py:74-83``, ``src/pyturb/infinite.py:67-85``)."""
    if interp == "linear":
        return (0, 1), (1.0 - fr, fr)
    if interp == "lanczos":
        offs = tuple(range(-2, 4))
        raw = [np.sinc(fr - d) * np.sinc((fr - d) / 3.0) for d in offs]
        tot = sum(raw)
        return offs, tuple(r / tot for r in raw)
    t2 = fr * fr
    t3 = t2 * fr
    return (-1, 0, 1, 2), (0.5 * (-fr + 2 * t2 - t3), 0.5 * (2 - 5 * t2 + 3 * t3),
                           0.5 * (fr + 4 * t2 - 3 * t3), 0.5 * (-t2 + t3))
