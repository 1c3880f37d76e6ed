"""Oracle (test infrastructure only): the reference's own CPU path for the
benchmark workloads, restated with the reference's float32 NumPy/SciPy
operations so its timing stands for the reference on the same host.

- ``frame``: ``Atmosphere._integrate`` without Numba
  (``src/pyturb/atmosphere.py:882-938``): float32 phasors per layer, the
  broadcast layer sum, one ``scipy.fft.ifft2`` with ``workers`` threads
  (``src/pyturb/backend.py:52-98``), the batched subharmonic matmuls, crop,
  OPD scale (``src/pyturb/atmosphere.py:764-778``).
- ``sample``: ``PhaseScreen.generate`` in float32 (``src/pyturb/fourier.py:233-282``)
  per L0 group, cropped and scaled (``src/pyturb/atmosphere.py:1191-1219``).

Used only by ``bench.py``'s CPU baseline and ``--impl reference`` arm.
"""

from __future__ import annotations

import numpy as np
import scipy.fft

from .spectral import build_filters


class ReferenceCPU:
    """Float32 state of the reference's spectral engine for one atmosphere."""

    def __init__(self, n, ns, dx, r0_layers, L0s, P, vx, vy, alt, crop, wavelength=500e-9,
                 seed=0, workers=-1):
        rng = np.random.default_rng(seed)
        self.n, self.ns, self.crop, self.workers = n, ns, crop, workers
        self.scale = wavelength / (2.0 * np.pi)
        self.vx, self.vy, self.alt = (np.asarray(v, dtype=np.float64) for v in (vx, vy, alt))
        spectra, coeffs, amps = [], [], []
        for r0, L0 in zip(r0_layers, L0s):
            amp, f, levels = build_filters(ns, dx, r0, L0, P)
            z = rng.standard_normal((2, ns, ns), dtype=np.float32)
            spectra.append(((z[0] + 1j * z[1]) * amp.astype(np.float32)).astype(np.complex64))
            cs = []
            for a, _b, _f in levels:
                z = rng.standard_normal((2, 3, 3), dtype=np.float32)
                cs.append(((z[0] + 1j * z[1]) * a).astype(np.complex64))
            coeffs.append(cs)
            amps.append(amp.astype(np.float32))
        self.f = f.astype(np.float32)
        self.spectra = np.stack(spectra)
        self.P = P
        if P:
            self.sh_coeffs = np.stack([np.stack([c[p] for c in coeffs]) for p in range(P)])
            self.sh_basis = np.stack([b for _a, b, _f in levels]).astype(np.complex64)
            self.sh_freqs = np.stack([f_p for _a, _b, f_p in levels]).astype(np.float32)
        self.amp0 = amps[0]
        self.levels0 = levels

    def frame(self, t: float) -> np.ndarray:
        ns = self.ns
        sx = (self.vx * t).astype(np.float32)
        sy = (self.vy * t).astype(np.float32)
        px = np.exp((2j * np.pi) * sx[:, None] * self.f[None, :]).astype(np.complex64)
        py = np.exp((2j * np.pi) * sy[:, None] * self.f[None, :]).astype(np.complex64)
        spectrum = (self.spectra * px[:, :, None] * py[:, None, :]).sum(axis=0)
        total = (scipy.fft.ifft2(spectrum, axes=(-2, -1), workers=self.workers) * (ns * ns)).real
        if self.P:
            fp = self.sh_freqs
            qx = np.exp((2j * np.pi) * sx[None, :, None] * fp[:, None, :]).astype(np.complex64)
            qy = np.exp((2j * np.pi) * sy[None, :, None] * fp[:, None, :]).astype(np.complex64)
            shifted = (self.sh_coeffs * qx[:, :, :, None] * qy[:, :, None, :]).sum(axis=1)
            m = np.matmul(shifted, self.sh_basis).reshape(self.P * 3, ns)
            low = (self.sh_basis.reshape(self.P * 3, ns).T @ m).real
            low -= low.mean()
            total = total + low
        c = self.crop
        out = np.ascontiguousarray(total[c:c + self.n, c:c + self.n].astype(np.float32))
        return out * np.float32(self.scale)

    def sample(self, count: int, rng: np.random.Generator) -> np.ndarray:
        """One L0 group's ``PhaseScreen.generate(count)`` in float32, cropped, scaled."""
        ns = self.ns
        n_fft = (count + 1) // 2
        z = rng.standard_normal((2, n_fft, ns, ns), dtype=np.float32)
        spec = (z[0] + 1j * z[1]) * self.amp0
        field = scipy.fft.ifft2(spec, axes=(-2, -1), workers=self.workers) * (ns * ns)
        screens = np.concatenate((field.real, field.imag))[:count]
        if self.P:
            cn = np.empty((self.P, count, 3, 3), dtype=np.complex64)
            for p, (a, _b, _f) in enumerate(self.levels0):
                zz = rng.standard_normal((2, count, 3, 3), dtype=np.float32)
                cn[p] = (zz[0] + 1j * zz[1]) * a.astype(np.float32)
            m = np.matmul(cn, self.sh_basis[:, None])
            m = np.ascontiguousarray(m.transpose(1, 0, 2, 3)).reshape(count, self.P * 3, ns)
            low = np.matmul(self.sh_basis.reshape(self.P * 3, ns).T, m).real
            low -= low.mean(axis=(-2, -1), keepdims=True)
            screens = screens + low
        c = self.crop
        return screens[:, c:c + self.n, c:c + self.n].astype(np.float32) * np.float32(self.scale)
