"""Test infrastructure (checker only): a NumPy restatement of the in-kernel
noise of ``pyturb_gb300`` so that screens drawn on the device with Philox
noise can be compared with the float64 oracle on the same normals.

- Philox4x32 with 10 rounds (Salmon, Moraes, Dror & Shaw, SC'11, "Parallel
  random numbers: as easy as 1, 2, 3"): multipliers 0xD2511F53 / 0xCD9E8D57,
  key increments 0x9E3779B9 / 0xBB67AE85; pinned by the published
  known-answer vectors in ``tests/test_philox_oracle.py``.
- Counter layout of the kernels: (idx lo, idx hi, call lo, call hi 24 bits |
  domain << 24), 64-bit key split (lo, hi).
- Box-Muller on the top 24 bits of two words: u1 = (a >> 8 + 1) 2^-24,
  u2 = (b >> 8) 2^-24 - 1/2, r = sqrt(-2 ln u1), (-r cos 2 pi u2, -r sin 2 pi u2)
  (the device evaluates it with hardware approximations, absolute error near
  1e-6; this restatement is float64).
- Screen noise of generate: element (row, ky) of a row of length n takes
  counter row * H + (ky mod H), H = ceil(n / 2), the first pair of the call
  for ky < H and the second otherwise; row = fft_index * n + kx.
- Subharmonic noise of screen gc, level p, cell ij: counter
  (gc * 16 + p) * 9 + ij, first pair.
"""

from __future__ import annotations

import numpy as np

M0, M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
W0, W1 = 0x9E3779B9, 0xBB67AE85
MASK = np.uint64(0xFFFFFFFF)
DOMAIN_SCREEN = 0x11
DOMAIN_SUB = 0x22
MAX_LEVELS = 16


def philox4x32_10(c0, c1, c2, c3, key: int):
    """Vectorised Philox4x32-10 of uint32 counter words (arrays broadcast)
    under a 64-bit key; returns the four output words as uint64 arrays."""
    x0, x1, x2, x3 = (np.asarray(v, dtype=np.uint64) & MASK for v in (c0, c1, c2, c3))
    k0, k1 = key & 0xFFFFFFFF, (key >> 32) & 0xFFFFFFFF
    for r in range(10):
        p0 = M0 * x0
        p1 = M1 * x2
        hi0, lo0 = p0 >> np.uint64(32), p0 & MASK
        hi1, lo1 = p1 >> np.uint64(32), p1 & MASK
        x0, x1, x2, x3 = (hi1 ^ x1 ^ np.uint64(k0), lo1, hi0 ^ x3 ^ np.uint64(k1), lo0)
        k0 = (k0 + W0) & 0xFFFFFFFF
        k1 = (k1 + W1) & 0xFFFFFFFF
    return x0, x1, x2, x3


def _counter(idx, call: int, domain: int):
    idx = np.asarray(idx, dtype=np.uint64)
    c3 = ((call >> 32) & 0x00FFFFFF) | (domain << 24)
    return idx & MASK, idx >> np.uint64(32), np.uint64(call & 0xFFFFFFFF), np.uint64(c3)


def box_muller(a, b):
    u1 = ((a >> np.uint64(8)).astype(np.float64) + 1.0) / 16777216.0
    u2 = (b >> np.uint64(8)).astype(np.float64) / 16777216.0 - 0.5
    r = np.sqrt(-2.0 * np.log(u1))
    t = 2.0 * np.pi * u2
    return -r * np.cos(t), -r * np.sin(t)


def cnormal2(key: int, idx, call: int, domain: int):
    """Both complex normals (lo, hi) of the calls at counters ``idx``."""
    r = philox4x32_10(*_counter(idx, call, domain), key)
    lo = box_muller(r[0], r[1])
    hi = box_muller(r[2], r[3])
    return lo[0] + 1j * lo[1], hi[0] + 1j * hi[1]


def screen_noise(key: int, call: int, n: int, n_fft: int) -> np.ndarray:
    """(n_fft, n, n) complex screen noise of one generate call."""
    H = (n + 1) // 2
    rows = np.arange(n_fft * n, dtype=np.uint64)[:, None]
    ky = np.arange(n)
    idx = rows * np.uint64(H) + (ky % H).astype(np.uint64)[None, :]
    lo, hi = cnormal2(key, idx, call, DOMAIN_SCREEN)
    z = np.where((ky < H)[None, :], lo, hi)
    return z.reshape(n_fft, n, n)


def sub_noise(key: int, call: int, count: int, levels: int) -> np.ndarray:
    """(levels, count, 3, 3) complex subharmonic noise of one generate call."""
    gc = np.arange(count, dtype=np.uint64)[:, None, None]
    p = np.arange(levels, dtype=np.uint64)[None, :, None]
    ij = np.arange(9, dtype=np.uint64)[None, None, :]
    idx = (gc * np.uint64(MAX_LEVELS) + p) * np.uint64(9) + ij
    lo, _ = cnormal2(key, idx, call, DOMAIN_SUB)
    return lo.transpose(1, 0, 2).reshape(levels, count, 3, 3)


class PhiloxDraws:
    """A stand-in for ``numpy.random.Generator`` that hands
    :class:`oracle.OraclePhaseScreen` the device's normals in the reference's
    draw order: ``(2, ceil(count / 2), n, n)`` then ``(2, count, 3, 3)`` per
    level, real parts first."""

    def __init__(self, key: int, call: int, n: int, count: int, levels: int) -> None:
        n_fft = (count + 1) // 2
        z = screen_noise(key, call, n, n_fft)
        self._queue = [np.stack([z.real, z.imag])]
        if levels:
            s = sub_noise(key, call, count, levels)
            self._queue += [np.stack([s[p].real, s[p].imag]) for p in range(levels)]

    def standard_normal(self, shape, dtype=np.float64):
        a = self._queue.pop(0)
        assert a.shape == tuple(shape), (a.shape, shape)
        return a.astype(dtype)
