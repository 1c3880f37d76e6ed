"""The oracle's restatement of the kernels' noise (oracle/philox.py), on the
CPU: Philox4x32-10 against the published known-answer vectors of Salmon et
al. (SC'11), the Box-Muller normals' moments, and the screen-noise pairing."""

import numpy as np

from oracle.philox import cnormal2, philox4x32_10, screen_noise, sub_noise


def test_philox4x32_10_known_answers():
    kats = [((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
            ((0xFFFFFFFF,) * 4, (0xFFFFFFFF, 0xFFFFFFFF),
             (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
            ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
             (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1))]
    for ctr, key, want in kats:
        got = tuple(int(v) for v in philox4x32_10(*ctr, key[0] | (key[1] << 32)))
        assert got == want


def test_normals_have_unit_variance():
    lo, hi = cnormal2(12345, np.arange(50000, dtype=np.uint64), 3, 0x11)
    z = np.concatenate([lo, hi])
    for part in (z.real, z.imag):
        assert abs(part.mean()) < 0.02 and abs(part.var() - 1.0) < 0.02
    assert abs(np.mean(z.real * z.imag)) < 0.02


def test_screen_noise_pairs_share_a_call():
    n, H = 10, 5
    z = screen_noise(7, 2, n, 3)
    for b in range(3):
        for kx in range(n):
            row = b * n + kx
            lo, hi = cnormal2(7, np.arange(row * H, row * H + H, dtype=np.uint64), 2, 0x11)
            np.testing.assert_array_equal(z[b, kx, :H], lo)
            np.testing.assert_array_equal(z[b, kx, H:], hi)
    s = sub_noise(7, 2, 4, 3)
    assert s.shape == (3, 4, 3, 3)
    lo, _ = cnormal2(7, np.array([(1 * 16 + 2) * 9 + 5], dtype=np.uint64), 2, 0x22)
    assert s[2, 1, 1, 2] == lo[0]
