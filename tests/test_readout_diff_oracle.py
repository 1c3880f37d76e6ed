"""The float64 readout oracle's gradient against central finite differences and
against torch autograd (CPU; no GPU needed)."""

import numpy as np
import pytest

from oracle import readout_diff as rd


def small_case(seed=3, B=2, L=3, S=24, T=2, D=3, n=12):
    rng = np.random.default_rng(seed)
    screens = rng.standard_normal((B, L, S, S))
    w = rng.uniform(0.5, 1.5, L)
    mag = np.ones((D, L))
    mag[-1] = [1.0, 0.83, 0.71][:L] if L <= 3 else np.linspace(1.0, 0.7, L)
    pos0 = rng.uniform(-40.0, 40.0, (T, D, L, 2))
    g = rng.standard_normal((B, T, D, n, n))
    return screens, w, pos0, mag, n, g


def loss(screens, w, pos0, mag, n, g):
    return float(np.sum(rd.layer_readout(screens, w, pos0, mag, n) * g))


def test_vjp_matches_central_differences():
    screens, w, pos0, mag, n, g = small_case()
    gs, gw, gp = rd.layer_readout_vjp(screens, w, pos0, mag, n, g)
    eps = 1e-6
    rng = np.random.default_rng(0)
    for _ in range(6):
        idx = tuple(rng.integers(0, s) for s in screens.shape)
        sp, sm = screens.copy(), screens.copy()
        sp[idx] += eps
        sm[idx] -= eps
        fd = (loss(sp, w, pos0, mag, n, g) - loss(sm, w, pos0, mag, n, g)) / (2 * eps)
        assert fd == pytest.approx(gs[idx], rel=1e-6, abs=1e-8)
    for l in range(w.size):
        wp, wm = w.copy(), w.copy()
        wp[l] += eps
        wm[l] -= eps
        fd = (loss(screens, wp, pos0, mag, n, g) - loss(screens, wm, pos0, mag, n, g)) / (2 * eps)
        assert fd == pytest.approx(gw[l], rel=1e-6)
    for idx in [(0, 0, 0, 0), (1, 2, 1, 1), (0, 1, 2, 0), (1, 0, 1, 1)]:
        pp, pm = pos0.copy(), pos0.copy()
        pp[idx] += eps
        pm[idx] -= eps
        fd = (loss(screens, w, pp, mag, n, g) - loss(screens, w, pm, mag, n, g)) / (2 * eps)
        assert fd == pytest.approx(gp[idx], rel=1e-5, abs=1e-7)


def test_vjp_matches_torch_autograd():
    torch = pytest.importorskip("torch")
    screens, w, pos0, mag, n, g = small_case(seed=5)
    B, L, S, _ = screens.shape
    T, D = pos0.shape[:2]
    ts = torch.tensor(screens, requires_grad=True)
    tw = torch.tensor(w, requires_grad=True)
    tp = torch.tensor(pos0, requires_grad=True)
    idx = torch.arange(n, dtype=torch.float64)
    out = []
    for t in range(T):
        for d in range(D):
            acc = 0
            for l in range(L):
                ur = tp[t, d, l, 0] + float(mag[d, l]) * idx
                uc = tp[t, d, l, 1] + float(mag[d, l]) * idx
                r0f, c0f = torch.floor(ur), torch.floor(uc)
                fr, fc = ur - r0f, uc - c0f
                r0, c0 = r0f.long() % S, c0f.long() % S
                r1, c1 = (r0 + 1) % S, (c0 + 1) % S
                s = ts[:, l]
                v00 = s[:, r0][:, :, c0]
                v01 = s[:, r0][:, :, c1]
                v10 = s[:, r1][:, :, c0]
                v11 = s[:, r1][:, :, c1]
                top = v00 * (1 - fc) + v01 * fc
                bot = v10 * (1 - fc) + v11 * fc
                acc = acc + tw[l] * (top * (1 - fr)[:, None] + bot * fr[:, None])
            out.append(acc)
    out = torch.stack(out, dim=1).reshape(B, T, D, n, n)
    (out * torch.tensor(g)).sum().backward()
    gs, gw, gp = rd.layer_readout_vjp(screens, w, pos0, mag, n, g)
    # the oracle rounds positions to the device's 2^-32 px fixed point
    np.testing.assert_allclose(out.detach().numpy(), rd.layer_readout(screens, w, pos0, mag, n),
                               rtol=1e-7, atol=1e-8)
    np.testing.assert_allclose(ts.grad.numpy(), gs, rtol=1e-7, atol=1e-8)
    np.testing.assert_allclose(tw.grad.numpy(), gw, rtol=1e-7)
    np.testing.assert_allclose(tp.grad.numpy(), gp, rtol=1e-7, atol=1e-7)


def test_positions_follow_the_reference_geometry():
    # pupil centre lands on the screen centre, scaled about it by mag; x displaces rows
    n, S, dx = 16, 40, 0.5
    mag = np.array([[1.0, 0.75]])
    pos0 = rd.positions(n, S, dx, [0.0, 1000.0], [[1e-4, -2e-4]], mag,
                        [[3.0, -1.0], [0.0, 2.0]], [0.0, 0.5])
    centre = (S - 1) / 2
    for t, tt in enumerate([0.0, 0.5]):
        for l, (alt, v) in enumerate(zip([0.0, 1000.0], [[3.0, -1.0], [0.0, 2.0]])):
            m = mag[0, l]
            mid = pos0[t, 0, l] + m * (n - 1) / 2
            disp = np.array(v) * tt + alt * np.array([1e-4, -2e-4])
            np.testing.assert_allclose(mid, centre + disp / dx, rtol=0, atol=1e-12)


def test_samples_on_grid_lines_take_the_fixed_point_cell():
    # mag = 37/45 (an LGS at 90 km over a layer at 16 km) puts samples exactly on
    # grid lines; the cell (and so the one-sided position derivative) is the
    # one the 32.32 fixed-point position selects, as on the device
    S, n = 64, 48
    m = 1.0 - 16000.0 / 90000.0
    p0 = (S - 1) / 2.0 - m * (n - 1) / 2.0
    i0, i1, f = rd._axis(p0, m, n, S)
    one = 2 ** 32
    v = int(np.rint(p0 * one)) + np.arange(n, dtype=np.int64) * int(np.rint(m * one))
    np.testing.assert_array_equal(i0, v >> 32)
    np.testing.assert_allclose(f, (v & (one - 1)) / one, rtol=0, atol=0)
    exact = (p0 + m * np.arange(n))
    assert np.max(np.abs(i0 + f - exact)) < 1e-8

