"""The float64 synthesis oracle's VJP against central differences and torch
autograd (CPU)."""

import numpy as np
import pytest

from oracle import synth_diff as sd


def case(seed=4, L=3, ns=16, F=3, crop=2, n_out=11):
    rng = np.random.default_rng(seed)
    S = rng.standard_normal((L, ns, ns)) + 1j * rng.standard_normal((L, ns, ns))
    w = rng.uniform(0.5, 1.5, L)
    dx = 0.1
    sx = rng.uniform(-3, 3, (F, L))
    sy = rng.uniform(-3, 3, (F, L))
    g = rng.standard_normal((F, n_out, n_out))
    return S, w, sx, sy, dx, crop, n_out, 0.7, g


def value(S, w, sx, sy, dx, crop, n_out, scale, g):
    return float(np.sum(sd.synth_frames(S, w, sx, sy, dx, crop, n_out, scale) * g))


def test_vjp_matches_central_differences():
    S, w, sx, sy, dx, crop, n_out, scale, g = case()
    gS, gw, gsx, gsy = sd.synth_vjp(S, w, sx, sy, dx, crop, n_out, scale, g)
    eps = 1e-6
    args = (dx, crop, n_out, scale, g)
    for idx in [(0, 1, 2), (2, 15, 0), (1, 8, 8)]:
        for part, unit in (("re", 1.0), ("im", 1j)):
            Sp, Sm = S.copy(), S.copy()
            Sp[idx] += eps * unit
            Sm[idx] -= eps * unit
            fd = (value(Sp, w, sx, sy, *args) - value(Sm, w, sx, sy, *args)) / (2 * eps)
            want = gS[idx].real if part == "re" else gS[idx].imag
            assert fd == pytest.approx(want, rel=1e-6, abs=1e-7)
    for l in range(w.size):
        wp, wm = w.copy(), w.copy()
        wp[l] += eps
        wm[l] -= eps
        fd = (value(S, wp, sx, sy, *args) - value(S, wm, sx, sy, *args)) / (2 * eps)
        assert fd == pytest.approx(gw[l], rel=1e-6)
    for idx in [(0, 0), (2, 1), (1, 2)]:
        for arr, gref in ((sx, gsx), (sy, gsy)):
            ap, am = arr.copy(), arr.copy()
            ap[idx] += eps
            am[idx] -= eps
            if arr is sx:
                fd = (value(S, w, ap, sy, *args) - value(S, w, am, sy, *args)) / (2 * eps)
            else:
                fd = (value(S, w, sx, ap, *args) - value(S, w, sx, am, *args)) / (2 * eps)
            assert fd == pytest.approx(gref[idx], rel=1e-5, abs=1e-6)


def test_vjp_matches_torch_autograd():
    torch = pytest.importorskip("torch")
    S, w, sx, sy, dx, crop, n_out, scale, g = case(seed=9)
    L, ns, _ = S.shape
    tS = torch.tensor(S, requires_grad=True)
    tw = torch.tensor(w, requires_grad=True)
    tsx = torch.tensor(sx, requires_grad=True)
    tsy = torch.tensor(sy, requires_grad=True)
    f = torch.tensor(np.fft.fftfreq(ns, dx))
    px = torch.exp(2j * np.pi * f[None, None, :] * tsx[..., None])
    py = torch.exp(2j * np.pi * f[None, None, :] * tsy[..., None])
    X = torch.einsum("l,lij,fli,flj->fij", tw.to(torch.complex128), tS, px, py)
    y = scale * torch.fft.ifft2(X).real * ns * ns
    y = y[:, crop:crop + n_out, crop:crop + n_out]
    (y * torch.tensor(g)).sum().backward()
    gS, gw, gsx, gsy = sd.synth_vjp(S, w, sx, sy, dx, crop, n_out, scale, g)
    np.testing.assert_allclose(y.detach().numpy(),
                               sd.synth_frames(S, w, sx, sy, dx, crop, n_out, scale),
                               rtol=1e-12, atol=1e-10)
    np.testing.assert_allclose(tS.grad.numpy(), gS, rtol=1e-10, atol=1e-9)
    np.testing.assert_allclose(tw.grad.numpy(), gw, rtol=1e-10)
    np.testing.assert_allclose(tsx.grad.numpy(), gsx, rtol=1e-9, atol=1e-8)
    np.testing.assert_allclose(tsy.grad.numpy(), gsy, rtol=1e-9, atol=1e-8)
